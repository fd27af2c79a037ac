/*
 * lcirs_oracle.h - CPU restatement of TripleLens' extended-source light-curve
 * path (LightCurveIRS): test infrastructure, used ONLY by the tests, the
 * smoke check and the CPU-baseline leg of bench.py to check and time against.  Nothing in the product links,
 * loads or calls this library.
 *
 * Parity is pinned against the reference built from its own sources
 * (oracle/Makefile.ref -> oracle/_ref/) and against the committed golden
 * fixtures in tests/golden/ that were generated from that build.
 *
 * Every function cites the reference file:line whose algorithm it restates.
 */
#ifndef LCIRS_ORACLE_H
#define LCIRS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_lcirs orc_lcirs;

/* Grid parameters of the image plane (lcirs.cc:51-92). */
typedef struct {
  double corner_x, corner_y;   /* _bottomLeftCornerImg */
  double top_x, top_y;         /* _topRightCornerImg */
  double size_double;          /* _imgPlaneSizeDouble = 2*halfEdge */
  double h;                    /* _imgGridPointSize */
  double amp_scale;            /* _ampScale */
  int64_t n;                   /* _imgPlaneSize */
} orc_grid;

/* lcirs.cc:6-37 (constructor) */
orc_lcirs *orc_new(double a, double b, double th, double m2, double m3,
                   double rho, unsigned int lc_length, long ppr);
void orc_free(orc_lcirs *o);

/* Restart the image solver's warm-start chain cold every k points
 * (k = 0: a single chain, as the reference). */
void orc_set_chain_chunk(orc_lcirs *o, int k);
/* Residual below which a root rejected by the 1e-6 filter although it solves
 * the lens equation (or accepted although it does not) marks its point as
 * fragile (default 1e-4). */
void orc_set_fragile_band(orc_lcirs *o, double r);

/* lcirs.cc:579-598 (set_limb_darkening): model "linear" -> v-normalised. */
void orc_set_limb_darkening(orc_lcirs *o, const char *model, double v);

void orc_grid_params(const orc_lcirs *o, orc_grid *g);
/* caustic / critical-curve samples, 6 branches x 500, branch-major */
void orc_copy_cc_ca(const orc_lcirs *o, double *cc_xy, double *ca_xy);
void orc_lens(const orc_lcirs *o, double *m123, double *z_xy /* 6 */);
void orc_ld(const orc_lcirs *o, double *A, double *B, double *intensity);

/* lcirs.cc:103-191: n+1 points; amps[i] = sum(weights)*ampScale,
 * counts[i] = rays accepted.  Arrays hold lc_length+1 entries. */
void orc_get_lc_irs(orc_lcirs *o, double x0, double y0, double x1, double y1,
                    double *amps, uint64_t *counts);

/* Same walk but stops after computing the seeds for every point: seeds are
 * written as pixel pairs (nx, ny) into seeds_xy (capacity max_seeds per
 * point), seed_count[i] = number of seeds for point i (may exceed max_seeds:
 * the surplus is dropped).  fragile[i] (optional) is 1 when some root's
 * lens-equation residual lay within a decade of the 1e-6 image filter
 * radius (imgpoint.cc:72-90), i.e. the image set of that point depends on
 * rounding.  Returns the total number of seeds. */
long orc_lc_seeds(orc_lcirs *o, double x0, double y0, double x1, double y1,
                  int max_seeds, int64_t *seeds_xy, int *seed_count, int *fragile);

/* Flood fill of one source position from explicit seed pixels
 * (lcirs.cc:171-174 + lineFloodFill lcirs.cc:381-466). */
void orc_fill(orc_lcirs *o, double sx, double sy, const int64_t *seeds_xy,
              int n_seeds, double *amp, uint64_t *count);

/* Rows / ranges of the last fill, as the amoeba dump (amoeba.cc:90-108):
 * returns the number of ranges; writes up to cap triples (ny, xl, xr). */
long orc_last_amoeba(const orc_lcirs *o, int64_t *triples, long cap);

/* lcbase.cc:40-52: point-source curve, n points at i/(n-1). */
void orc_get_lc(orc_lcirs *o, double x0, double y0, double x1, double y1,
                double *amps);

/* imgpoint.cc:281-286: images of one source position through the
 * warm-started solver state of this object.  Returns the count. */
int orc_get_images(orc_lcirs *o, double sx, double sy, double *img_xy /*20*/);

/* Cold images of a source position (fresh solver, no warm start). */
int orc_images_cold(double a, double b, double th, double m2, double m3,
                    double sx, double sy, double *img_xy);

/* Squared distance of the mapped ray from the source, irsSIMD lane order
 * (lcirs.cc:290-341). */
double orc_irs(const orc_lcirs *o, double x, double y, double sx, double sy);

/* Laguerre (laguerre.cc:103-167): coefficients c[0..deg] (re,im pairs),
 * init either NULL or deg+1 roots (init[deg] emulates the reference's
 * one-past-the-end read).  Writes deg roots. */
void orc_solve_roots(const double *coeffs, int deg, const double *init,
                     double *roots);
/* laguerre.cc:18-99 single-root iteration; returns 1 on convergence. */
int orc_laguerre(const double *coeffs, int deg, double *x);

/* Degree-10 lens polynomial coefficients for source zeta. */
void orc_lens_poly(const orc_lcirs *o, double sx, double sy, double *c /*22*/);

/* lcirs.cc:195-255 (Q5 geometry) for the segment A-B and the object's rho;
 * returns 1 on a hit and writes the trial point. */
int orc_intersection_check(const orc_lcirs *o, double sx, double sy, double ax, double ay,
                           double bx, double by, double *trial_xy);

/* lcbase.cc:17-38: one image's term of the point-source magnification. */
double orc_image_amp(const orc_lcirs *o, double ix, double iy);

/* lcirs.cc:355-379: grid maps of the object's image plane. */
void orc_grid_maps(const orc_lcirs *o, int64_t nx, int64_t ny, double x, double y,
                   double *xy_out, int64_t *n_out);

#ifdef __cplusplus
}
#endif
#endif
