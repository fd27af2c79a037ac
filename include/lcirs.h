/*
 * lcirs.h - C ABI of liblcirs.so, the GB300 engine for TripleLens'
 * extended-source light curves (inverse-ray shooting, LightCurveIRS).
 *
 * The first six entry points keep the reference's ctypes ABI exactly
 * (src/LightCurves/lcirs.cc:515-609; bound by Examples/ctypes_classes.py:128-193),
 * so the reference's Python drivers load this library unchanged.  The object
 * pointer is opaque.  As in the reference, calls are synchronous, return
 * nothing, and report to stdout; GPU-side conditions are additionally
 * readable through lcirs_last_status().
 *
 * The remaining entry points are additive.
 */
#ifndef TL_LCIRS_H
#define TL_LCIRS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct LightCurveIRS LightCurveIRS;

/* Replaces lcirs_new (src/LightCurves/lcirs.cc:517-537).  Lens a, b, th, m2,
 * m3 (z1 = 0, z2 = (a,0), z3 = b e^{i th}, m1 = 1 - m2 - m3), source radius,
 * light-curve length n, rays per source radius.  Computes the critical curve,
 * caustics and image-plane grid on the GPU.  With parameters the set-up
 * cannot use (a non-finite value, a source radius <= 0, rays per radius
 * outside 1..2^31-1) the object is still returned but never reaches the GPU:
 * lcirs_last_status reads 32 (bad input), and every curve it computes has
 * zero counts and magnifications with status 32 on every point. */
LightCurveIRS* lcirs_new(double a, double b, double th, double m2, double m3, double sourceSize,
                         unsigned int lcLength, long pointsPerRadius);

/* Replaces get_lc (src/LightCurves/lcirs.cc:539-549 -> lcbase.cc:40-52):
 * point-source magnification at n points t = i/(n-1) into the curve. */
void get_lc(LightCurveIRS* lcirs, double iniX, double iniY, double finX, double finY);

/* Replaces get_lc_irs (src/LightCurves/lcirs.cc:552-562 -> 103-191):
 * extended-source magnification at n+1 points t = i/n; prints the
 * reference's per-point line "irs amplification: A and the count N and amp
 * scale s". */
void get_lc_irs(LightCurveIRS* lcirs, double iniX, double iniY, double finX, double finY);

/* Replaces copy_lc (src/LightCurves/lcirs.cc:566-576): copies exactly n
 * doubles (the first n points of the last curve). */
void copy_lc(LightCurveIRS* lc, double* lcArray);

/* Replaces set_limb_darkening (src/LightCurves/lcirs.cc:579-598): "linear"
 * selects the v-normalised linear model (limbdarkeningmodel.cc:18-28), any
 * other string the default A = 0.6, B = 0.4. */
void set_limb_darkening(LightCurveIRS* lc, const char* model, double v);

/* Replaces set_amoeba_printout (src/LightCurves/lcirs.cc:601-607): after each
 * point of get_lc_irs, write "<prefix><i>" with one "ny,xleft,xright" line
 * per filled row range (amoeba.cc:90-108), and the grid parameters as JSON to
 * parFilename (lcirs.cc:479-512, including its "m3" field holding m2). */
void set_amoeba_printout(LightCurveIRS* lc, const char* amoebaFilename, const char* parFilename);

/* ---- additive entry points (no counterpart in the reference ABI) ---- */

/* Frees an object (the reference has no destroy export). */
void lcirs_delete(LightCurveIRS* lc);

/* OR of the status bits of the points of the last curve (0 = clean):
 * 1 seed overflow, 2 plane edge reached, 4 tile table full, 8 bounded wait
 * expired, 16 wrong image count after retry, 32 bad input,
 * 0x100 CUDA error. */
unsigned int lcirs_last_status(LightCurveIRS* lc);

/* Ray counts of the last get_lc_irs, n+1 entries. */
void lcirs_copy_counts(LightCurveIRS* lc, uint64_t* counts);

/* All n+1 magnifications of the last get_lc_irs (copy_lc stops at n). */
void lcirs_copy_lc_full(LightCurveIRS* lc, double* out);

/* Per-point status bits of the last get_lc_irs, n+1 entries. */
void lcirs_copy_status(LightCurveIRS* lc, uint32_t* status);

/* 0 silences the per-point stdout lines (default 1, as the reference). */
void lcirs_set_verbose(LightCurveIRS* lc, int verbose);

/* Grid of the object: corner_x, corner_y, top_x, top_y, size, h, ampScale,
 * N (as double).  8 doubles. */
void lcirs_grid(LightCurveIRS* lc, double* out8);

/* Seeds of the last get_lc_irs: per point up to 64 (nx, ny) pixel pairs and
 * their number.  seeds: (n+1)*64*2 int32, nseeds: n+1 int32. */
void lcirs_copy_seeds(LightCurveIRS* lc, int32_t* seeds, int32_t* nseeds);

/* Fill only: given explicit seed pixels for each of the n+1 points of the
 * trajectory (same layout as lcirs_copy_seeds), compute counts and
 * magnifications with the GPU fill kernel. */
void lcirs_fill_from_seeds(LightCurveIRS* lc, double iniX, double iniY, double finX, double finY,
                           const int32_t* seeds, const int32_t* nseeds);

/* Ray statistics of the last get_lc_irs: rays evaluated, rays evaluated in
 * FP64, tiles visited (3 x uint64 totals). */
void lcirs_copy_stats(LightCurveIRS* lc, uint64_t* out3);

/* Bytes the library has copied host -> device and device -> host for the
 * lcirs_* and tlb_* calls of this process (2 x uint64 totals since load):
 * the parameters, point lists and jobs going in; the per-point results and
 * seeds coming back.  Additive, for end-to-end accounting; no GPU work. */
void lcirs_copy_transfer_bytes(uint64_t* out2);

/* Ray-map precision: 0 = every ray in FP64 (irsSIMD order); 1 = FP32
 * tile-relative map with an FP64 guard band at the limb (default). */
void lcirs_set_precision(LightCurveIRS* lc, int mode);

/* Warm-start chain of the image solver.  0 (default): one chain carried
 * through every get_lc_irs / get_lc call of the object, as the reference's
 * ImgPoint member carries it (imgpoint.cc:160-205) - ray counts equal the
 * reference's (strict IEEE build) on every point, and the chain runs serially
 * on the GPU.  k > 0: the chain restarts from the constructor's state every
 * k points and chunks run in parallel; counts then differ from the
 * reference's at the few points whose image decisions depend on the last
 * bits of the warm start. */
void lcirs_set_chain(LightCurveIRS* lc, int points);

/* Fill diagnostics of the last get_lc_irs, n+1 entries, from the fill stage
 * that completed the point: team fill: bits 0-15 its rounds; CTA fill: bits
 * 0-15 the largest number of passes over one tile, bit 17 dequeue limit
 * reached, bits 24-31 the tile state seen then; warp fill: 0.  Bit 16: a
 * bound on passes, visits or rounds was reached. */
void lcirs_copy_diag(LightCurveIRS* lc, uint32_t* diag);

/* No counterpart in the reference.  Fill-only run that allocates no device
 * memory, for callers that cannot call cudaMalloc when they compute
 * magnifications: programs that hand the GPU's memory to their own pool at
 * start-up (a later cudaMalloc fails or escapes their accounting), and
 * latency-bound loops that cannot take the device-wide synchronisation of
 * cudaFree (often of cudaMalloc too).  The other entry points grow their
 * buffers with cudaMalloc on demand.
 *
 * Same work as lcirs_fill_from_seeds for explicit source positions, on
 * DEVICE arrays of the caller: src_xy (npoints x 2 doubles), seeds
 * (npoints x 64 x 2 int32, the layout of lcirs_copy_seeds), nseeds (npoints
 * int32); outputs mag (npoints doubles), and optionally counts (uint64) and
 * status (uint32, bits as lcirs_last_status).  The object's lens, grid,
 * limb darkening and precision are used; the current device must be the one
 * the object was created on (another current device returns -1 and prints
 * both device numbers).  Seed counts are clamped to 0..64 (a negative count
 * fills nothing, a count above 64 uses the 64 stored pixels).  Work is queued
 * on `stream` (a cudaStream_t, NULL for the default stream) and the call
 * returns without waiting.
 *
 * Scratch memory is one static device array of 80 MiB, held by every GPU
 * that loads the library's device code until the process exits.  The first
 * call on a device looks up the array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * All calls share the array and each call clears what must start at zero,
 * so calls whose GPU work overlaps (different streams, or several host
 * threads without ordering) race: order them on one stream.
 *
 * Limits: at most LCIRS_NOALLOC_MAX_POINTS points per call (larger calls
 * return -3 and print the limit to stderr, nothing runs), and per point a
 * table of 16384 blocks of 32 x 32 rays (3/4 usable: magnifications up to
 * ~100 at 200 rays per source radius, ~15 at 500); a point whose images need
 * more gets status bit 4 and an incomplete magnification (the allocating
 * entry points retry it with larger tables).
 *
 * Returns 0 when the work was queued, -1 bad argument, -2 CUDA error,
 * -3 too many points. */
#define LCIRS_NOALLOC_MAX_POINTS 8192
int lcirs_fill_device_noalloc(LightCurveIRS* lc, int npoints, const double* src_xy,
                              const int32_t* seeds, const int32_t* nseeds, double* mag,
                              uint64_t* counts, uint32_t* status, void* stream);

#ifdef __cplusplus
}
#endif
#endif
