/*
 * lcirs_oracle.c - CPU restatement of TripleLens' LightCurveIRS path.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle: tests/, the smoke check
 * and bench.py's CPU-baseline leg call it; the product never does.
 *
 * It restates, in plain C99, the algorithm of the reference files cited at
 * each function (paths relative to the TripleLens project root).  Where the
 * reference has undefined behaviour the restatement makes a defined choice,
 * named at the spot (quirks Q4 and Q9).  Arithmetic is written out operation
 * by operation and the file is compiled with -ffp-contract=off, so that the
 * FP64 ray map reproduces the reference built with -ffp-contract=off.
 */
#include "lcirs_oracle.h"

#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------------ */
/* complex arithmetic with the semantics std::complex<double> has in a       */
/* strict IEEE build (g++ -O2 -fno-fast-math -ffp-contract=off):             */
/*   a * b   the textbook product (the library's NaN recovery never applies  */
/*           to the finite values of this path);                             */
/*   a / b   Smith's algorithm (R. L. Smith, "Algorithm 116: Complex         */
/*           division", CACM 5(8), 1962), the method of libgcc's __divdc3;   */
/*   |a|     hypot, computed as in C. F. Borges, "An improved algorithm for  */
/*           hypot(a,b)", 2019 (arXiv:1904.09481): a naive square root       */
/*           corrected by the exactly re-expressed residual, the no-FMA form;*/
/*   sqrt(a) the half-angle principal root built on that hypot (W. Kahan,    */
/*           "Branch cuts for complex elementary functions", 1987).         */
/* Each agrees bit for bit with glibc's hypot/csqrt and libgcc's division   */
/* (checked on 2e7 random operands), so the oracle rounds exactly as the    */
/* reference's strict build does.                                            */
/* ------------------------------------------------------------------------ */
typedef struct { double re, im; } cx;

static inline cx mk(double re, double im) { cx z = {re, im}; return z; }
static inline cx cadd(cx a, cx b) { return mk(a.re + b.re, a.im + b.im); }
static inline cx csub(cx a, cx b) { return mk(a.re - b.re, a.im - b.im); }
static inline cx cneg(cx a) { return mk(-a.re, -a.im); }
static inline cx cconj(cx a) { return mk(a.re, -a.im); }
static inline cx cmul(cx a, cx b) {
  return mk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
static inline cx cscale(cx a, double s) { return mk(a.re * s, a.im * s); }
static inline cx cdiv(cx a, cx b) {
  if (fabs(b.re) < fabs(b.im)) {
    double r = b.re / b.im, den = b.re * r + b.im;
    if (fabs(r) > DBL_MIN) return mk((a.re * r + a.im) / den, (a.im * r - a.re) / den);
    return mk((b.re * (a.re / b.im) + a.im) / den, (b.re * (a.im / b.im) - a.re) / den);
  }
  double r = b.im / b.re, den = b.im * r + b.re;
  if (fabs(r) > DBL_MIN) return mk((a.im * r + a.re) / den, (a.im - a.re * r) / den);
  return mk((a.re + b.im * (a.im / b.re)) / den, (a.im - b.im * (a.re / b.re)) / den);
}
/* real / complex, as complex<double>(x) /= y */
static inline cx rdiv(double x, cx b) { return cdiv(mk(x, 0.0), b); }
static inline double cnorm(cx a) { return a.re * a.re + a.im * a.im; }
static double hypot_kernel(double ax, double ay) {
  double h = sqrt(ax * ax + ay * ay), t1, t2;
  if (h <= 2.0 * ay) {
    double d = h - ay;
    t1 = ax * (2.0 * d - ax);
    t2 = (d - 2.0 * (ax - ay)) * d;
  } else {
    double d = h - ax;
    t1 = 2.0 * d * (ax - 2.0 * ay);
    t2 = (4.0 * d - ay) * ay + d * d;
  }
  return h - (t1 + t2) / (2.0 * h);
}
static double hypot_(double x, double y) {
  x = fabs(x);
  y = fabs(y);
  double ax = x < y ? y : x, ay = x < y ? x : y;
  if (ax > 0x1p+511) {
    if (ay <= ax * 0x1p-54) return ax + ay;
    return hypot_kernel(ax * 0x1p-600, ay * 0x1p-600) / 0x1p-600;
  }
  if (ay < 0x1p-511) {
    if (ax >= ay / 0x1p-54) return ax + ay;
    return hypot_kernel(ax / 0x1p-600, ay / 0x1p-600) * 0x1p-600;
  }
  if (ay <= ax * 0x1p-54) return ax + ay;
  return hypot_kernel(ax, ay);
}
static inline double cabs_(cx a) { return hypot_(a.re, a.im); }
static cx csqrt_(cx a) {
  if (a.im == 0.0) {
    if (a.re < 0.0) return mk(0.0, copysign(sqrt(-a.re), a.im));
    return mk(fabs(sqrt(a.re)), copysign(0.0, a.im));
  }
  if (a.re == 0.0) {
    double r = sqrt(0.5 * fabs(a.im));
    return mk(r, copysign(r, a.im));
  }
  double d = hypot_(a.re, a.im);
  if (a.re > 0.0) {
    double r = sqrt(0.5 * (d + a.re));
    return mk(r, 0.5 * (a.im / r));
  }
  double s = sqrt(0.5 * (d - a.re));
  return mk(fabs(0.5 * (a.im / s)), copysign(s, a.im));
}

/* ------------------------------------------------------------------------ */
/* Laguerre root finder: src/Laguerre/laguerre.cc, laguerre.h:37-38         */
/* ------------------------------------------------------------------------ */
#define ORC_MAX_IT 300
#define ORC_MT 8
#define ORC_MAXC 16
static const double ORC_EPS = 2.220446049250313080847e-16; /* DBL_EPSILON */
static const double kFrac[8] = {0.5, 0.23, 0.73, 0.13, 0.37, 0.61, 0.89, 1.0};

/* laguerre.cc:18-99.  poly has m+1 coefficients, poly[m] the leading one.
 * Q9: the reference indexes frac[i/MT] for i up to MAX_IT, i.e. past the
 * 8-entry table from i = 64 on (undefined behaviour); the restatement wraps
 * the index modulo 8. */
static int lag_iter(const cx *poly, int m, cx *px) {
  cx x = *px;
  if (m == 1) {
    if (cabs_(poly[1]) != 0.0) {
      *px = cneg(cdiv(poly[0], poly[1]));
      return 1;
    }
    *px = mk(999.0, 999.0);
    return 0;
  }
  const double md = (double)m;
  for (int i = 1; i <= ORC_MAX_IT; i++) {
    cx b = poly[m];
    double err = cabs_(b);
    cx s = mk(0.0, 0.0), f = mk(0.0, 0.0);
    for (int j = m - 1; j >= 0; j--) {
      s = cadd(cmul(x, s), f);
      f = cadd(cmul(x, f), b);
      b = cadd(cmul(x, b), poly[j]);
      err = cabs_(b) + cabs_(x) * err;
    }
    err *= ORC_EPS;
    if (cabs_(b) <= err) {
      *px = x;
      return 1;
    }
    cx g = cdiv(f, b);
    cx h = csub(cmul(g, g), cdiv(cscale(s, 2.0), b));
    cx sq = csqrt_(cscale(csub(cscale(h, md), cmul(g, g)), md - 1.0));
    cx gp = cadd(g, sq), gm = csub(g, sq);
    if (cabs_(gp) < cabs_(gm)) gp = gm;
    cx dx;
    if (cabs_(gp) > 0.0)
      dx = rdiv(md, gp);
    else
      dx = cscale(mk(cos(1.0 * i), sin(1.0 * i)), 1.0 + cabs_(x));
    cx x1 = csub(x, dx);
    if (x.re == x1.re && x.im == x1.im) {
      *px = x;
      return 1;
    }
    if (i % ORC_MT)
      x = x1;
    else
      x = csub(x, cscale(dx, kFrac[(i / ORC_MT) & 7]));
  }
  *px = x;
  return 0;
}

/* laguerre.cc:103-167.  init == NULL: cold start from (EPS, EPS).  Otherwise
 * init holds deg+1 entries and root j (j = deg..1) starts from init[j].
 * Q4: the reference's init vector holds only deg roots, so its j = deg start
 * reads one element past the end; callers pass that slot explicitly. */
static void solve_roots(const cx *poly, int deg, const cx *init, cx *roots) {
  cx temp[ORC_MAXC];
  memcpy(temp, poly, (size_t)(deg + 1) * sizeof(cx));
  int nr = 0;
  for (int j = deg; j >= 1; j--) {
    cx x = init ? init[j] : mk(ORC_EPS, ORC_EPS);
    if (lag_iter(temp, j, &x)) {
      roots[nr++] = x;
    } else {
      if (init) x = mk(ORC_EPS, ORC_EPS);
      roots[nr++] = x;
    }
    cx b = temp[j];
    for (int jj = j - 1; jj >= 0; jj--) {
      cx c = temp[jj];
      temp[jj] = b;
      b = cadd(cmul(x, b), c);
    }
  }
  for (int j = 0; j < deg; j++) lag_iter(poly, deg, &roots[j]);
}

/* laguerre.cc:170-183 */
static void polish_roots(const cx *poly, int deg, cx *roots) {
  for (int j = 0; j < deg; j++) lag_iter(poly, deg, &roots[j]);
}

/* laguerre.cc:188-198 */
static int check_roots(const cx *poly, int deg, const cx *roots) {
  cx c0 = poly[deg];
  for (int k = 0; k < deg; k++) c0 = cmul(c0, cneg(roots[k]));
  if (cabs_(poly[0]) > 1.0e-8) return (1.0 - cabs_(cdiv(c0, poly[0]))) < 1.0e-5;
  return cabs_(csub(c0, poly[0])) < 1.0e-10;
}

/* ------------------------------------------------------------------------ */
/* Lens, limb darkening, object state                                        */
/* ------------------------------------------------------------------------ */
#define NCC 500
#define NBR 6

typedef struct { int64_t xl, xr; int32_t next; } orc_range;
typedef struct { int64_t key; int32_t head, tail; int used; } orc_row;

struct orc_lcirs {
  /* lens.cc:4-18,35-40 */
  double a, b, th, m1, m2, m3;
  cx z1, z2, z3;
  int is_binary_img; /* imgpoint.cc:56-68: a==0 || b==0 || m3==0 */
  /* lcirs.cc:6-37 */
  double rho, rho2;
  unsigned int lc_length;
  int ppr;
  /* limbdarkeningmodel.cc:8-37 */
  double ld_a, ld_b, intensity;
  /* ccc */
  cx cc[NBR][NCC], ca[NBR][NCC];
  cx box_min[NBR], box_max[NBR];
  orc_grid g;
  /* ImgPoint warm-start state (imgpoint.h:104-110) */
  cx temp_roots[11];
  int have_temp;
  /* zeta-free coefficients, computed once per object (imgpoint.cc:164-168) */
  cx coef_nozeta[11];
  /* Model of the heap memory the warm start reads (quirk Q4).  The reference
   * starts root 10 of a warm solve from _tempRoots[10], one element past the
   * end of a 10-element vector whose buffer has capacity 16 (256 bytes).  That
   * slot holds whatever the chunk held before: glibc serves 256-byte requests
   * from a per-thread LIFO cache of freed chunks (tcache), and the only
   * 256-byte buffers on this path are vectors of capacity 16 - the roots
   * vectors, the image list of a point with 9+ seeds, the ImgPoint image list
   * with 9+ images, and, during construction, the critical-curve branches
   * growing past 16 samples.  heap[] holds the slot-10 contents of the cached
   * chunks (top last); temp_slot is the slot of the chunk _tempRoots holds. */
  cx heap[8];     /* the path never caches more than 5 */
  int heap_n;
  cx temp_slot;
  int have_temp_chunk;
  int imgs_big;   /* the ImgPoint image list has grown to capacity 16 */
  double *trace;  /* optional record of the slot read by each warm solve */
  long trace_cap, trace_n;
  int chain_chunk; /* 0: one warm-start chain (reference); K: restart every K points */
  int fragile;     /* set when an image decision sat near the filter radius */
  double fragile_band; /* residual below which a filter/lens-equation
                          disagreement marks the point fragile */
  double kappa_max;    /* images with a larger sum m_i/|z - z_i|^2 are fragile */
  /* amoeba (amoeba.h) */
  orc_row *rows;
  long rows_cap, rows_used;
  orc_range *ranges;
  long ranges_cap, ranges_used;
  /* fill stack */
  void *stack;
  long stack_cap;
  /* accumulators (lcirs.h:126-127) */
  double amplification;
  uint64_t irs_count;
};

/* limbdarkeningmodel.cc:8-15 default A=0.6, B=0.4 */
static void ld_default(orc_lcirs *o) {
  o->ld_a = 0.6;
  o->ld_b = 0.4;
  o->intensity = 1.0 / (o->ld_a + 2.0 / 3.0 * o->ld_b);
}
/* limbdarkeningmodel.cc:18-28 normalised linear model */
static void ld_linear(orc_lcirs *o, double v) {
  double i0 = 1.0 / ((1.0 - v / 3.0));
  o->ld_a = i0 * (1.0 - v);
  o->ld_b = i0 * v;
  o->intensity = 1.0;
}

/* ------------------------------------------------------------------------ */
/* Critical curve and caustic: src/CCC/ccc.cc:42-98, 160-203                 */
/* The coefficient expressions follow ccc.cc:52-65 term for term (same       */
/* evaluation order), so the samples - and through them the image-plane     */
/* grid - agree with the reference to the last bit.                          */
/* ------------------------------------------------------------------------ */
static void get_cc(orc_lcirs *o) {
  cx c[7];
  const cx z2 = o->z2, z3 = o->z3;
  const double m2 = o->m2, m3 = o->m3;
  const double msum = m2 + m3 - 1.0;
  /* cc[1] = 2 z2 z3 (z2+z3) (m2+m3-1),  cc[0] = -z2 z2 z3 z3 (m2+m3-1) */
  c[1] = cscale(cmul(cmul(cscale(z2, 2.0), z3), cadd(z2, z3)), msum);
  c[0] = cscale(cmul(cmul(cmul(cneg(z2), z2), z3), z3), msum);
  cx temp[NBR];
  int have = 0;
  for (unsigned j = 0; j < NCC; j++) {
    double phi = 2.0 * 3.14159265359 * j / NCC;
    cx e = mk(cos(phi), sin(phi));
    c[6] = cneg(e);
    c[5] = cmul(cscale(e, 2.0), cadd(z2, z3));
    /* 1 - e (z2 z2 + z3 z3 + 4 z2 z3) */
    c[4] = csub(mk(1.0, 0.0),
                cmul(e, cadd(cadd(cmul(z2, z2), cmul(z3, z3)),
                             cmul(cscale(z2, 4.0), z3))));
    /* 2 e z2 z3 (z2+z3) + 2 z2 (m2-1) + 2 z3 (m3-1) */
    c[3] = cadd(cadd(cmul(cmul(cmul(cscale(e, 2.0), z2), z3), cadd(z2, z3)),
                     cscale(cscale(z2, 2.0), m2 - 1.0)),
                cscale(cscale(z3, 2.0), m3 - 1.0));
    /* -e z2 z2 z3 z3 + 4 (1-m3-m2) z2 z3 - z2 z2 (m2-1) - z3 z3 (m3-1) */
    c[2] = csub(csub(cadd(cmul(cmul(cmul(cmul(cneg(e), z2), z2), z3), z3),
                          cmul(cscale(z2, 4.0 * (1.0 - m3 - m2)), z3)),
                     cscale(cmul(z2, z2), m2 - 1.0)),
                cscale(cmul(z3, z3), m3 - 1.0));
    if (!have) {
      solve_roots(c, 6, NULL, temp);
      have = 1;
    } else {
      polish_roots(c, 6, temp);
      if (!check_roots(c, 6, temp)) solve_roots(c, 6, NULL, temp);
    }
    for (int k = 0; k < NBR; k++) o->cc[k][j] = temp[k];
  }
}

/* ccc.cc:160-203 (triple branch: the LensPar constructor never sets
 * _binaryLens, ccc.cc:29-39) */
static void get_ca(orc_lcirs *o) {
  for (int k = 0; k < NBR; k++)
    for (int j = 0; j < NCC; j++) {
      cx s = o->cc[k][j];
      cx t = csub(s, rdiv(o->m1, cconj(csub(s, o->z1))));
      t = csub(t, rdiv(o->m2, cconj(csub(s, o->z2))));
      t = csub(t, rdiv(o->m3, cconj(csub(s, o->z3))));
      o->ca[k][j] = t;
    }
}

/* utils.h:16-29 */
static void minmax(const cx *v, int n, cx *mn, cx *mx) {
  for (int i = 0; i < n; i++) {
    if (v[i].re < mn->re) mn->re = v[i].re;
    if (v[i].im < mn->im) mn->im = v[i].im;
    if (v[i].re > mx->re) mx->re = v[i].re;
    if (v[i].im > mx->im) mx->im = v[i].im;
  }
}

/* lcirs.cc:39-48.  Q3: min/max start at the origin and are never reset, so
 * box k envelopes branches 0..k and the origin. */
static void get_ca_boxes(orc_lcirs *o) {
  cx mn = mk(0.0, 0.0), mx = mk(0.0, 0.0);
  for (int k = 0; k < NBR; k++) {
    minmax(o->ca[k], NCC, &mn, &mx);
    o->box_min[k] = mn;
    o->box_max[k] = mx;
  }
}

/* lcirs.cc:51-92 */
static void get_img_plane_pars(orc_lcirs *o) {
  const double resizing = 3.0;
  cx mn = mk(0.0, 0.0), mx = mk(0.0, 0.0);
  for (int k = 0; k < NBR; k++) minmax(o->cc[k], NCC, &mn, &mx);
  double half = mx.re - mn.re;
  if (mx.im - mn.im > half) half = mx.im - mn.im;
  half *= resizing / 2.0;
  double cxr = (mx.re + mn.re) / 2.0, cxi = (mx.im + mn.im) / 2.0;
  o->g.top_x = cxr + half;
  o->g.top_y = cxi + half;
  o->g.corner_x = cxr - half;
  o->g.corner_y = cxi - half;
  o->g.n = (int64_t)(2 * half / o->rho * o->ppr);
  o->g.size_double = 2 * half;
  o->g.amp_scale = o->intensity / M_PI / pow((double)o->ppr, 2.0);
  o->g.h = o->g.size_double / ((double)o->g.n - 1.0);
}

/* ------------------------------------------------------------------------ */
/* Degree-10 lens polynomial: imgpoint.cc:160-176 adds the cached zeta-free  */
/* part (imgpointcoeff.cc:223-278) and the zeta part (:280-447) term by      */
/* term.  Both expression trees live in lens_coeffs.c, in the reference's   */
/* evaluation order.                                                         */
/* ------------------------------------------------------------------------ */
void orc_coeffs_nozeta(double m2, double m3, const double z2xy[2], const double z3xy[2],
                       double _Complex out[11]);
void orc_coeffs_zeta(double m2, double m3, const double z2xy[2], const double z3xy[2],
                     double zx, double zy, double _Complex out[11]);

static void lens_poly_init(orc_lcirs *o) {
  double _Complex c[11];
  const double z2[2] = {o->z2.re, o->z2.im}, z3[2] = {o->z3.re, o->z3.im};
  orc_coeffs_nozeta(o->m2, o->m3, z2, z3, c);
  for (int k = 0; k < 11; k++) o->coef_nozeta[k] = mk(__real__ c[k], __imag__ c[k]);
}

static void lens_poly(const orc_lcirs *o, cx zeta, cx *c /* 11 */) {
  double _Complex d[11];
  const double z2[2] = {o->z2.re, o->z2.im}, z3[2] = {o->z3.re, o->z3.im};
  orc_coeffs_zeta(o->m2, o->m3, z2, z3, zeta.re, zeta.im, d);
  for (int k = 0; k < 11; k++) c[k] = cadd(o->coef_nozeta[k], mk(__real__ d[k], __imag__ d[k]));
}

/* imgpoint.cc:72-90 */
static int img_check(const orc_lcirs *o, cx img, cx src, double radius) {
  cx t = csub(img, rdiv(o->m1, cconj(csub(img, o->z1))));
  t = csub(t, rdiv(o->m2, cconj(csub(img, o->z2))));
  t = csub(t, rdiv(o->m3, cconj(csub(img, o->z3))));
  return cabs_(csub(t, src)) < radius;
}

/* tcache model: a 256-byte request takes the most recently freed chunk */
static cx heap_pop(orc_lcirs *o) {
  if (o->heap_n > 0) return o->heap[--o->heap_n];
  return mk(0.0, 0.0); /* a chunk carved from fresh memory */
}
static void heap_push(orc_lcirs *o, cx slot) {
  if (o->heap_n < 8) o->heap[o->heap_n++] = slot;
}
/* _tempRoots = <new roots vector>: the solver's result vector took a chunk
 * (pushed to capacity 16 by its 9th root), then the old buffer is freed. */
static void temp_roots_replaced(orc_lcirs *o) {
  cx v = heap_pop(o);
  if (o->have_temp_chunk) heap_push(o, o->temp_slot);
  o->temp_slot = v;
  o->have_temp_chunk = 1;
}

/* imgpoint.cc:160-205 */
static void get_roots_precalculated(orc_lcirs *o, cx zeta, int force, cx *roots) {
  cx c[11];
  lens_poly(o, zeta, c);
  if (!o->have_temp || force) {
    solve_roots(c, 10, NULL, o->temp_roots);
    temp_roots_replaced(o);
    o->have_temp = 1;
  } else {
    cx fresh[10];
    o->temp_roots[10] = o->temp_slot;
    if (o->trace && o->trace_n < o->trace_cap) {
      o->trace[2 * o->trace_n] = o->temp_slot.re;
      o->trace[2 * o->trace_n + 1] = o->temp_slot.im;
      o->trace_n++;
    }
    solve_roots(c, 10, o->temp_roots, fresh);
    memcpy(o->temp_roots, fresh, sizeof(fresh));
    temp_roots_replaced(o);
    if (!check_roots(c, 10, o->temp_roots)) {
      solve_roots(c, 10, NULL, o->temp_roots);
      temp_roots_replaced(o);
    }
  }
  memcpy(roots, o->temp_roots, 10 * sizeof(cx));
}

static double img_residual(const orc_lcirs *o, cx img, cx src) {
  cx t = csub(img, rdiv(o->m1, cconj(csub(img, o->z1))));
  t = csub(t, rdiv(o->m2, cconj(csub(img, o->z2))));
  t = csub(t, rdiv(o->m3, cconj(csub(img, o->z3))));
  return cabs_(csub(t, src));
}

/* Is the root a genuine solution of the lens equation?  Newton's method on
 * F(z) = z - sum m_i/conj(z - z_i) - zeta, whose linearisation is
 * F(z+d) = F + d + gamma conj(d) with gamma = sum m_i/conj(z - z_i)^2, so
 * d = (gamma conj(F) - F)/(1 - |gamma|^2).  Diagnostic only: it never changes
 * the image set, it tells whether the filter's decision was safe. */
static int true_image(const orc_lcirs *o, cx z, cx zeta) {
  const cx zs[3] = {o->z1, o->z2, o->z3};
  const double ms[3] = {o->m1, o->m2, o->m3};
  cx z0 = z;
  for (int it = 0; it < 30; it++) {
    cx F = csub(z, zeta), g = mk(0.0, 0.0);
    for (int i = 0; i < 3; i++) {
      cx w = cconj(csub(z, zs[i]));
      F = csub(F, rdiv(ms[i], w));
      g = cadd(g, rdiv(ms[i], cmul(w, w)));
    }
    double det = 1.0 - cnorm(g);
    if (cabs_(F) < 1e-13) return cabs_(csub(z, z0)) < 1e-3;
    if (fabs(det) < 1e-300) return 0;
    cx d = cscale(csub(cmul(g, cconj(F)), F), 1.0 / det);
    z = cadd(z, d);
  }
  return 0;
}

static int filter_images(orc_lcirs *o, const cx *roots, cx zeta, cx *imgs) {
  int n = 0;
  for (int k = 0; k < 10; k++) {
    int accepted = img_check(o, roots[k], zeta, 1.0e-6);
    if (accepted) {
      imgs[n++] = roots[k];
      /* the ImgPoint image list outgrows capacity 8 once and keeps its
       * 256-byte buffer for the life of the object */
      if (n == 9 && !o->imgs_big) {
        heap_pop(o);
        o->imgs_big = 1;
      }
    }
    /* The image set depends on rounding when a residual sits within a decade
     * of the 1e-6 filter radius (double roots at caustic points), or when
     * the filter's verdict disagrees with the lens equation itself (roots
     * next to a small-mass lens, where the residual amplifies the root's
     * rounding error by m_i/|z - z_i|^2). */
    double r = img_residual(o, roots[k], zeta);
    if (r > 1.0e-7 && r < 1.0e-5) o->fragile = 1;
    if (r < o->fragile_band && accepted != true_image(o, roots[k], zeta)) o->fragile = 1;
    /* an image next to a lens: the residual amplifies the root's rounding
     * error by kappa = sum m_i/|z - z_i|^2, so implementations whose
     * polynomial coefficients round differently accept or reject it */
    if (r < 1.0e-2 && (accepted || true_image(o, roots[k], zeta))) {
      cx z = roots[k];
      double kap = o->m1 / cnorm(csub(z, o->z1)) + o->m2 / cnorm(csub(z, o->z2)) +
                   o->m3 / cnorm(csub(z, o->z3));
      if (kap > o->kappa_max) o->fragile = 1;
    }
  }
  return n;
}

static int wrong_count(const orc_lcirs *o, int n) {
  if (!o->is_binary_img) return (n % 2 != 0 || n < 4);
  return (n % 2 != 1 || n < 3);
}

/* imgpoint.cc:208-274, 281-286 */
static int get_images(orc_lcirs *o, cx zeta, cx *imgs) {
  cx roots[10];
  get_roots_precalculated(o, zeta, 0, roots);
  int n = filter_images(o, roots, zeta, imgs);
  if (wrong_count(o, n)) {
    get_roots_precalculated(o, zeta, 1, roots);
    n = filter_images(o, roots, zeta, imgs);
  }
  return n;
}

/* ------------------------------------------------------------------------ */
/* Ray map, grid maps                                                        */
/* ------------------------------------------------------------------------ */
/* lcirs.cc:290-341 (irsSIMD), lanes (L0..L3) = (z3, z2, z1, zeta). */
static inline double irs_simd(const orc_lcirs *o, double x, double y, cx src) {
  double wr0 = o->z3.re - x, wr1 = o->z2.re - x, wr2 = o->z1.re - x, wr3 = src.re - x;
  double wi0 = o->z3.im - y, wi1 = o->z2.im - y, wi2 = o->z1.im - y, wi3 = src.im - y;
  double n0 = wr0 * wr0 + wi0 * wi0;
  double n1 = wr1 * wr1 + wi1 * wi1;
  double n2 = wr2 * wr2 + wi2 * wi2;
  double c0 = o->m3 / n0, c1 = o->m2 / n1, c2 = o->m1 / n2, c3 = 1.0 / -1.0;
  double tr0 = wr0 * c0, tr1 = wr1 * c1, tr2 = wr2 * c2, tr3 = wr3 * c3;
  double ti0 = wi0 * c0, ti1 = wi1 * c1, ti2 = wi2 * c2, ti3 = wi3 * c3;
  double sr0 = tr0 + tr2, sr1 = tr1 + tr3;
  double si0 = ti0 + ti2, si1 = ti1 + ti3;
  return (sr0 + sr1) * (sr0 + sr1) + (si0 + si1) * (si0 + si1);
}

/* lcirs.cc:345-353 (irsBinary, used when m3 == 0) */
static inline double irs_binary(const orc_lcirs *o, double x, double y, cx src) {
  cx img = mk(x, y);
  cx t = csub(img, rdiv(o->m1, cconj(csub(img, o->z1))));
  t = csub(t, rdiv(o->m2, cconj(csub(img, o->z2))));
  return cnorm(csub(t, src));
}

static inline double irs(const orc_lcirs *o, double x, double y, cx src) {
  return o->m3 == 0.0 ? irs_binary(o, x, y, src) : irs_simd(o, x, y, src);
}

double orc_irs(const orc_lcirs *o, double x, double y, double sx, double sy) {
  return irs(o, x, y, mk(sx, sy));
}

/* lcirs.cc:355-379 */
static inline double nx_to_x(const orc_lcirs *o, int64_t nx) {
  return o->g.corner_x + o->g.h * (double)nx;
}
static inline double ny_to_y(const orc_lcirs *o, int64_t ny) {
  return o->g.corner_y + o->g.h * (double)ny;
}
static inline int64_t x_to_nx(const orc_lcirs *o, double x) {
  return (int64_t)((x - o->g.corner_x) * (double)o->g.n / o->g.size_double + 0.5);
}
static inline int64_t y_to_ny(const orc_lcirs *o, double y) {
  return (int64_t)((y - o->g.corner_y) * (double)o->g.n / o->g.size_double + 0.5);
}

/* ------------------------------------------------------------------------ */
/* Amoeba: src/Utils/amoeba.cc (row -> list of x ranges)                     */
/* ------------------------------------------------------------------------ */
static void amoeba_reset(orc_lcirs *o) {
  if (!o->rows) {
    o->rows_cap = 1 << 12;
    o->rows = (orc_row *)calloc((size_t)o->rows_cap, sizeof(orc_row));
    o->ranges_cap = 1 << 12;
    o->ranges = (orc_range *)malloc((size_t)o->ranges_cap * sizeof(orc_range));
  } else {
    memset(o->rows, 0, (size_t)o->rows_cap * sizeof(orc_row));
  }
  o->rows_used = 0;
  o->ranges_used = 0;
}

static inline uint64_t mix64(uint64_t k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdULL;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ULL;
  k ^= k >> 33;
  return k;
}

static orc_row *row_find(orc_lcirs *o, int64_t ny) {
  uint64_t m = (uint64_t)o->rows_cap - 1;
  for (uint64_t i = mix64((uint64_t)ny) & m;; i = (i + 1) & m) {
    orc_row *r = &o->rows[i];
    if (!r->used) return NULL;
    if (r->key == ny) return r;
  }
}

static void rows_grow(orc_lcirs *o);

static orc_row *row_insert(orc_lcirs *o, int64_t ny) {
  if (2 * (o->rows_used + 1) > o->rows_cap) rows_grow(o);
  uint64_t m = (uint64_t)o->rows_cap - 1;
  for (uint64_t i = mix64((uint64_t)ny) & m;; i = (i + 1) & m) {
    orc_row *r = &o->rows[i];
    if (!r->used) {
      r->used = 1;
      r->key = ny;
      r->head = r->tail = -1;
      o->rows_used++;
      return r;
    }
  }
}

static void rows_grow(orc_lcirs *o) {
  orc_row *old = o->rows;
  long oc = o->rows_cap;
  o->rows_cap = oc * 2;
  o->rows = (orc_row *)calloc((size_t)o->rows_cap, sizeof(orc_row));
  o->rows_used = 0;
  for (long i = 0; i < oc; i++)
    if (old[i].used) {
      orc_row *r = row_insert(o, old[i].key);
      r->head = old[i].head;
      r->tail = old[i].tail;
    }
  free(old);
}

static void range_append(orc_lcirs *o, orc_row *r, int64_t xl, int64_t xr) {
  if (o->ranges_used == o->ranges_cap) {
    o->ranges_cap *= 2;
    o->ranges = (orc_range *)realloc(o->ranges, (size_t)o->ranges_cap * sizeof(orc_range));
  }
  int32_t id = (int32_t)o->ranges_used++;
  o->ranges[id].xl = xl;
  o->ranges[id].xr = xr;
  o->ranges[id].next = -1;
  if (r->tail < 0)
    r->head = id;
  else
    o->ranges[r->tail].next = id;
  r->tail = id;
}

/* amoeba.cc:15-30 */
static void add_node(orc_lcirs *o, int64_t nl, int64_t nr, int64_t ny) {
  orc_row *r = row_find(o, ny);
  if (!r) {
    r = row_insert(o, ny);
    range_append(o, r, nl, nr);
    return;
  }
  for (int32_t i = r->head; i >= 0; i = o->ranges[i].next)
    if (o->ranges[i].xr == nr && o->ranges[i].xl == nl) return;
  range_append(o, r, nl, nr);
}

/* amoeba.cc:34-52 */
static int check_line(orc_lcirs *o, int64_t ny, int64_t nx) {
  orc_row *r = row_find(o, ny);
  if (!r) return 1;
  if (ny < 0 || ny >= o->g.n) return 0;
  for (int32_t i = r->head; i >= 0; i = o->ranges[i].next)
    if (nx <= o->ranges[i].xr && o->ranges[i].xl <= nx) return 0;
  return 1;
}

/* amoeba.cc:56-82 */
static int check_line_shift(orc_lcirs *o, int64_t ny, int64_t *nx) {
  if (ny < 0 || ny >= o->g.n) {
    *nx += o->g.n;
    return 0;
  }
  orc_row *r = row_find(o, ny);
  if (!r) return 1;
  for (int32_t i = r->head; i >= 0; i = o->ranges[i].next)
    if (*nx <= o->ranges[i].xr && o->ranges[i].xl <= *nx) {
      *nx = o->ranges[i].xr + 2;
      return 0;
    }
  return 1;
}

/* ------------------------------------------------------------------------ */
/* lineFloodFill: lcirs.cc:381-466, recursion unrolled onto an explicit     */
/* stack that visits pixels in the reference's order (so the FP64 sum of    */
/* weights is accumulated in the same order).                                */
/* ------------------------------------------------------------------------ */
typedef struct {
  int64_t nx, ny, nl, nr, nn;
  double y;
  int stage, checked;
} fill_frame;

static inline void accept_ray(orc_lcirs *o, double rsq) {
  rsq = rsq / o->rho2;
  o->amplification += o->ld_a + o->ld_b * sqrt(1.0 - rsq);
  o->irs_count++;
}

static void line_flood_fill(orc_lcirs *o, int64_t nx0, int64_t ny0, cx src) {
  long sp = 0;
  fill_frame *st = (fill_frame *)o->stack;
  const int64_t N = o->g.n;
#define PUSH(NX, NY, CHK)                                                    \
  do {                                                                       \
    if (sp == o->stack_cap) {                                                \
      o->stack_cap = o->stack_cap ? 2 * o->stack_cap : 1024;                 \
      o->stack = realloc(o->stack, (size_t)o->stack_cap * sizeof(fill_frame)); \
      st = (fill_frame *)o->stack;                                           \
    }                                                                        \
    st[sp].nx = (NX);                                                        \
    st[sp].ny = (NY);                                                        \
    st[sp].stage = 0;                                                        \
    st[sp].checked = (CHK);                                                  \
    sp++;                                                                    \
  } while (0)

  PUSH(nx0, ny0, 0);
  while (sp > 0) {
    fill_frame *f = &st[sp - 1];
    if (f->stage == 0) {
      if (!f->checked) {
        if (f->ny <= 0 || f->ny >= N) { sp--; continue; }
        if (!check_line(o, f->ny, f->nx)) { sp--; continue; }
      }
      double y = ny_to_y(o, f->ny);
      double rsq = irs(o, nx_to_x(o, f->nx), y, src);
      if (!(rsq < o->rho2)) { sp--; continue; }
      accept_ray(o, rsq);
      int64_t nr, nl;
      for (nr = f->nx + 1; nr < N; nr++) {
        rsq = irs(o, nx_to_x(o, nr), y, src);
        if (!(rsq < o->rho2)) { nr--; break; }
        accept_ray(o, rsq);
      }
      for (nl = f->nx - 1; nl > 0; nl--) {
        rsq = irs(o, nx_to_x(o, nl), y, src);
        if (!(rsq < o->rho2)) { nl++; break; }
        accept_ray(o, rsq);
      }
      add_node(o, nl, nr, f->ny);
      f->nl = nl;
      f->nr = nr;
      f->nn = nl;
      f->y = y;
      f->stage = 1;
    }
    if (f->stage == 1 || f->stage == 2) {
      int64_t row = f->stage == 1 ? f->ny + 1 : f->ny - 1;
      int pushed = 0;
      while (f->nn <= f->nr) {
        int64_t nn = f->nn;
        if (check_line_shift(o, row, &nn)) {
          f->nn = nn + 1;
          int64_t cnx = nn;
          PUSH(cnx, row, 1);
          pushed = 1;
          break;
        }
        f->nn = nn;
      }
      if (pushed) continue;
      if (f->stage == 1) {
        f->stage = 2;
        f->nn = f->nl;
        continue;
      }
      sp--;
    }
  }
#undef PUSH
}

/* ------------------------------------------------------------------------ */
/* Caustic-crossing seeds: lcirs.cc:195-255                                  */
/* ------------------------------------------------------------------------ */
static int intersection_check(const orc_lcirs *o, cx src, cx A, cx B, cx *trial) {
  double rs2 = pow(o->rho, 2.0);
  cx bs = csub(B, src);
  double bd = cnorm(bs);
  cx as = csub(A, src);
  double ad = cnorm(as);
  int aout = ad > rs2, bout = bd > rs2;
  if (aout != bout) {
    *trial = bout ? A : B;
    return 1;
  } else if (aout && bout) {
    cx ab = csub(A, B);
    double abd = cnorm(ab);
    double proj = as.re * ab.re + as.im * ab.im;
    if (proj < 0) return 0;
    if (proj > abd) return 0;
    /* Q5: compares against rho (not rho^2 * |AB|) and forms A - B*proj/|AB|^2 */
    if (proj < o->rho) {
      *trial = csub(A, cscale(B, fabs(proj) / abd));
      cx st = csub(*trial, src);
      return cnorm(st) < rs2;
    }
    return 0;
  }
  return 0;
}

static void heap_construction_state(orc_lcirs *o) {
  /* Construction leaves five 256-byte chunks in the cache: each critical-
   * curve branch vector outgrows capacity 16 at sample 16 (ccc.cc:88-95,
   * branches in order) and frees a buffer whose slot 10 is sample 10 of that
   * branch; branch 5's chunk is taken again by the caustic branches and the
   * caustic boxes (lcirs.cc:39-48).  Verified on the reference build. */
  o->heap_n = 0;
  for (int k = 0; k < 5; k++) heap_push(o, o->cc[k][10]);
  o->have_temp_chunk = 0;
  o->temp_slot = mk(0.0, 0.0);
  o->imgs_big = 0;
}

/* The point's seed list imgPos (lcirs.cc:123) starts as a copy of the
 * image list, capacity = size, and doubles when full (libstdc++).  Its
 * 256-byte stage (capacity 16) takes a cached chunk and gives it back when it
 * grows again or when the point ends; slot 10 then holds seed 10. */
typedef struct { int size, cap; cx slot; } seed_list;

static void seed_list_push(orc_lcirs *o, seed_list *l, cx z) {
  if (l->size == l->cap) {
    int nc = l->cap ? 2 * l->cap : 1;
    cx slot = l->slot;
    if (nc == 16) l->slot = heap_pop(o);
    if (l->cap == 16) heap_push(o, slot);
    l->cap = nc;
  }
  if (l->size == 10 && l->cap == 16) l->slot = z;
  l->size++;
}

/* seeds of one point, lcirs.cc:123-165; returns the number of seeds */
static int point_seeds(orc_lcirs *o, cx pos, cx *seeds, int cap) {
  cx imgs[10];
  int n = get_images(o, pos, imgs);
  int ns = 0;
  seed_list sl = {n, n, mk(0.0, 0.0)};
  for (int k = 0; k < n; k++)
    if (ns < cap) seeds[ns++] = imgs[k];
  for (int k = 0; k < NBR; k++) {
    if (pos.re + o->rho >= o->box_min[k].re && pos.re - o->rho <= o->box_max[k].re &&
        pos.im + o->rho >= o->box_min[k].im && pos.im - o->rho <= o->box_max[k].im) {
      int taken = 0;
      for (int j = 0; j < NCC - 1; j++) {
        cx trial;
        if (intersection_check(o, pos, o->ca[k][j], o->ca[k][j + 1], &trial)) {
          if (!taken) {
            int m = get_images(o, trial, imgs);
            for (int q = 0; q < m; q++) {
              seed_list_push(o, &sl, imgs[q]);
              if (ns < cap) seeds[ns++] = imgs[q];
            }
            taken = 1;
          }
        } else {
          taken = 0;
        }
      }
    }
  }
  if (sl.cap == 16) heap_push(o, sl.slot);
  return ns;
}

/* ------------------------------------------------------------------------ */
/* public entry points                                                       */
/* ------------------------------------------------------------------------ */
orc_lcirs *orc_new(double a, double b, double th, double m2, double m3,
                   double rho, unsigned int lc_length, long ppr) {
  orc_lcirs *o = (orc_lcirs *)calloc(1, sizeof(orc_lcirs));
  o->a = a;
  o->b = b;
  o->th = th;
  o->m1 = 1.0 - m2 - m3;
  o->m2 = m2;
  o->m3 = m3;
  o->z1 = mk(0.0, 0.0);
  o->z2 = mk(a, 0.0);
  o->z3 = mk(b * cos(th), b * sin(th));
  o->is_binary_img = (a == 0.0 || b == 0.0 || m3 == 0.0);
  o->fragile_band = 1.0e-4;
  o->kappa_max = 300.0;
  o->rho = rho;
  o->rho2 = rho * rho;
  o->lc_length = lc_length;
  o->ppr = (int)ppr;
  ld_default(o);
  get_cc(o);
  get_ca(o);
  get_ca_boxes(o);
  get_img_plane_pars(o);
  lens_poly_init(o);
  heap_construction_state(o);
  return o;
}

/* Record the slot-10 value each warm solve starts root 10 from. */
void orc_set_trace(orc_lcirs *o, double *buf, long cap) {
  o->trace = buf;
  o->trace_cap = cap;
  o->trace_n = 0;
}
long orc_trace_count(const orc_lcirs *o) { return o->trace_n; }

void orc_free(orc_lcirs *o) {
  if (!o) return;
  free(o->rows);
  free(o->ranges);
  free(o->stack);
  free(o);
}

void orc_set_limb_darkening(orc_lcirs *o, const char *model, double v) {
  if (strcmp(model, "linear") == 0)
    ld_linear(o, v);
  else
    ld_default(o);
  o->g.amp_scale = o->intensity / M_PI / pow((double)o->ppr, 2.0);
}

void orc_grid_params(const orc_lcirs *o, orc_grid *g) { *g = o->g; }

void orc_copy_cc_ca(const orc_lcirs *o, double *cc_xy, double *ca_xy) {
  for (int k = 0; k < NBR; k++)
    for (int j = 0; j < NCC; j++) {
      long i = (long)k * NCC + j;
      if (cc_xy) { cc_xy[2 * i] = o->cc[k][j].re; cc_xy[2 * i + 1] = o->cc[k][j].im; }
      if (ca_xy) { ca_xy[2 * i] = o->ca[k][j].re; ca_xy[2 * i + 1] = o->ca[k][j].im; }
    }
}

void orc_lens(const orc_lcirs *o, double *m123, double *z_xy) {
  m123[0] = o->m1; m123[1] = o->m2; m123[2] = o->m3;
  z_xy[0] = o->z1.re; z_xy[1] = o->z1.im;
  z_xy[2] = o->z2.re; z_xy[3] = o->z2.im;
  z_xy[4] = o->z3.re; z_xy[5] = o->z3.im;
}

void orc_ld(const orc_lcirs *o, double *A, double *B, double *intensity) {
  *A = o->ld_a; *B = o->ld_b; *intensity = o->intensity;
}

/* Warm-start chain restarts.  The reference keeps one chain for the life of
 * the object (imgpoint.cc:184-198).  With chain_chunk = K > 0 the chain is
 * restarted cold at every point index that is a multiple of K, which is how
 * the GPU engine splits a trajectory into independent chunks. */
/* A restart returns the solver to the state the constructor leaves: no
 * roots, and the constructor's cache of freed chunks. */
static inline void chain_restart(orc_lcirs *o, unsigned i) {
  if (o->chain_chunk > 0 && i % (unsigned)o->chain_chunk == 0) {
    o->have_temp = 0;
    heap_construction_state(o);
  }
}

void orc_set_chain_chunk(orc_lcirs *o, int k) { o->chain_chunk = k; }
void orc_set_fragile_band(orc_lcirs *o, double r) { o->fragile_band = r; }

static inline cx traj_pos(cx s, cx e, unsigned i, unsigned n) {
  double t = (double)i / (double)n;
  cx d = csub(e, s);
  return cadd(s, cscale(d, t));
}

void orc_fill(orc_lcirs *o, double sx, double sy, const int64_t *seeds_xy,
              int n_seeds, double *amp, uint64_t *count) {
  cx src = mk(sx, sy);
  amoeba_reset(o);
  o->amplification = 0.0;
  o->irs_count = 0;
  for (int k = 0; k < n_seeds; k++)
    line_flood_fill(o, seeds_xy[2 * k], seeds_xy[2 * k + 1], src);
  *amp = o->amplification * o->g.amp_scale;
  *count = o->irs_count;
}

void orc_get_lc_irs(orc_lcirs *o, double x0, double y0, double x1, double y1,
                    double *amps, uint64_t *counts) {
  cx s = mk(x0, y0), e = mk(x1, y1);
  cx seeds[256];
  for (unsigned i = 0; i <= o->lc_length; i++) {
    cx pos = traj_pos(s, e, i, o->lc_length);
    chain_restart(o, i);
    int ns = point_seeds(o, pos, seeds, 256);
    amoeba_reset(o);
    o->amplification = 0.0;
    o->irs_count = 0;
    for (int k = 0; k < ns; k++)
      line_flood_fill(o, x_to_nx(o, seeds[k].re), y_to_ny(o, seeds[k].im), pos);
    amps[i] = o->amplification * o->g.amp_scale;
    counts[i] = o->irs_count;
  }
}

long orc_lc_seeds(orc_lcirs *o, double x0, double y0, double x1, double y1,
                  int max_seeds, int64_t *seeds_xy, int *seed_count, int *fragile) {
  cx s = mk(x0, y0), e = mk(x1, y1);
  cx seeds[256];
  long total = 0;
  for (unsigned i = 0; i <= o->lc_length; i++) {
    cx pos = traj_pos(s, e, i, o->lc_length);
    chain_restart(o, i);
    o->fragile = 0;
    int ns = point_seeds(o, pos, seeds, 256);
    seed_count[i] = ns;
    if (fragile) fragile[i] = o->fragile;
    for (int k = 0; k < ns && k < max_seeds; k++) {
      int64_t *p = seeds_xy + 2 * ((long)i * max_seeds + k);
      p[0] = x_to_nx(o, seeds[k].re);
      p[1] = y_to_ny(o, seeds[k].im);
    }
    total += ns;
  }
  return total;
}

long orc_last_amoeba(const orc_lcirs *o, int64_t *triples, long cap) {
  long n = 0;
  for (long i = 0; i < o->rows_cap; i++) {
    const orc_row *r = &o->rows[i];
    if (!r->used) continue;
    for (int32_t k = r->head; k >= 0; k = o->ranges[k].next) {
      if (n < cap) {
        triples[3 * n] = r->key;
        triples[3 * n + 1] = o->ranges[k].xl;
        triples[3 * n + 2] = o->ranges[k].xr;
      }
      n++;
    }
  }
  return n;
}

/* lcbase.cc:17-38: sum over images of 1/|1 - |sum m_i/(img-z_i)^2|^2|, with
 * std::pow(complex, 2.0) = polar(exp(2 log|w|), 2 arg w); NaN -> 0. */
static cx cpow2(cx w) {
  if (w.im == 0.0 && w.re > 0.0) return mk(pow(w.re, 2.0), 0.0);
  double lr = log(cabs_(w)), ar = atan2(w.im, w.re);
  double r = exp(2.0 * lr), t = 2.0 * ar;
  return mk(r * cos(t), r * sin(t));
}

static double image_amp(const orc_lcirs *o, cx img) {
  cx s = cadd(cadd(rdiv(o->m1, cpow2(csub(img, o->z1))), rdiv(o->m2, cpow2(csub(img, o->z2)))),
              rdiv(o->m3, cpow2(csub(img, o->z3))));
  double t = 1.0 / fabs(1.0 - cnorm(s));
  if (t != t) t = 0.0;
  return t;
}

static double point_amp(orc_lcirs *o, cx pos) {
  cx imgs[10];
  int n = get_images(o, pos, imgs);
  double amp = 0.0;
  for (int k = 0; k < n; k++) amp += image_amp(o, imgs[k]);
  return amp;
}

/* lcbase.cc:40-52 */
void orc_get_lc(orc_lcirs *o, double x0, double y0, double x1, double y1,
                double *amps) {
  cx s = mk(x0, y0), e = mk(x1, y1);
  for (unsigned i = 0; i < o->lc_length; i++) {
    double t = i / (o->lc_length - 1.0);
    cx pos = cadd(s, cscale(csub(e, s), t));
    chain_restart(o, i);
    amps[i] = point_amp(o, pos);
  }
}

int orc_get_images(orc_lcirs *o, double sx, double sy, double *img_xy) {
  cx imgs[10];
  int n = get_images(o, mk(sx, sy), imgs);
  for (int k = 0; k < n; k++) {
    img_xy[2 * k] = imgs[k].re;
    img_xy[2 * k + 1] = imgs[k].im;
  }
  return n;
}

int orc_images_cold(double a, double b, double th, double m2, double m3,
                    double sx, double sy, double *img_xy) {
  orc_lcirs o;
  memset(&o, 0, sizeof(o));
  o.m1 = 1.0 - m2 - m3;
  o.m2 = m2;
  o.m3 = m3;
  o.z1 = mk(0.0, 0.0);
  o.z2 = mk(a, 0.0);
  o.z3 = mk(b * cos(th), b * sin(th));
  o.is_binary_img = (a == 0.0 || b == 0.0 || m3 == 0.0);
  lens_poly_init(&o);
  cx imgs[10];
  int n = get_images(&o, mk(sx, sy), imgs);
  for (int k = 0; k < n; k++) {
    img_xy[2 * k] = imgs[k].re;
    img_xy[2 * k + 1] = imgs[k].im;
  }
  return n;
}

void orc_solve_roots(const double *coeffs, int deg, const double *init,
                     double *roots) {
  cx c[ORC_MAXC] = {{0.0, 0.0}}, in[ORC_MAXC], r[ORC_MAXC];
  if (deg < 1 || deg >= ORC_MAXC) return;
  for (int k = 0; k <= deg; k++) c[k] = mk(coeffs[2 * k], coeffs[2 * k + 1]);
  if (init)
    for (int k = 0; k <= deg; k++) in[k] = mk(init[2 * k], init[2 * k + 1]);
  solve_roots(c, deg, init ? in : NULL, r);
  for (int k = 0; k < deg; k++) { roots[2 * k] = r[k].re; roots[2 * k + 1] = r[k].im; }
}

int orc_laguerre(const double *coeffs, int deg, double *x) {
  cx c[ORC_MAXC];
  if (deg < 1 || deg >= ORC_MAXC) return 0;
  for (int k = 0; k <= deg; k++) c[k] = mk(coeffs[2 * k], coeffs[2 * k + 1]);
  cx z = mk(x[0], x[1]);
  int ok = lag_iter(c, deg, &z);
  x[0] = z.re;
  x[1] = z.im;
  return ok;
}

void orc_lens_poly(const orc_lcirs *o, double sx, double sy, double *c) {
  cx cc[11];
  lens_poly(o, mk(sx, sy), cc);
  for (int k = 0; k < 11; k++) { c[2 * k] = cc[k].re; c[2 * k + 1] = cc[k].im; }
}

/* Test hooks: the helpers above, for the host comparison tests. */
int orc_intersection_check(const orc_lcirs *o, double sx, double sy, double ax, double ay,
                           double bx, double by, double *trial_xy) {
  cx t = mk(0.0, 0.0);
  int hit = intersection_check(o, mk(sx, sy), mk(ax, ay), mk(bx, by), &t);
  trial_xy[0] = t.re;
  trial_xy[1] = t.im;
  return hit;
}

double orc_image_amp(const orc_lcirs *o, double ix, double iy) {
  return image_amp(o, mk(ix, iy));
}

void orc_grid_maps(const orc_lcirs *o, int64_t nx, int64_t ny, double x, double y,
                   double *xy_out, int64_t *n_out) {
  xy_out[0] = nx_to_x(o, nx);
  xy_out[1] = ny_to_y(o, ny);
  n_out[0] = x_to_nx(o, x);
  n_out[1] = y_to_ny(o, y);
}
