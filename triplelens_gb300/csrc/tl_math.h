// tl_math.h - lens math shared by host and device code of the engine.
//
// FP64 throughout.  Every operation is written as a separately rounded IEEE
// operation: the translation units that include this header are compiled with
// --fmad=false (device) and -ffp-contract=off (host), so a host build and the
// device build produce bit-identical roots, caustic samples and grid
// parameters.  Square roots and divisions are IEEE correctly rounded on both
// sides (nvcc's default -prec-div/-prec-sqrt).
//
// Reference algorithms restated here (TripleLens, paths from its root):
//   Laguerre iteration / deflation / polish / check  src/Laguerre/laguerre.cc:18-198
//   critical curve polynomial                         src/CCC/ccc.cc:52-65
//   caustic map                                       src/CCC/ccc.cc:160-203
//   image filter                                      src/Images/imgpoint.cc:72-90
//   image-count retry                                 src/Images/imgpoint.cc:208-274
//   caustic-crossing test                             src/LightCurves/lcirs.cc:195-255
//   grid maps                                         src/LightCurves/lcirs.cc:355-379
#pragma once

#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define TL_HD __host__ __device__ __forceinline__
#else
#define TL_HD inline
#endif

namespace tl {

struct cx {
  double re, im;
};

TL_HD cx mk(double re, double im) {
  cx z;
  z.re = re;
  z.im = im;
  return z;
}
TL_HD cx add(cx a, cx b) { return mk(a.re + b.re, a.im + b.im); }
TL_HD cx sub(cx a, cx b) { return mk(a.re - b.re, a.im - b.im); }
TL_HD cx neg(cx a) { return mk(-a.re, -a.im); }
TL_HD cx conj(cx a) { return mk(a.re, -a.im); }
TL_HD cx mul(cx a, cx b) { return mk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
TL_HD cx scale(cx a, double s) { return mk(a.re * s, a.im * s); }

// Complex division as std::complex<double> divides in a strict IEEE build:
// Smith's algorithm (R. L. Smith, "Algorithm 116: Complex division",
// CACM 5(8), 1962), the method of libgcc's __divdc3.  For operands of this
// path no scaling branch of that routine is ever taken, and scaling by a
// power of two would not change the quotient anyway; the branch for a
// subnormal ratio is kept.
TL_HD cx div(cx a, cx b) {
  if (fabs(b.re) < fabs(b.im)) {
    const double r = b.re / b.im, den = b.re * r + b.im;
    if (fabs(r) > 2.2250738585072014e-308)
      return mk((a.re * r + a.im) / den, (a.im * r - a.re) / den);
    return mk((b.re * (a.re / b.im) + a.im) / den, (b.re * (a.im / b.im) - a.re) / den);
  }
  const double r = b.im / b.re, den = b.im * r + b.re;
  if (fabs(r) > 2.2250738585072014e-308)
    return mk((a.im * r + a.re) / den, (a.im - a.re * r) / den);
  return mk((a.re + b.im * (a.im / b.re)) / den, (a.im - b.im * (a.re / b.re)) / den);
}
TL_HD cx rdiv(double x, cx b) { return div(mk(x, 0.0), b); }
TL_HD double norm(cx a) { return a.re * a.re + a.im * a.im; }

// |z| as std::abs(complex<double>) computes it in a strict IEEE build: the
// C library's hypot.  Method of C. F. Borges, "An improved algorithm for
// hypot(a,b)" (2019, arXiv:1904.09481): the naive root h = sqrt(x^2 + y^2),
// corrected by the residual h^2 - x^2 - y^2 re-expressed exactly through
// delta = h - max or h - min (the form without fused multiply-add), with
// power-of-two scaling far from 1.  Agrees bit for bit with glibc's hypot on
// x86-64 (checked on 2e7 random operands).
TL_HD double hypot_kernel(double ax, double ay) {
  double h = sqrt(ax * ax + ay * ay), t1, t2;
  if (h <= 2.0 * ay) {
    const double d = h - ay;
    t1 = ax * (2.0 * d - ax);
    t2 = (d - 2.0 * (ax - ay)) * d;
  } else {
    const double d = h - ax;
    t1 = 2.0 * d * (ax - 2.0 * ay);
    t2 = (4.0 * d - ay) * ay + d * d;
  }
  return h - (t1 + t2) / (2.0 * h);
}
TL_HD double hypot_ieee(double x, double y) {
  x = fabs(x);
  y = fabs(y);
  const double ax = x < y ? y : x, ay = x < y ? x : y;
  const double big = 6.703903964971299e+153;    // 2^511
  const double small = 1.4916681462400413e-154;  // 2^-511
  const double sc = 2.409919865102884e-181;      // 2^-600
  const double eps = 5.551115123125783e-17;      // 2^-54
  if (ax > big) {
    if (ay <= ax * eps) return ax + ay;
    return hypot_kernel(ax * sc, ay * sc) / sc;
  }
  if (ay < small) {
    if (ax >= ay / eps) return ax + ay;
    return hypot_kernel(ax / sc, ay / sc) * sc;
  }
  if (ay <= ax * eps) return ax + ay;
  return hypot_kernel(ax, ay);
}
TL_HD double cabs(cx a) { return hypot_ieee(a.re, a.im); }

// Principal square root as std::sqrt(complex<double>) computes it (the C
// library's csqrt): the half-angle form on hypot (W. Kahan, "Branch cuts for
// complex elementary functions", 1987), with 2 Re(r) Im(r) = Im(z) giving the
// smaller component without cancellation.
TL_HD cx csqrt(cx a) {
  if (a.im == 0.0) {
    if (a.re < 0.0) return mk(0.0, copysign(sqrt(-a.re), a.im));
    return mk(fabs(sqrt(a.re)), copysign(0.0, a.im));
  }
  if (a.re == 0.0) {
    const double r = sqrt(0.5 * fabs(a.im));
    return mk(r, copysign(r, a.im));
  }
  const double d = hypot_ieee(a.re, a.im);
  if (a.re > 0.0) {
    const double r = sqrt(0.5 * (d + a.re));
    return mk(r, 0.5 * (a.im / r));
  }
  const double s = sqrt(0.5 * (d - a.re));
  return mk(fabs(0.5 * (a.im / s)), copysign(s, a.im));
}

// Operators with std::complex<double>'s rounding: a real operand scales or
// shifts componentwise, complex products are (ac - bd, ad + bc).
TL_HD cx C(cx z) { return z; }
TL_HD cx C(double d) { return mk(d, 0.0); }
TL_HD cx operator+(cx a, cx b) { return add(a, b); }
TL_HD cx operator+(cx a, double d) { return mk(a.re + d, a.im); }
TL_HD cx operator+(double d, cx a) { return mk(d + a.re, a.im); }
TL_HD cx operator-(cx a, cx b) { return sub(a, b); }
TL_HD cx operator-(cx a, double d) { return mk(a.re - d, a.im); }
TL_HD cx operator-(double d, cx a) { return mk(d - a.re, -a.im); }
TL_HD cx operator-(cx a) { return neg(a); }
TL_HD cx operator*(cx a, cx b) { return mul(a, b); }
TL_HD cx operator*(cx a, double d) { return mk(a.re * d, a.im * d); }
TL_HD cx operator*(double d, cx a) { return mk(d * a.re, d * a.im); }

}  // namespace tl

#include "tl_coeffs.h"

namespace tl {

// ---------------------------------------------------------------------------
// Laguerre (laguerre.h:37-38: MAX_IT 300, MT 8)
// ---------------------------------------------------------------------------
constexpr int kMaxIt = 300;
constexpr int kMT = 8;
constexpr double kEps = 2.220446049250313080847e-16;

// cos(i), sin(i) for i = 0..kMaxIt, filled once on the host with libm and
// handed to the device, so both sides see the same values (laguerre.cc:77).
struct TrigTable {
  double c[kMaxIt + 1];
  double s[kMaxIt + 1];
};

TL_HD double frac_step(int k) {
  // laguerre.cc:22 fractional kicks; the reference indexes the 8-entry table
  // past its end from i = 64 on, here the index wraps modulo 8.
  switch (k & 7) {
    case 0: return 0.5;
    case 1: return 0.23;
    case 2: return 0.73;
    case 3: return 0.13;
    case 4: return 0.37;
    case 5: return 0.61;
    case 6: return 0.89;
    default: return 1.0;
  }
}

// laguerre.cc:18-99: one root of poly[0..m] starting from *px.
TL_HD bool laguerre(const cx* poly, int m, cx* px, const TrigTable* trig) {
  cx x = *px;
  if (m == 1) {
    if (cabs(poly[1]) != 0.0) {
      *px = neg(div(poly[0], poly[1]));
      return true;
    }
    *px = mk(999.0, 999.0);
    return false;
  }
  const double md = (double)m;
  for (int i = 1; i <= kMaxIt; i++) {
    cx b = poly[m];
    double err = cabs(b);
    cx s = mk(0.0, 0.0), f = mk(0.0, 0.0);
    const double ax = cabs(x);  // the reference takes |x| per term: same value
    for (int j = m - 1; j >= 0; j--) {
      s = add(mul(x, s), f);
      f = add(mul(x, f), b);
      b = add(mul(x, b), poly[j]);
      err = cabs(b) + ax * err;
    }
    err *= kEps;
    if (cabs(b) <= err) {
      *px = x;
      return true;
    }
    cx g = div(f, b);
    cx h = sub(mul(g, g), div(scale(s, 2.0), b));
    cx sq = csqrt(scale(sub(scale(h, md), mul(g, g)), md - 1.0));
    cx gp = add(g, sq), gm = sub(g, sq);
    if (cabs(gp) < cabs(gm)) gp = gm;
    cx dx;
    if (cabs(gp) > 0.0)
      dx = rdiv(md, gp);
    else
      dx = scale(mk(trig->c[i], trig->s[i]), 1.0 + cabs(x));
    cx x1 = sub(x, dx);
    if (x.re == x1.re && x.im == x1.im) {
      *px = x;
      return true;
    }
    if (i % kMT)
      x = x1;
    else
      x = sub(x, scale(dx, frac_step(i / kMT)));
  }
  *px = x;
  return false;
}

// laguerre.cc:103-167.  init == nullptr: cold start from (EPS, EPS); else root
// j (j = deg..1) starts from init[j] (init holds deg+1 entries: the
// reference's warm start reads one element past its deg roots at j = deg).
TL_HD void solve_roots(const cx* poly, int deg, const cx* init, cx* roots,
                       const TrigTable* trig) {
  cx temp[11];
  for (int k = 0; k <= deg; k++) temp[k] = poly[k];
  int nr = 0;
  for (int j = deg; j >= 1; j--) {
    cx x = init ? init[j] : mk(kEps, kEps);
    if (laguerre(temp, j, &x, trig)) {
      roots[nr++] = x;
    } else {
      if (init) x = mk(kEps, kEps);
      roots[nr++] = x;
    }
    cx b = temp[j];
    for (int jj = j - 1; jj >= 0; jj--) {
      cx c = temp[jj];
      temp[jj] = b;
      b = add(mul(x, b), c);
    }
  }
  for (int j = 0; j < deg; j++) laguerre(poly, deg, &roots[j], trig);
}

// laguerre.cc:188-198
TL_HD bool check_roots(const cx* poly, int deg, const cx* roots) {
  cx c0 = poly[deg];
  for (int k = 0; k < deg; k++) c0 = mul(c0, neg(roots[k]));
  if (cabs(poly[0]) > 1.0e-8) return (1.0 - cabs(div(c0, poly[0]))) < 1.0e-5;
  return cabs(sub(c0, poly[0])) < 1.0e-10;
}

// ---------------------------------------------------------------------------
// Lens
// ---------------------------------------------------------------------------
struct Lens {
  double m1, m2, m3;
  cx z1, z2, z3;
  int is_binary_img;  // imgpoint.cc:64: a == 0 || b == 0 || m3 == 0
  cx coef0[11];       // source-free polynomial part (imgpointcoeff.cc:223-278)
};

// Lens from the reference's constructor arguments, after z3 = b (cos, sin)
// has been formed with the host's libm (lens.cc:4-18, 35-40).
TL_HD void lens_finish(Lens* L) { coeffs_nozeta(L->m2, L->m3, L->z2, L->z3, L->coef0); }

// Degree-10 lens polynomial, coefficients low -> high (imgpoint.cc:164-176):
// the cached source-free part plus the source part, term by term.
TL_HD void lens_poly(const Lens& L, cx zeta, cx* c) {
  cx d[11];
  coeffs_zeta(L.m2, L.m3, L.z2, L.z3, zeta, d);
  for (int k = 0; k < 11; k++) c[k] = add(L.coef0[k], d[k]);
}

// imgpoint.cc:72-90: |zeta(img) - zeta_s| < radius
TL_HD bool img_check(const Lens& L, cx img, cx src, double radius) {
  cx t = sub(img, rdiv(L.m1, conj(sub(img, L.z1))));
  t = sub(t, rdiv(L.m2, conj(sub(img, L.z2))));
  t = sub(t, rdiv(L.m3, conj(sub(img, L.z3))));
  return cabs(sub(t, src)) < radius;
}

// ---------------------------------------------------------------------------
// Warm-start state of the image solver along a trajectory (imgpoint.h:104-110:
// _tempRoots), including the heap memory the reference's warm start reads.
//
// ImgPoint::getRootsPrecalculated warm-starts Laguerre::solveRoots from
// _tempRoots, whose root j = 10..1 starts from initRoots[j] (laguerre.cc:
// 111-128): root 10 reads one element past the end of the 10-element vector.
// That vector's buffer has capacity 16 (push_back growth), 256 bytes, and the
// slot holds whatever its chunk held before.  glibc serves 256-byte requests
// from a per-thread LIFO cache of freed chunks, and on this path only vectors
// of capacity 16 use that size class: each solver's result vector, the
// ImgPoint image list once it holds 9 images, a point's seed list while it
// holds 9-16 seeds, and, during construction, the six critical-curve branch
// vectors, which free their capacity-16 buffers at sample 16 (ccc.cc:88-95) -
// five of them stay cached (the sixth goes to the caustics and the caustic
// boxes).  The model keeps the slot-10 contents of the cached chunks (top
// last) and of the chunk _tempRoots holds, and replays every allocation and
// release of that size class in the reference's order.
// ---------------------------------------------------------------------------
constexpr int kHeapSlots = 8;   // the path never caches more than 5

struct RootChain {
  cx roots[11];        // _tempRoots; [10] is the slot a warm start reads
  int have;            // _tempRoots holds 10 roots
  int heap_n;          // cached chunks
  cx heap[kHeapSlots];
  int temp_chunk;      // _tempRoots owns a 256-byte chunk
  int imgs_big;        // the image list owns one (capacity 16)
};

// The state right after the LightCurveIRS constructor: heap0[k] = sample 10
// of critical-curve branch k, k = 0..4 (nullptr: an empty cache).
TL_HD void chain_reset(RootChain* ch, const cx* heap0) {
  ch->have = 0;
  for (int k = 0; k < 11; k++) ch->roots[k] = mk(0.0, 0.0);
  ch->heap_n = 0;
  for (int k = 0; k < kHeapSlots; k++) ch->heap[k] = mk(0.0, 0.0);
  if (heap0)
    for (int k = 0; k < 5; k++) ch->heap[ch->heap_n++] = heap0[k];
  ch->temp_chunk = 0;
  ch->imgs_big = 0;
}

TL_HD cx heap_take(RootChain* ch) {
  if (ch->heap_n > 0) return ch->heap[--ch->heap_n];
  return mk(0.0, 0.0);  // a chunk carved from fresh (zeroed) memory
}
TL_HD void heap_give(RootChain* ch, cx slot) {
  if (ch->heap_n < kHeapSlots) ch->heap[ch->heap_n++] = slot;
}

// _tempRoots = <solver result>: the result vector took a chunk, then the old
// buffer was released.
TL_HD void chain_replace_roots(RootChain* ch) {
  const cx v = heap_take(ch);
  if (ch->temp_chunk) heap_give(ch, ch->roots[10]);
  ch->roots[10] = v;
  ch->temp_chunk = 1;
}

// imgpoint.cc:160-205 (getRootsPrecalculated)
TL_HD void chain_roots(const Lens& L, RootChain* ch, cx zeta, bool force, const TrigTable* trig) {
  cx c[11];
  lens_poly(L, zeta, c);
  if (!ch->have || force) {
    solve_roots(c, 10, nullptr, ch->roots, trig);
    chain_replace_roots(ch);
    ch->have = 1;
  } else {
    cx fresh[10];
    solve_roots(c, 10, ch->roots, fresh, trig);
    for (int k = 0; k < 10; k++) ch->roots[k] = fresh[k];
    chain_replace_roots(ch);
    if (!check_roots(c, 10, ch->roots)) {
      solve_roots(c, 10, nullptr, ch->roots, trig);
      chain_replace_roots(ch);
    }
  }
}

TL_HD int filter_images(const Lens& L, RootChain* ch, cx zeta, cx* imgs) {
  int n = 0;
  for (int k = 0; k < 10; k++)
    if (img_check(L, ch->roots[k], zeta, 1.0e-6)) {
      imgs[n++] = ch->roots[k];
      if (n == 9 && !ch->imgs_big) {  // the image list outgrows capacity 8
        heap_take(ch);
        ch->imgs_big = 1;
      }
    }
  return n;
}

TL_HD bool wrong_count(const Lens& L, int n) {
  if (!L.is_binary_img) return (n % 2 != 0 || n < 4);
  return (n % 2 != 1 || n < 3);
}

// imgpoint.cc:208-274, 281-286: images of zeta through the chain.
TL_HD int chain_images(const Lens& L, RootChain* ch, cx zeta, cx* imgs, const TrigTable* trig) {
  chain_roots(L, ch, zeta, false, trig);
  int n = filter_images(L, ch, zeta, imgs);
  if (wrong_count(L, n)) {
    chain_roots(L, ch, zeta, true, trig);
    n = filter_images(L, ch, zeta, imgs);
  }
  return n;
}

// A point's seed list (lcirs.cc:123, imgPos): a copy of the image list
// (capacity = size) that doubles when full.  Its capacity-16 stage takes a
// cached chunk and gives it back when it grows again or when the point ends;
// slot 10 then holds seed 10.
struct SeedList {
  int size, cap;
  cx slot;
};
TL_HD void seed_list_start(SeedList* l, int n) {
  l->size = n;
  l->cap = n;
  l->slot = mk(0.0, 0.0);
}
TL_HD void seed_list_push(RootChain* ch, SeedList* l, cx z) {
  if (l->size == l->cap) {
    const int nc = l->cap ? 2 * l->cap : 1;
    const cx old = l->slot;
    if (nc == 16) l->slot = heap_take(ch);
    if (l->cap == 16) heap_give(ch, old);
    l->cap = nc;
  }
  if (l->size == 10 && l->cap == 16) l->slot = z;
  l->size++;
}
TL_HD void seed_list_end(RootChain* ch, const SeedList* l) {
  if (l->cap == 16) heap_give(ch, l->slot);
}

// lcbase.cc:17-38 per-image point magnification 1/|1 - |sum m_i/(z-z_i)^2|^2|
TL_HD double image_amp(const Lens& L, cx img) {
  cx w1 = sub(img, L.z1), w2 = sub(img, L.z2), w3 = sub(img, L.z3);
  cx s = add(add(rdiv(L.m1, mul(w1, w1)), rdiv(L.m2, mul(w2, w2))), rdiv(L.m3, mul(w3, w3)));
  double t = 1.0 / fabs(1.0 - norm(s));
  if (t != t) t = 0.0;
  return t;
}

// ---------------------------------------------------------------------------
// Critical curves and caustics (ccc.cc:42-98, 160-203)
// ---------------------------------------------------------------------------
constexpr int kCCLen = 500;
constexpr int kBranches = 6;

// Coefficients of the degree-6 critical-curve polynomial for one phase
// sample e = exp(i phi); the expressions keep ccc.cc:52-65's evaluation
// order so the samples agree with the reference to rounding.
TL_HD void cc_poly(const Lens& L, cx e, cx* c) {
  const cx z2 = L.z2, z3 = L.z3;
  const double m2 = L.m2, m3 = L.m3;
  const double msum = m2 + m3 - 1.0;
  c[1] = scale(mul(mul(scale(z2, 2.0), z3), add(z2, z3)), msum);
  c[0] = scale(mul(mul(mul(neg(z2), z2), z3), z3), msum);
  c[6] = neg(e);
  c[5] = mul(scale(e, 2.0), add(z2, z3));
  c[4] = sub(mk(1.0, 0.0), mul(e, add(add(mul(z2, z2), mul(z3, z3)), mul(scale(z2, 4.0), z3))));
  c[3] = add(add(mul(mul(mul(scale(e, 2.0), z2), z3), add(z2, z3)), scale(scale(z2, 2.0), m2 - 1.0)),
             scale(scale(z3, 2.0), m3 - 1.0));
  c[2] = sub(sub(add(mul(mul(mul(mul(neg(e), z2), z2), z3), z3), mul(scale(z2, 4.0 * (1.0 - m3 - m2)), z3)),
                 scale(mul(z2, z2), m2 - 1.0)),
             scale(mul(z3, z3), m3 - 1.0));
}

// ccc.cc:190-197 caustic point of a critical-curve point
TL_HD cx caustic_point(const Lens& L, cx s) {
  cx t = sub(s, rdiv(L.m1, conj(sub(s, L.z1))));
  t = sub(t, rdiv(L.m2, conj(sub(s, L.z2))));
  t = sub(t, rdiv(L.m3, conj(sub(s, L.z3))));
  return t;
}

// ---------------------------------------------------------------------------
// Grid (lcirs.cc:51-92, 355-379)
// ---------------------------------------------------------------------------
struct Grid {
  double corner_x, corner_y, top_x, top_y;
  double size_double, h, amp_scale;
  int64_t n;
};

TL_HD double nx_to_x(const Grid& g, int64_t nx) { return g.corner_x + g.h * (double)nx; }
TL_HD double ny_to_y(const Grid& g, int64_t ny) { return g.corner_y + g.h * (double)ny; }
TL_HD int64_t x_to_nx(const Grid& g, double x) {
  return (int64_t)((x - g.corner_x) * (double)g.n / g.size_double + 0.5);
}
TL_HD int64_t y_to_ny(const Grid& g, double y) {
  return (int64_t)((y - g.corner_y) * (double)g.n / g.size_double + 0.5);
}

// lcirs.cc:195-255 (Q5 replicated: compares proj*|AB| against rho and forms
// trial = A - B*proj/|AB|^2)
TL_HD bool intersection_check(double rho, cx src, cx A, cx B, cx* trial) {
  double rs2 = rho * rho;  // pow(rho, 2.0) is exact-rounded x*x
  cx bs = sub(B, src);
  double bd = norm(bs);
  cx as = sub(A, src);
  double ad = norm(as);
  bool aout = ad > rs2, bout = bd > rs2;
  if (aout != bout) {
    *trial = bout ? A : B;
    return true;
  } else if (aout && bout) {
    cx ab = sub(A, B);
    double abd = norm(ab);
    double proj = as.re * ab.re + as.im * ab.im;
    if (proj < 0) return false;
    if (proj > abd) return false;
    if (proj < rho) {
      *trial = sub(A, scale(B, fabs(proj) / abd));
      cx st = sub(*trial, src);
      return norm(st) < rs2;
    }
    return false;
  }
  return false;
}

}  // namespace tl
