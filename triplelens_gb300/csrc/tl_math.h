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
// naive complex division (the reference's -Ofast build uses the same form)
TL_HD cx div(cx a, cx b) {
  double d = b.re * b.re + b.im * b.im;
  return mk((a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d);
}
TL_HD cx rdiv(double x, cx b) { return div(mk(x, 0.0), b); }
TL_HD double norm(cx a) { return a.re * a.re + a.im * a.im; }
TL_HD double cabs(cx a) { return sqrt(a.re * a.re + a.im * a.im); }
// principal square root, half-angle form: t = sqrt((|x| + |z|)/2)
TL_HD cx csqrt(cx a) {
  if (a.re == 0.0 && a.im == 0.0) return mk(0.0, a.im);
  double t = sqrt((fabs(a.re) + cabs(a)) * 0.5);
  if (a.re >= 0.0) return mk(t, a.im / (2.0 * t));
  return mk(fabs(a.im) / (2.0 * t), a.im < 0.0 ? -t : t);
}

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
    for (int j = m - 1; j >= 0; j--) {
      s = add(mul(x, s), f);
      f = add(mul(x, f), b);
      b = add(mul(x, b), poly[j]);
      err = cabs(b) + cabs(x) * err;
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
};

// Degree-10 lens polynomial, coefficients low -> high.  Own derivation: with
// Q = prod(z - z_k), P = sum_i m_i prod_{k!=i}(z - z_k) and
// R_i = (conj(zeta) - conj(z_i)) Q + P, the lens equation
// zeta = z - sum m_i / conj(z - z_i) becomes
//   (z - zeta) R1 R2 R3 - Q (m1 R2 R3 + m2 R1 R3 + m3 R1 R2) = 0,
// which is the reference's polynomial (imgpointcoeff.cc:223-447) up to a
// constant factor.
TL_HD void pmul(const cx* a, int da, const cx* b, int db, cx* out) {
  for (int i = 0; i <= da + db; i++) out[i] = mk(0.0, 0.0);
  for (int i = 0; i <= da; i++)
    for (int j = 0; j <= db; j++) out[i + j] = add(out[i + j], mul(a[i], b[j]));
}

TL_HD void lens_poly(const Lens& L, cx zeta, cx* c) {
  const cx zs[3] = {L.z1, L.z2, L.z3};
  const double ms[3] = {L.m1, L.m2, L.m3};
  cx l[3][2];
  for (int k = 0; k < 3; k++) {
    l[k][0] = neg(zs[k]);
    l[k][1] = mk(1.0, 0.0);
  }
  cx q2[3], Q[4];
  pmul(l[0], 1, l[1], 1, q2);
  pmul(q2, 2, l[2], 1, Q);
  cx P[3] = {mk(0.0, 0.0), mk(0.0, 0.0), mk(0.0, 0.0)};
  for (int i = 0; i < 3; i++) {
    cx t[3];
    pmul(l[(i + 1) % 3], 1, l[(i + 2) % 3], 1, t);
    for (int d = 0; d < 3; d++) P[d] = add(P[d], scale(t[d], ms[i]));
  }
  cx R[3][4];
  cx zc = conj(zeta);
  for (int i = 0; i < 3; i++) {
    cx f = sub(zc, conj(zs[i]));
    for (int d = 0; d < 4; d++) R[i][d] = mul(f, Q[d]);
    for (int d = 0; d < 3; d++) R[i][d] = add(R[i][d], P[d]);
  }
  cx r12[7], r13[7], r23[7], r123[10];
  pmul(R[0], 3, R[1], 3, r12);
  pmul(R[0], 3, R[2], 3, r13);
  pmul(R[1], 3, R[2], 3, r23);
  pmul(r12, 6, R[2], 3, r123);
  cx zl[2] = {neg(zeta), mk(1.0, 0.0)};
  pmul(zl, 1, r123, 9, c);
  cx s[7];
  for (int d = 0; d < 7; d++)
    s[d] = add(add(scale(r23[d], ms[0]), scale(r13[d], ms[1])), scale(r12[d], ms[2]));
  cx rhs[10];
  pmul(Q, 3, s, 6, rhs);
  for (int d = 0; d < 10; d++) c[d] = sub(c[d], rhs[d]);
}

// imgpoint.cc:72-90: |zeta(img) - zeta_s| < radius
TL_HD bool img_check(const Lens& L, cx img, cx src, double radius) {
  cx t = sub(img, rdiv(L.m1, conj(sub(img, L.z1))));
  t = sub(t, rdiv(L.m2, conj(sub(img, L.z2))));
  t = sub(t, rdiv(L.m3, conj(sub(img, L.z3))));
  return cabs(sub(t, src)) < radius;
}

// Warm-start state of the image solver along a trajectory
// (imgpoint.h:104-110: _tempRoots and its availability).
struct RootChain {
  cx roots[11];  // [10] is the slot the reference reads past its 10 roots
  int have;
};

TL_HD void chain_reset(RootChain* ch) {
  ch->have = 0;
  for (int k = 0; k < 11; k++) ch->roots[k] = mk(0.0, 0.0);
}

// imgpoint.cc:160-205 (getRootsPrecalculated)
TL_HD void chain_roots(const Lens& L, RootChain* ch, cx zeta, bool force, const TrigTable* trig) {
  cx c[11];
  lens_poly(L, zeta, c);
  if (!ch->have || force) {
    solve_roots(c, 10, nullptr, ch->roots, trig);
    ch->have = 1;
  } else {
    cx fresh[10];
    solve_roots(c, 10, ch->roots, fresh, trig);
    for (int k = 0; k < 10; k++) ch->roots[k] = fresh[k];
    if (!check_roots(c, 10, ch->roots)) solve_roots(c, 10, nullptr, ch->roots, trig);
  }
}

TL_HD int filter_images(const Lens& L, const cx* roots, cx zeta, cx* imgs) {
  int n = 0;
  for (int k = 0; k < 10; k++)
    if (img_check(L, roots[k], zeta, 1.0e-6)) imgs[n++] = roots[k];
  return n;
}

TL_HD bool wrong_count(const Lens& L, int n) {
  if (!L.is_binary_img) return (n % 2 != 0 || n < 4);
  return (n % 2 != 1 || n < 3);
}

// imgpoint.cc:208-274, 281-286: images of zeta through the chain.
TL_HD int chain_images(const Lens& L, RootChain* ch, cx zeta, cx* imgs, const TrigTable* trig) {
  chain_roots(L, ch, zeta, false, trig);
  int n = filter_images(L, ch->roots, zeta, imgs);
  if (wrong_count(L, n)) {
    chain_roots(L, ch, zeta, true, trig);
    n = filter_images(L, ch->roots, zeta, imgs);
  }
  return n;
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
