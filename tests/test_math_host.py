"""The engine's shared FP64 math (triplelens_gb300/csrc/tl_math.h, compiled
into the seeds, chain, caustic and image kernels) against the oracle
(oracle/lcirs_oracle.c), bit for bit, without a GPU.

Both sides are compiled for the host with the engine's rounding rules (no
FMA contraction, no fast math): the engine's header with g++, the oracle
with gcc.  Compared on random lenses of the bench's distribution (every
tenth binary, m3 = 0):
  - the degree-10 lens polynomial (imgpoint.cc:164-176),
  - cold Laguerre solves with deflation and polish (laguerre.cc:103-167) of
    degree-10 lens polynomials and degree-6 polynomials,
  - single Laguerre iterations from random starts (laguerre.cc:18-99),
  - the warm-started image chain with its filter and cold retry
    (imgpoint.cc:160-274) and the heap-slot model of the warm start's read
    past the roots (laguerre.cc:111-128), along trajectories that run from
    one caustic sample to another, where images appear and vanish,
  - the critical curve and caustics in the lens set-up kernel's sequence
    (ccc.cc:55-94, 160-203), 3000 samples per lens,
  - the caustic-segment test with the reference's geometry (Q5,
    lcirs.cc:195-255), the grid maps (lcirs.cc:355-379),
  - and, to rounding times its condition number, each image's point-source
    magnification term (lcbase.cc:17-38; the reference squares with
    std::pow, the engine multiplies).
The oracle is pinned to the reference's strict build by the fixture tests,
so equality here pins the header the device kernels use.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

DRIVER = r"""
#include <cstdio>
#include <cstring>
#include <cmath>
#include "tl_math.h"

extern "C" {
struct orc_lcirs;
orc_lcirs* orc_new(double a, double b, double th, double m2, double m3, double rho,
                   unsigned int lc_length, long ppr);
void orc_free(orc_lcirs* o);
void orc_lens(const orc_lcirs* o, double* m123, double* z_xy);
void orc_copy_cc_ca(const orc_lcirs* o, double* cc_xy, double* ca_xy);
void orc_lens_poly(const orc_lcirs* o, double sx, double sy, double* c);
void orc_solve_roots(const double* coeffs, int deg, const double* init, double* roots);
int orc_laguerre(const double* coeffs, int deg, double* x);
int orc_get_images(orc_lcirs* o, double sx, double sy, double* img_xy);
int orc_intersection_check(const orc_lcirs* o, double sx, double sy, double ax, double ay,
                           double bx, double by, double* trial_xy);
double orc_image_amp(const orc_lcirs* o, double ix, double iy);
struct orc_grid {
  double corner_x, corner_y, top_x, top_y, size_double, h, amp_scale;
  int64_t n;
};
void orc_grid_params(const orc_lcirs* o, orc_grid* g);
void orc_grid_maps(const orc_lcirs* o, int64_t nx, int64_t ny, double x, double y,
                   double* xy_out, int64_t* n_out);
}

static unsigned long long s = 0x2545f4914f6cdd1dull;
static double u01() {
  s ^= s << 13; s ^= s >> 7; s ^= s << 17;
  return (double)(s >> 11) * (1.0 / 9007199254740992.0);
}
static bool eq(double a, double b) { return std::memcmp(&a, &b, 8) == 0; }
static bool eqc(tl::cx a, const double* b) { return eq(a.re, b[0]) && eq(a.im, b[1]); }

static double amp_rel_max = 0.0;
static long n_poly = 0, n_solve = 0, n_lag = 0, n_img = 0, n_pts = 0, n_cc = 0, n_isect = 0,
            n_hits = 0, n_grid = 0;

int main() {
  tl::TrigTable trig;
  for (int i = 0; i <= tl::kMaxIt; i++) {
    trig.c[i] = cos(1.0 * i);
    trig.s[i] = sin(1.0 * i);
  }
  static double cc[6 * 500 * 2], ca[6 * 500 * 2];
  // phase samples of the critical curve, filled on the host as the engine does
  static double pc[500], ps[500];
  for (unsigned j = 0; j < 500u; j++) {
    const double phi = 2.0 * 3.14159265359 * j / 500;
    pc[j] = cos(phi);
    ps[j] = sin(phi);
  }
  for (int lens = 0; lens < 60; lens++) {
    const double q2 = std::pow(10.0, -3.0 * u01());
    const double q3 = lens % 10 == 3 ? 0.0 : std::pow(10.0, -3.0 * u01());
    const double m2 = q2 / (1.0 + q2 + q3), m3 = q3 / (1.0 + q2 + q3);
    const double a = 0.5 * std::pow(4.0, u01()), b = 0.5 * std::pow(4.0, u01());
    const double th = 6.283185307179586 * u01();
    orc_lcirs* o = orc_new(a, b, th, m2, m3, 1e-3, 100, 10);
    double m123[3], z[6];
    orc_lens(o, m123, z);
    tl::Lens L;
    L.m1 = m123[0]; L.m2 = m123[1]; L.m3 = m123[2];
    L.z1 = tl::mk(z[0], z[1]); L.z2 = tl::mk(z[2], z[3]); L.z3 = tl::mk(z[4], z[5]);
    L.is_binary_img = (a == 0.0 || b == 0.0 || m3 == 0.0) ? 1 : 0;
    tl::lens_finish(&L);
    orc_copy_cc_ca(o, cc, ca);

    // critical curve and caustics: the lens set-up kernel's sequence (a cold
    // solve at the first phase, then each root polished on its own, a cold
    // solve again where the product check fails), ccc.cc:55-94, 182-200
    {
      tl::cx roots[6];
      for (int j = 0; j < 500; j++) {
        tl::cx c[7];
        tl::cc_poly(L, tl::mk(pc[j], ps[j]), c);
        if (j == 0) {
          tl::solve_roots(c, 6, nullptr, roots, &trig);
        } else {
          for (int k = 0; k < 6; k++) tl::laguerre(c, 6, &roots[k], &trig);
          if (!tl::check_roots(c, 6, roots)) tl::solve_roots(c, 6, nullptr, roots, &trig);
        }
        for (int k = 0; k < 6; k++, n_cc++) {
          const double* occ = cc + 2 * (k * 500 + j);
          const double* oca = ca + 2 * (k * 500 + j);
          if (!eqc(roots[k], occ) || !eqc(tl::caustic_point(L, roots[k]), oca)) {
            printf("FAIL critical curve lens %d branch %d sample %d\n", lens, k, j);
            return 1;
          }
        }
      }
    }

    // caustic-segment test (Q5 geometry) around random sources
    for (int p = 0; p < 400; p++, n_isect++) {
      const double rho = 1e-3;
      const double sx = 2.0 * (u01() - 0.5), sy = 2.0 * (u01() - 0.5);
      const double ra = rho * (0.3 + 2.0 * u01()), ta = 6.283185307179586 * u01();
      const double rb = rho * (0.3 + 2.0 * u01()), tb = 6.283185307179586 * u01();
      const double ax = sx + ra * cos(ta), ay = sy + ra * sin(ta);
      const double bx = sx + rb * cos(tb), by = sy + rb * sin(tb);
      tl::cx trial = tl::mk(0.0, 0.0);
      double otr[2];
      const bool hit = tl::intersection_check(rho, tl::mk(sx, sy), tl::mk(ax, ay), tl::mk(bx, by),
                                              &trial);
      const int ohit = orc_intersection_check(o, sx, sy, ax, ay, bx, by, otr);
      if (hit != (ohit != 0) || (hit && !eqc(trial, otr))) {
        printf("FAIL intersection lens %d case %d: %d vs %d\n", lens, p, (int)hit, ohit);
        return 1;
      }
      n_hits += hit;
    }

    // grid maps of the oracle's own grid
    {
      orc_grid og;
      orc_grid_params(o, &og);
      tl::Grid g;
      g.corner_x = og.corner_x; g.corner_y = og.corner_y; g.top_x = og.top_x; g.top_y = og.top_y;
      g.size_double = og.size_double; g.h = og.h; g.amp_scale = og.amp_scale; g.n = og.n;
      for (int p = 0; p < 200; p++, n_grid++) {
        const int64_t nx = (int64_t)(u01() * (double)g.n), ny = (int64_t)(u01() * (double)g.n);
        const double x = g.corner_x + u01() * g.size_double, y = g.corner_y + u01() * g.size_double;
        double oxy[2];
        int64_t on[2];
        orc_grid_maps(o, nx, ny, x, y, oxy, on);
        if (!eq(tl::nx_to_x(g, nx), oxy[0]) || !eq(tl::ny_to_y(g, ny), oxy[1]) ||
            tl::x_to_nx(g, x) != on[0] || tl::y_to_ny(g, y) != on[1]) {
          printf("FAIL grid lens %d case %d\n", lens, p);
          return 1;
        }
      }
    }

    // polynomial, cold solve, single iterations
    for (int p = 0; p < 40; p++) {
      const double sx = 3.0 * (u01() - 0.5), sy = 3.0 * (u01() - 0.5);
      tl::cx c[11], r[11];
      double oc[22], orr[22];
      tl::lens_poly(L, tl::mk(sx, sy), c);
      orc_lens_poly(o, sx, sy, oc);
      for (int k = 0; k < 11; k++, n_poly++)
        if (!eqc(c[k], oc + 2 * k)) { printf("FAIL lens_poly %d %d %d\n", lens, p, k); return 1; }
      tl::solve_roots(c, 10, nullptr, r, &trig);
      orc_solve_roots(oc, 10, nullptr, orr);
      for (int k = 0; k < 10; k++, n_solve++)
        if (!eqc(r[k], orr + 2 * k)) { printf("FAIL solve10 %d %d %d\n", lens, p, k); return 1; }
      tl::cx x = tl::mk(2.0 * (u01() - 0.5), 2.0 * (u01() - 0.5));
      double ox[2] = {x.re, x.im};
      const bool ok = tl::laguerre(c, 10, &x, &trig);
      const int ook = orc_laguerre(oc, 10, ox);
      n_lag++;
      if (ok != (ook != 0) || !eqc(x, ox)) { printf("FAIL laguerre %d %d\n", lens, p); return 1; }
      // a degree-6 polynomial from random roots (the critical-curve degree)
      tl::cx q[7] = {tl::mk(1.0, 0.0)};
      for (int k = 1; k < 7; k++) q[k] = tl::mk(0.0, 0.0);
      for (int k = 0; k < 6; k++) {
        const tl::cx root = tl::mk(2.0 * (u01() - 0.5), 2.0 * (u01() - 0.5));
        for (int j = 6; j >= 1; j--) q[j] = tl::sub(q[j - 1], tl::mul(root, q[j]));
        q[0] = tl::neg(tl::mul(root, q[0]));
      }
      double oq[14], orr6[12];
      for (int k = 0; k < 7; k++) { oq[2 * k] = q[k].re; oq[2 * k + 1] = q[k].im; }
      tl::solve_roots(q, 6, nullptr, r, &trig);
      orc_solve_roots(oq, 6, nullptr, orr6);
      for (int k = 0; k < 6; k++, n_solve++)
        if (!eqc(r[k], orr6 + 2 * k)) { printf("FAIL solve6 %d %d %d\n", lens, p, k); return 1; }
    }

    // warm-started image chain from the constructor's state, across caustics
    tl::RootChain ch;
    tl::cx heap0[5];
    for (int k = 0; k < 5; k++) heap0[k] = tl::mk(cc[2 * (k * 500 + 10)], cc[2 * (k * 500 + 10) + 1]);
    tl::chain_reset(&ch, heap0);
    for (int seg = 0; seg < 4; seg++) {
      const int i0 = (int)(u01() * 3000), i1 = (int)(u01() * 3000);
      const double x0 = ca[2 * i0], y0 = ca[2 * i0 + 1], x1 = ca[2 * i1], y1 = ca[2 * i1 + 1];
      if (!std::isfinite(x0 + y0 + x1 + y1)) continue;
      for (int p = 0; p <= 300; p++, n_pts++) {
        const double t = p / 300.0;
        const double sx = x0 + (x1 - x0) * t, sy = y0 + (y1 - y0) * t;
        tl::cx im[10];
        double oim[20];
        const int n = tl::chain_images(L, &ch, tl::mk(sx, sy), im, &trig);
        const int on = orc_get_images(o, sx, sy, oim);
        if (n != on) { printf("FAIL image count lens %d seg %d p %d: %d vs %d\n", lens, seg, p, n, on); return 1; }
        for (int k = 0; k < n; k++, n_img++) {
          if (!eqc(im[k], oim + 2 * k)) { printf("FAIL image lens %d seg %d p %d k %d\n", lens, seg, p, k); return 1; }
          // the image's point-source magnification term (lcbase.cc:17-38):
          // the reference squares (img - z_i) with std::pow, which evaluates
          // it in polar form through exp, log, cos and sin (the oracle does
          // the same); the engine multiplies, so the two agree to rounding
          const double ea = tl::image_amp(L, im[k]);
          const double oa = orc_image_amp(o, oim[2 * k], oim[2 * k + 1]);
          // the term's condition number is about the term itself: near the
          // critical curve 1/|1 - |sum|^2| amplifies the last bit of |sum|^2
          const double rel = std::fabs(ea - oa) / std::fmax(std::fabs(oa), 1e-300);
          const double ulps = rel / (2.220446049250313e-16 * std::fmax(1.0, oa));
          if (ulps > amp_rel_max) amp_rel_max = ulps;
        }
      }
    }
    orc_free(o);
  }
  printf("OK %ld %ld %ld %ld %ld %ld %ld %ld %ld %.3e\n", n_poly, n_solve, n_lag, n_pts, n_img,
         n_cc, n_isect, n_hits, n_grid, amp_rel_max);
  return 0;
}
"""

STRICT = ["-O2", "-ffp-contract=off", "-fno-fast-math"]
# point-source magnification terms A_k = 1/|1 - |sum|^2|: a multiplication
# against the reference's std::pow (polar form), so they agree to rounding
# times the term's condition number, which is about A_k itself (up to 1e7 at
# the caustic samples the trajectories start from): relative error <=
# IMAGE_AMP_ULPS * eps * max(1, A_k); 36 is the largest seen
IMAGE_AMP_ULPS = 256.0


def test_engine_math_equals_the_oracle_bit_for_bit(tmp_path):
    gcc, gxx = shutil.which("gcc"), shutil.which("g++")
    if not gcc or not gxx:
        pytest.skip("no gcc/g++")
    objs = []
    for src in ("lcirs_oracle.c", "lens_coeffs.c"):
        obj = tmp_path / (src + ".o")
        r = subprocess.run([gcc, "-std=c11", "-c"] + STRICT +
                           [os.path.join(ROOT, "oracle", src), "-o", str(obj)],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        objs.append(str(obj))
    drv = tmp_path / "math_test.cc"
    drv.write_text(DRIVER)
    exe = tmp_path / "math_test"
    r = subprocess.run([gxx, "-std=c++17"] + STRICT +
                       ["-I", os.path.join(ROOT, "triplelens_gb300", "csrc"), str(drv)] + objs +
                       ["-o", str(exe), "-lm"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("OK"), r.stdout + r.stderr
    f = r.stdout.split()[1:]
    n_poly, n_solve, n_lag, n_pts, n_img, n_cc, n_isect, n_hits, n_grid = map(int, f[:9])
    assert float(f[9]) < IMAGE_AMP_ULPS, f[9]
    assert n_poly == 60 * 40 * 11 and n_solve == 60 * 40 * 16 and n_lag == 60 * 40
    assert n_pts > 60 * 3 * 301 and n_img > 3 * n_pts
    assert n_cc == 60 * 6 * 500 and n_grid == 60 * 200
    assert n_isect == 60 * 400 and 0.1 * n_isect < n_hits < 0.9 * n_isect
