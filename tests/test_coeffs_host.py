"""The image polynomial's coefficients as the engine computes them
(triplelens_gb300/csrc/tl_coeffs.h, the header the GPU prep and chain
kernels include) against the oracle's (oracle/lens_coeffs.c), bit for bit,
without a GPU.

Both restate the reference's ImgPoint::getCoeffsOptNoZ and getCoeffsOptJustZ
(src/Images/imgpointcoeff.cc:223-447) in its evaluation order, the engine
with its own complex type and the oracle with C99 complex arithmetic; the
oracle is pinned to the reference's strict build by the fixture tests.  Here
both are compiled for the host with the engine's rounding rules (no FMA
contraction, no fast math) and compared on random lenses and source
positions, including binary lenses (m3 = 0) and sources near the lenses.
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
#include "tl_math.h"   // defines the complex operations, then includes tl_coeffs.h

extern "C" void orc_coeffs_nozeta(double m2, double m3, const double* z2, const double* z3,
                                  double* out22);
extern "C" void orc_coeffs_zeta(double m2, double m3, const double* z2, const double* z3,
                                double zx, double zy, double* out22);

static unsigned long long s = 0x9e3779b97f4a7c15ull;
static double u01() {
  s ^= s << 13; s ^= s >> 7; s ^= s << 17;
  return (double)(s >> 11) * (1.0 / 9007199254740992.0);
}

static bool same(const tl::cx* a, const double* b, int k) {
  return std::memcmp(&a[k].re, &b[2 * k], 8) == 0 && std::memcmp(&a[k].im, &b[2 * k + 1], 8) == 0;
}

int main() {
  long compared = 0;
  for (int lens = 0; lens < 2000; lens++) {
    // masses from ratios log-uniform in [1e-3, 1]; separations in [0.5, 2]
    const double q2 = std::pow(10.0, -3.0 * u01());
    const double q3 = lens % 10 == 0 ? 0.0 : std::pow(10.0, -3.0 * u01());
    const double m2 = q2 / (1.0 + q2 + q3), m3 = q3 / (1.0 + q2 + q3);
    const double a = 0.5 * std::pow(4.0, u01()), b = 0.5 * std::pow(4.0, u01());
    const double th = 6.283185307179586 * u01();
    const double z2[2] = {a, 0.0}, z3[2] = {b * std::cos(th), b * std::sin(th)};
    tl::cx c0[11], cz[11];
    double o0[22], oz[22];
    tl::coeffs_nozeta(m2, m3, tl::mk(z2[0], z2[1]), tl::mk(z3[0], z3[1]), c0);
    orc_coeffs_nozeta(m2, m3, z2, z3, o0);
    for (int k = 0; k < 11; k++, compared++)
      if (!same(c0, o0, k)) {
        printf("FAIL nozeta lens %d k %d: %.17g %.17g vs %.17g %.17g\n", lens, k, c0[k].re,
               c0[k].im, o0[2 * k], o0[2 * k + 1]);
        return 1;
      }
    for (int p = 0; p < 50; p++) {
      double zx, zy;
      if (p % 5 == 0) {   // next to a lens
        const double* zl = p % 2 ? z2 : z3;
        zx = zl[0] + 1e-3 * (u01() - 0.5);
        zy = zl[1] + 1e-3 * (u01() - 0.5);
      } else {
        zx = 4.0 * (u01() - 0.5);
        zy = 4.0 * (u01() - 0.5);
      }
      tl::coeffs_zeta(m2, m3, tl::mk(z2[0], z2[1]), tl::mk(z3[0], z3[1]), tl::mk(zx, zy), cz);
      orc_coeffs_zeta(m2, m3, z2, z3, zx, zy, oz);
      for (int k = 0; k < 11; k++, compared++)
        if (!same(cz, oz, k)) {
          printf("FAIL zeta lens %d point %d k %d: %.17g %.17g vs %.17g %.17g\n", lens, p, k,
                 cz[k].re, cz[k].im, oz[2 * k], oz[2 * k + 1]);
          return 1;
        }
    }
  }
  printf("OK %ld\n", compared);
  return 0;
}
"""

STRICT = ["-O2", "-ffp-contract=off", "-fno-fast-math"]


def test_engine_coefficients_equal_the_oracle_bit_for_bit(tmp_path):
    gcc, gxx = shutil.which("gcc"), shutil.which("g++")
    if not gcc or not gxx:
        pytest.skip("no gcc/g++")
    obj = tmp_path / "lens_coeffs.o"
    r = subprocess.run([gcc, "-std=c11", "-c"] + STRICT +
                       [os.path.join(ROOT, "oracle", "lens_coeffs.c"), "-o", str(obj)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    src = tmp_path / "coeffs_test.cc"
    src.write_text(DRIVER)
    exe = tmp_path / "coeffs_test"
    r = subprocess.run([gxx, "-std=c++17"] + STRICT +
                       ["-I", os.path.join(ROOT, "triplelens_gb300", "csrc"), str(src), str(obj),
                        "-o", str(exe), "-lm"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.startswith("OK"), r.stdout + r.stderr
    assert int(r.stdout.split()[1]) == 2000 * 11 * 51
