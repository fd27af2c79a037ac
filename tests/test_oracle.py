"""The oracle (C restatement, oracle/lcirs_oracle.c) against the reference's
own known answers: the Laguerre tests of tests/laguerretest.cc and golden
fixtures produced by the reference build (tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

from triplelens_gb300 import workloads


def _sorted_real(r):
    return np.array(sorted(r, key=lambda z: z.real))


def _ulps(a, b):
    """Distance in units in the last place (googletest's EXPECT_DOUBLE_EQ
    accepts up to 4)."""
    ia = np.array([a], np.float64).view(np.int64)[0]
    ib = np.array([b], np.float64).view(np.int64)[0]
    if ia < 0:
        ia = -(ia & 0x7FFFFFFFFFFFFFFF)
    if ib < 0:
        ib = -(ib & 0x7FFFFFFFFFFFFFFF)
    return abs(int(ia) - int(ib))


def test_laguerre_second_order(oracle_lib):
    # laguerretest.cc:32-48: x^2 + 2x + 1, both roots have real part -1
    r = oracle_lib.solve_roots([1.0, 2.0, 1.0])
    assert len(r) == 2
    assert _ulps(r[0].real, -1.0) <= 4 and _ulps(r[1].real, -1.0) <= 4
    assert abs(r[0]) < 1.0 + 1e-10 and abs(r[1]) < 1.0 + 1e-10


@pytest.mark.parametrize("coeffs,expected", [
    ([-6.0, 11.0, -6.0, 1.0], [1.0, 2.0, 3.0]),                  # laguerretest.cc:50-83
    ([24.0, -50.0, 35.0, -10.0, 1.0], [1.0, 2.0, 3.0, 4.0]),     # laguerretest.cc:85-118
])
def test_laguerre_real_roots(oracle_lib, coeffs, expected):
    r = _sorted_real(oracle_lib.solve_roots(coeffs))
    assert len(r) == len(expected)
    for got, want in zip(r, expected):
        assert abs(got - want) < 1e-10
        assert abs(got.imag) < 1e-10


def test_laguerre_polish(oracle_lib):
    # laguerretest.cc:121-142, with a seeded perturbation of magnitude 1e-2
    c = [24.0, -50.0, 35.0, -10.0, 1.0]
    rng = np.random.default_rng(3)
    for root in [1.0, 2.0, 3.0, 4.0]:
        for _ in range(8):
            x0 = root + 1e-2 * np.exp(1j * rng.uniform(0, 100))
            x, ok = oracle_lib.laguerre(c, x0)
            assert ok and abs(x - root) < 1e-10


def test_critical_curve_matches_reference(oracle_lib, golden_c1):
    lens, traj, n = workloads.config1()
    o = oracle_lib.OracleIRS(*lens[:5], lens[5], n, int(lens[7]))
    cc, ca = o.cc_ca()
    cc = (cc[..., 0] + 1j * cc[..., 1]).ravel()
    ca = (ca[..., 0] + 1j * ca[..., 1]).ravel()
    # same branch order and samples, to rounding
    assert np.max(np.abs(cc - golden_c1["cc"])) < 1e-12
    assert np.max(np.abs(ca - golden_c1["ca"])) < 1e-12


def test_images_match_reference(oracle_lib, golden_c1):
    lens, _, _ = workloads.config1()
    for (sx, sy), roots, isimg in zip(golden_c1["img_positions"], golden_c1["img_roots"],
                                      golden_c1["img_isimg"]):
        mine = oracle_lib.images_cold(*lens[:5], sx, sy)
        mine = mine[:, 0] + 1j * mine[:, 1]
        ref = roots[isimg]
        assert len(mine) == len(ref)
        for z in ref:
            assert np.min(np.abs(mine - z)) < 1e-9


GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("tag,v", [("uniform", 0.0), ("default", -1.0), ("linear05", 0.5)])
def test_config1_counts_match_reference(oracle_lib, golden_c1, tag, v):
    """Config 1, all 101 points: ray counts and magnifications equal the
    strict reference build's bit for bit (same fill order, same FP64 sums)."""
    lens, traj, n = workloads.config1()
    o = oracle_lib.OracleIRS(*lens[:5], lens[5], n, int(lens[7]))
    if v >= 0:
        o.set_limb_darkening("linear", v)
    else:
        o.set_limb_darkening("default", 0.0)
    amps, counts = o.lc_irs(*traj)
    assert np.array_equal(counts, golden_c1["counts_%s_strict" % tag])
    assert np.array_equal(amps[:n], golden_c1["amps_%s_strict" % tag])


def test_config1_amoeba_sets_match_reference(oracle_lib, golden_c1):
    lens, traj, n = workloads.config1()
    o = oracle_lib.OracleIRS(*lens[:5], lens[5], n, int(lens[7]))
    o.set_limb_darkening("linear", 0.0)
    seeds, cnt, fragile = o.lc_seeds(*traj)
    for p in golden_c1["amoeba_points"]:
        s = seeds[p, :cnt[p]]
        t = traj
        x = t[0] + (t[2] - t[0]) * (p / n)
        y = t[1] + (t[3] - t[1]) * (p / n)
        o.fill(x, y, s)
        mine = o.last_amoeba()
        assert np.array_equal(mine, golden_c1["amoeba_%d" % p])


def test_config2_short_matches_reference(oracle_lib):
    """Config-2 lenses (small planets), 3 curves x 201 points: counts and
    magnifications equal the strict reference build's on every point."""
    z = np.load(os.path.join(GOLDEN, "config2_short.npz"))
    n = int(z["n"])
    for k in range(len(z["lenses"])):
        L = z["lenses"][k]
        o = oracle_lib.OracleIRS(*L[:5], L[5], n, int(L[7]))
        o.set_limb_darkening("linear", L[6])
        amps, counts = o.lc_irs(*z["trajs"][k])
        assert np.array_equal(counts, z["counts_%d" % k]), (k, np.nonzero(counts != z["counts_%d" % k]))
        assert np.array_equal(amps[:n], z["amps_%d" % k]), k


@pytest.mark.parametrize("case", ["binary", "short", "far"])
def test_extra_cases_match_reference(oracle_lib, case):
    """A binary lens (m3 = 0: the two-lens ray map and image count), a
    two-point curve and a curve far from the caustics: counts and
    magnifications equal the strict reference build's on every point."""
    z = np.load(os.path.join(GOLDEN, "extra_cases.npz"))
    L, t, n = z["lens_" + case], z["traj_" + case], int(z["n_" + case])
    o = oracle_lib.OracleIRS(*L[:5], L[5], n, int(L[7]))
    o.set_limb_darkening("linear", L[6])
    amps, counts = o.lc_irs(*t)
    assert np.array_equal(counts, z["counts_%s_strict" % case])
    assert np.array_equal(amps[:n], z["amps_%s_strict" % case])


def test_config4_sample_matches_reference(oracle_lib):
    """Config-4 curves (each its own lens; rho from 3e-4 to 2.3e-2, 200, 500
    and 1000 rays per radius, v from 0.32 to 0.59; up to 3.2e7 rays per point):
    counts and magnifications equal the strict reference build's on every
    point (its -Ofast build differs from it at 7 of 168)."""
    z = np.load(os.path.join(GOLDEN, "config4_sample.npz"))
    n = int(z["n"])
    for k in range(len(z["lenses"])):
        L = z["lenses"][k]
        o = oracle_lib.OracleIRS(*L[:5], L[5], n, int(L[7]))
        o.set_limb_darkening("linear", L[6])
        amps, counts = o.lc_irs(*z["trajs"][k])
        assert np.array_equal(counts, z["counts_strict"][k]), (k, np.nonzero(counts != z["counts_strict"][k]))
        assert np.array_equal(amps[:n], z["amps_strict"][k]), k


def _sampled_counts(oracle_lib, L, t, n, points):
    """Counts at the given points: the whole warm-start chain (every point's
    seeds, in order), then the fill of the sampled points only."""
    o = oracle_lib.OracleIRS(*L[:5], L[5], n, int(L[7]))
    o.set_limb_darkening("linear", L[6])
    seeds, cnt, _ = o.lc_seeds(*t)
    out = []
    for p in points:
        x = t[0] + (t[2] - t[0]) * (p / n)
        y = t[1] + (t[3] - t[1]) * (p / n)
        out.append(o.fill(x, y, seeds[p, :cnt[p]])[1])
    return np.array(out, np.uint64)


def test_config2_seed0_matches_reference(oracle_lib):
    """The 5000-point curve: every point's seeds through the single chain;
    counts at every 25th point and at every point where the reference's
    -Ofast builds disagree with its strict build equal the strict build's."""
    z = np.load(os.path.join(GOLDEN, "config2_seed0.npz"))
    n = int(z["n"])
    ref = z["counts"]
    spread = np.nonzero((z["counts_nfc"] != ref) | (z["counts_fast"] != ref))[0]
    pts = np.union1d(np.arange(0, n + 1, 25), spread)
    got = _sampled_counts(oracle_lib, z["lenses"][0], z["trajs"][0], n, pts)
    assert np.array_equal(got, ref[pts]), pts[got != ref[pts]]


def test_bench_workload_matches_reference(oracle_lib):
    """The benchmark's 8 curves (seed 2024): counts at every 125th point of
    each curve equal the strict reference build's."""
    z = np.load(os.path.join(GOLDEN, "bench_seed2024.npz"))
    n = int(z["n"])
    pts = np.arange(0, n + 1, 125)
    for k in range(len(z["lenses"])):
        got = _sampled_counts(oracle_lib, z["lenses"][k], z["trajs"][k], n, pts)
        assert np.array_equal(got, z["counts"][k][pts]), (k, pts[got != z["counts"][k][pts]])


def test_reference_build_spread():
    """The reference's -Ofast builds (FMA contraction off/on) re-associate its
    coefficient expressions at the compiler's discretion: their counts leave
    the strict build's at points where an image next to a small-mass lens
    sits at the 1e-6 filter radius, by a few rays each."""
    z = np.load(os.path.join(GOLDEN, "config2_short.npz"))
    for k in range(len(z["lenses"])):
        a = z["counts_%d" % k].astype(np.int64)
        for key in ("counts_nfc_%d", "counts_fast_%d"):
            b = z[key % k].astype(np.int64)
            assert np.max(np.abs(a - b)) <= 64
    s0 = np.load(os.path.join(GOLDEN, "config2_seed0.npz"))
    for key in ("counts_nfc", "counts_fast"):
        assert np.mean(s0[key] != s0["counts"]) < 0.03


def test_point_source_curves_match_reference(oracle_lib):
    """Point-source curves (get_lc, lcbase.cc:40-52) against the reference
    built as strict IEEE (tests/golden/point_lc.npz): the config-1
    lens to 1e-9; config-2 lenses, whose small-mass lenses make single image
    magnifications rounding-sensitive, to 1e-4 (the reference's own -Ofast
    build differs from that build by up to 45 % at single points)."""
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "point_lc.npz"))
    for k in range(int(z["cases"])):
        L, t, ref = z["lens_%d" % k], z["traj_%d" % k], z["amps_%d" % k]
        o = oracle_lib.OracleIRS(*L[:5], L[5], len(ref), int(L[7]))
        o.set_chain_chunk(0)
        rel = np.abs(o.lc_point(*t) - ref) / ref
        assert rel.max() < (1e-9 if k == 0 else 1e-4), (k, rel.max())
