"""GPU engine (bin/liblcirs.so, through its C ABI) against the oracle and the
reference's golden fixtures.

The pinned reference is the strict IEEE build of the reference's own sources
(oracle/Makefile.ref, liblcirs_ref_strict.so); the oracle reproduces it bit for
bit on every fixture (tests/test_oracle.py).  Parity levels here:
  * exact chain (the default of an lcirs object, and tl_batch with chain 0):
    seed sets and ray counts equal the reference's on every point;
  * parallel chunks (chain k > 0): seed sets and counts equal the oracle run
    with the same chain restarts, on every point;
  * given identical seed pixels, counts are bit-exact (the fill alone).
Magnifications: exact for uniform sources (weights are exactly 1), within
LD_RTOL for limb darkening (the GPU sums weights in FP32 per block and in
fixed point across blocks, the reference in FP64 along its fill order).
"""
import os

import numpy as np
import pytest

from triplelens_gb300 import workloads

pytestmark = pytest.mark.gpu

CHUNK = 4           # tl::kChainChunk, the parallel mode's chain length
# weights are summed in FP32 per 32x8 tile and in 64-bit fixed point across
# tiles; with limb darkening the magnification carries that rounding
LD_RTOL_FP64 = 1e-6
LD_RTOL_SPLIT = 1e-6


def _lc(product_lib, lens, n, precision, chain=0):
    from triplelens_gb300.lcirs import LC_irs
    lc = LC_irs(*lens[:5], lens[5], n, int(lens[7]), lib_path=product_lib)
    lc.set_verbose(0)
    lc.set_precision(precision)
    lc.set_chain(chain)
    if lens[6] >= 0:
        lc.set_limb_darkening("linear", lens[6])
    else:
        lc.set_limb_darkening("default", 0.0)
    return lc


def _oracle(oracle_lib, lens, n, chunk=0):
    o = oracle_lib.OracleIRS(*lens[:5], lens[5], n, int(lens[7]))
    o.set_chain_chunk(chunk)
    if lens[6] >= 0:
        o.set_limb_darkening("linear", lens[6])
    else:
        o.set_limb_darkening("default", 0.0)
    return o


def _seed_sets(seeds, cnt):
    return [set(map(tuple, seeds[i, :cnt[i]].tolist())) for i in range(len(cnt))]


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("v", [0.0, -1.0, 0.5])
def test_config1_full_pipeline(product_lib, oracle_lib, golden_c1, precision, v):
    lens, traj, n = workloads.config1()
    lens = lens.copy()
    lens[6] = v
    lc = _lc(product_lib, lens, n, precision)
    lc.get_lc_irs(*traj)
    assert lc.last_status() & ~0x10 == 0
    counts, amps = lc.counts(), lc.lc_full()
    o = _oracle(oracle_lib, lens, n)
    oseeds, ocnt, fragile = o.lc_seeds(*traj)
    gseeds, gcnt = lc.seeds()
    assert _seed_sets(gseeds, gcnt) == _seed_sets(oseeds, ocnt)
    oamps, ocounts = o.lc_irs(*traj)
    assert np.array_equal(counts, ocounts)
    tag = {0.0: "uniform", -1.0: "default", 0.5: "linear05"}[v]
    assert np.array_equal(counts, golden_c1["counts_%s_strict" % tag])
    if v == 0.0:
        assert np.array_equal(amps, oamps)
    else:
        tol = LD_RTOL_FP64 if precision == 0 else LD_RTOL_SPLIT
        assert np.max(np.abs(amps - oamps) / oamps) < tol
    # copy_lc returns exactly n values
    out = np.full(n + 4, -7.0)
    lc.copy_lc(out)
    assert np.array_equal(out[:n], amps[:n]) and np.all(out[n:] == -7.0)


@pytest.mark.parametrize("precision", [0, 1])
def test_fill_from_oracle_seeds_is_exact(product_lib, oracle_lib, precision):
    lens, traj, n = workloads.config1()
    lens = lens.copy()
    lens[6] = 0.5
    o = oracle_lib.OracleIRS(*lens[:5], lens[5], n, int(lens[7]))
    o.set_limb_darkening("linear", 0.5)
    seeds, cnt, _ = o.lc_seeds(*traj)       # reference chain (no restarts)
    lc = _lc(product_lib, lens, n, precision)
    lc.fill_from_seeds(*traj, seeds.astype(np.int32), cnt)
    counts, amps = lc.counts(), lc.lc_full()
    for p in range(n + 1):
        x = traj[0] + (traj[2] - traj[0]) * (p / n)
        y = traj[1] + (traj[3] - traj[1]) * (p / n)
        a, c = o.fill(x, y, seeds[p, :cnt[p]])
        assert counts[p] == c, p
        tol = LD_RTOL_FP64 if precision == 0 else LD_RTOL_SPLIT
        assert abs(amps[p] - a) <= tol * a, p


def test_fill_from_seeds_clamps_seed_counts(product_lib):
    """lcirs_fill_from_seeds takes seed counts as the caller gives them: a
    negative count fills nothing, a count above 64 uses the 64 stored pixels
    (include/lcirs.h); neither reads past the seed array."""
    lens, traj, n = workloads.config1()
    lens = lens.copy()
    lens[6] = 0.5
    lc = _lc(product_lib, lens, n, 1)
    lc.get_lc_irs(*traj)
    counts = lc.counts()
    seeds, cnt = lc.seeds()
    # slots past a point's count repeat its first seed pixel: all 64 stored
    # pixels seed the same components as the first cnt
    full = np.array(seeds, dtype=np.int32, copy=True)
    for i, c in enumerate(cnt):
        if 0 < c < 64:
            full[i, c:] = full[i, 0]
    lc.fill_from_seeds(*traj, full, np.full(n + 1, 1000, np.int32))
    c_big, a_big = lc.counts(), lc.lc_full()
    lc.fill_from_seeds(*traj, full, np.full(n + 1, 64, np.int32))
    c_64, a_64 = lc.counts(), lc.lc_full()
    assert np.array_equal(c_big, c_64)
    has = np.asarray(cnt) > 0
    assert np.array_equal(c_64[has], counts[has])
    assert np.max(np.abs(a_big[has] - a_64[has]) / a_64[has]) < LD_RTOL_SPLIT
    lc.fill_from_seeds(*traj, full, np.full(n + 1, -1, np.int32))
    assert np.all(lc.counts() == 0) and np.all(lc.lc_full() == 0.0)


def test_amoeba_dump_matches_reference(product_lib, golden_c1, tmp_path):
    lens, traj, n = workloads.config1()
    lens = lens.copy()
    lens[6] = 0.0
    lc = _lc(product_lib, lens, n, 1)
    prefix = str(tmp_path / "amo_")
    lc.set_amoeba_printout(prefix, str(tmp_path / "pars.json"))
    lc.get_lc_irs(*traj)
    for p in golden_c1["amoeba_points"]:
        t = np.loadtxt(prefix + str(p), delimiter=",", dtype=np.int64, ndmin=2).reshape(-1, 3)
        t = t[np.lexsort((t[:, 1], t[:, 0]))]
        assert np.array_equal(t, golden_c1["amoeba_%d" % p]), p
    with open(tmp_path / "pars.json") as f:
        assert f.read() == str(golden_c1["pars_json"])


def _assert_ld_close(amps, ref, tol):
    assert np.max(np.abs(amps - ref) / ref) < tol


@pytest.mark.parametrize("precision", [0, 1])
def test_config2_short_equals_reference(product_lib, oracle_lib, precision):
    """Config-2 lenses (small planets), 3 curves of 201 points, the exact
    chain: seed sets equal the oracle's and ray counts the reference's on
    every point."""
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "config2_short.npz"))
    n = int(z["n"])
    for k in range(len(z["lenses"])):
        L, t = z["lenses"][k], z["trajs"][k]
        lc = _lc(product_lib, L, n, precision)
        lc.get_lc_irs(*t)
        counts = lc.counts()
        o = _oracle(oracle_lib, L, n)
        oseeds, ocnt, _ = o.lc_seeds(*t)
        gseeds, gcnt = lc.seeds()
        assert _seed_sets(gseeds, gcnt) == _seed_sets(oseeds, ocnt), k
        ref = z["counts_%d" % k]
        assert np.array_equal(counts, ref), (k, np.nonzero(counts != ref)[0])
        tol = LD_RTOL_FP64 if precision == 0 else LD_RTOL_SPLIT
        _assert_ld_close(lc.lc_full()[:n], z["amps_%d" % k], tol)


def test_config2_short_chunked_equals_oracle(product_lib, oracle_lib):
    """Parallel chunks of 4 points: seed sets and counts equal the oracle run
    with the same chain restarts; against the reference's single chain they
    differ at a few points only (a count at such a point is the reference's
    with a differently rounded warm start)."""
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "config2_short.npz"))
    n = int(z["n"])
    differ = 0
    for k in range(len(z["lenses"])):
        L, t = z["lenses"][k], z["trajs"][k]
        lc = _lc(product_lib, L, n, 1, chain=CHUNK)
        lc.get_lc_irs(*t)
        o = _oracle(oracle_lib, L, n, chunk=CHUNK)
        oseeds, ocnt, _ = o.lc_seeds(*t)
        gseeds, gcnt = lc.seeds()
        assert _seed_sets(gseeds, gcnt) == _seed_sets(oseeds, ocnt), k
        _, ocounts = o.lc_irs(*t)
        counts = lc.counts()
        assert np.array_equal(counts, ocounts), (k, np.nonzero(counts != ocounts)[0])
        differ += int(np.sum(counts != z["counts_%d" % k]))
    assert differ <= 0.02 * 3 * (n + 1)


def test_config2_full_curve_equals_reference(product_lib, oracle_lib):
    """The 5000-point config-2 curve (seed 0), exact chain: ray counts equal
    the reference's on all 5001 points; relative magnification error of the
    split map within LD_RTOL."""
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "config2_seed0.npz"))
    n = int(z["n"])
    L, t = z["lenses"][0], z["trajs"][0]
    lc = _lc(product_lib, L, n, 1)
    lc.get_lc_irs(*t)
    assert lc.last_status() & ~0x10 == 0
    counts = lc.counts()
    assert np.array_equal(counts, z["counts"]), np.nonzero(counts != z["counts"])[0]
    _assert_ld_close(lc.lc_full()[:n], z["amps"], LD_RTOL_SPLIT)


def test_bench_workload_equals_reference(product_lib):
    """The benchmark's workload (8 config-2 curves of seed 2024, 5001 points
    each) through the batch API with one chain per curve: ray counts equal
    the reference's on all 40008 points, no point incomplete (status bits 4
    and 8 clear)."""
    from triplelens_gb300.batch import Batch
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "bench_seed2024.npz"))
    n = int(z["n"])
    lenses, trajs = z["lenses"], z["trajs"]
    b = Batch(product_lib)
    b.set_chain(0)
    b.set_lenses(lenses)
    amp, cnt, st = b.run(trajs, np.arange(len(trajs)), np.full(len(trajs), n))
    assert int(np.bitwise_or.reduce(st)) & 0xC == 0
    ref = z["counts"].ravel()
    assert np.array_equal(cnt, ref), np.nonzero(cnt != ref)[0][:20]
    for k in range(len(trajs)):
        sl = slice((n + 1) * k, (n + 1) * k + n)
        _assert_ld_close(amp[sl], z["amps"][k], LD_RTOL_SPLIT)


def test_batch_matches_objects(product_lib):
    from triplelens_gb300.batch import Batch
    lenses, trajs, _ = workloads.config2(seed=5, n_curves=4, n_points=60)
    b = Batch(product_lib)
    b.set_chain(0)
    b.set_lenses(lenses)
    amp, cnt, st = b.run(trajs, np.arange(4), np.full(4, 60))
    # point 29 of curve 0 crosses a caustic: ~2e5 tiles, more than the first
    # tile table holds; it completes in the overflow retry
    assert int(np.bitwise_or.reduce(st)) & ~0x10 == 0
    for k in range(4):
        lc = _lc(product_lib, lenses[k], 60, 1)
        lc.get_lc_irs(*trajs[k])
        sl = slice(61 * k, 61 * (k + 1))
        assert np.array_equal(cnt[sl], lc.counts())
        assert np.array_equal(amp[sl], lc.lc_full())


def test_point_source_curve(product_lib, oracle_lib):
    lens, traj, n = workloads.config1()
    lc = _lc(product_lib, lens, n, 1)
    lc.get_lc(*traj)
    out = np.zeros(n)
    lc.copy_lc(out)
    o = _oracle(oracle_lib, lens, n)
    ref = o.lc_point(*traj)
    assert np.max(np.abs(out - ref) / ref) < 1e-9


def test_binary_lens_m3_zero(product_lib, oracle_lib):
    # m3 == 0 selects the two-lens ray map (lcirs.cc:28-36)
    lens = np.array([1.2, 0.9, 1.0, 0.3, 0.0, 0.01, 0.0, 60.0])
    traj = np.array([-1.5, 0.05, 1.5, 0.15])
    n = 40
    lc = _lc(product_lib, lens, n, 1)
    lc.get_lc_irs(*traj)
    o = _oracle(oracle_lib, lens, n)
    _, ocounts = o.lc_irs(*traj)
    assert np.array_equal(lc.counts(), ocounts)
    # and the reference's own counts (strict build, tests/golden/extra_cases.npz)
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "extra_cases.npz"))
    assert np.array_equal(z["lens_binary"], lens) and int(z["n_binary"]) == n
    assert np.array_equal(lc.counts(), z["counts_binary_strict"])


def test_short_and_far_curves(product_lib, oracle_lib):
    # n = 1 (two points) and a source far from the caustics (A close to 1)
    lens = np.array([1.0, 1.0, 1.2, 0.1, 0.05, 0.02, 0.3, 40.0])
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "extra_cases.npz"))
    for traj, n in ((np.array([0.1, 0.2, 0.3, 0.1]), 1), (np.array([1.8, 1.9, 2.1, 1.7]), 5)):
        lc = _lc(product_lib, lens, n, 1)
        lc.get_lc_irs(*traj)
        o = _oracle(oracle_lib, lens, n)
        _, ocounts = o.lc_irs(*traj)
        assert np.array_equal(lc.counts(), ocounts)
        if n == 1:   # the reference's own counts (strict build)
            assert np.array_equal(lc.counts(), z["counts_short_strict"])


def test_bad_input_reports_status(product_lib):
    lens = np.array([1.0, 1.0, 1.2, 0.1, 0.05, 0.02, 0.3, 40.0])
    lc = _lc(product_lib, lens, 3, 1)
    lc.get_lc_irs(float("nan"), 0.0, 0.5, 0.5)
    st = lc.status()
    assert st[0] & 32 and lc.last_status() & 32
    assert lc.counts()[0] == 0


def _caustics(a, b, th, m2, m3):
    import os as _os
    from triplelens_gb300.ccc import CCC
    from triplelens_gb300.lcirs import LIB_DIR
    c = CCC(a, b, th, m2, m3, 500, lib_path=_os.path.join(LIB_DIR, "libccc.so"))
    c.get_ca()
    cc = np.zeros(3000, np.cdouble)
    ca = np.zeros(3000, np.cdouble)
    c.copy_cc_ca(cc, ca)
    return ca.reshape(6, 500)


@pytest.mark.parametrize("precision", [0, 1])
def test_config3_caustic_crossing(product_lib, oracle_lib, precision):
    """Config 3: config-2 lenses resampled until the trajectory crosses a
    caustic; 101 points over a window of +-20 source radii around the first
    crossing.  Seeds and ray counts equal the oracle's (FP64 IRS); the
    split-precision map re-evaluates only a small fraction of the rays in
    FP64; magnification error per point within the LD tolerance."""
    lenses, trajs, _ = workloads.config3(5, _caustics, n_curves=2)
    n = 100
    for k in range(len(lenses)):
        L, t = lenses[k], trajs[k]
        tc = workloads.crossings(t, _caustics(*L[:5]))[0]
        p0, d = t[:2], t[2:] - t[:2]
        w = 20.0 * L[5] / np.hypot(*d)
        win = np.concatenate([p0 + (tc - w) * d, p0 + (tc + w) * d])
        lc = _lc(product_lib, L, n, precision)
        lc.get_lc_irs(*win)
        assert lc.last_status() & 0x2d == 0
        o = _oracle(oracle_lib, L, n)
        oseeds, ocnt, fragile = o.lc_seeds(*win)
        gseeds, gcnt = lc.seeds()
        assert _seed_sets(gseeds, gcnt) == _seed_sets(oseeds, ocnt), k
        oamps, ocounts = o.lc_irs(*win)
        counts = lc.counts()
        assert np.array_equal(counts, ocounts), (k, np.nonzero(counts != ocounts)[0])
        err = np.abs(lc.lc_full() - oamps) / oamps
        assert np.max(err) < (LD_RTOL_FP64 if precision == 0 else LD_RTOL_SPLIT)
        ev, ev64, _ = lc.stats()
        frac64 = float(ev64) / float(ev)
        print("config3 curve %d precision %d: FP64 fraction %.3e, max rel err %.2e, "
              "counts %d..%d" % (k, precision, frac64, err.max(), counts.min(), counts.max()))
        if precision == 1:
            assert frac64 < 1e-2


def test_config4_graph_and_autotune(product_lib):
    """Config 4 (sub-sample: 8 curves x 301 points, each its own lens, rho
    log-uniform in [1e-4, 3e-2], 200/500/1000 rays per radius): the counts
    do not depend on the autotuner's choice of fill stages, and a CUDA-graph replay
    gives the plain run's counts, also after the trajectories are replaced."""
    from triplelens_gb300.batch import Batch
    lenses, trajs, _ = workloads.config4(3, n_curves=8)
    n = 300
    b = Batch(lib_path=product_lib)
    b.set_lenses(lenses)
    idx = np.arange(len(trajs))
    b.set_trajectories(trajs, idx, np.full(len(trajs), n))
    b.run_device(3)
    amp0, cnt0, st0 = b.download()
    assert np.bitwise_or.reduce(st0) & 0x2d == 0
    chosen, times = b.autotune(sample_points=1000)
    assert (chosen[0], chosen[1]) in ((7000, 1), (3000, 1), (1500, 1), (7000, 0), (0, 0))
    assert np.all(times[times >= 0] > 0)
    b.run_device(3)
    amp1, cnt1, _ = b.download()
    assert np.array_equal(cnt1, cnt0)
    assert np.max(np.abs(amp1 - amp0) / amp0) < LD_RTOL_SPLIT
    b.graph_capture()
    b.graph_launch()
    amp2, cnt2, _ = b.download()
    assert np.array_equal(cnt2, cnt0)
    # new trajectories, same counts: replay equals a plain run
    _, trajs2, _ = workloads.config4(4, n_curves=8)
    b.set_trajectories(trajs2, idx, np.full(len(trajs2), n))
    b.graph_launch()
    _, cnt3, _ = b.download()
    b.run_device(3)
    _, cnt4, _ = b.download()
    assert np.array_equal(cnt3, cnt4)


def test_img_abi_matches_reference(product_lib, golden_c1):
    """libimg.so (img_new / get_images / copy_images) against the reference's
    own img_* results for 64 source positions of the config-1 lens: the same
    images (to 1e-9) flagged as images."""
    import os as _os
    from triplelens_gb300.img import Img
    lens = golden_c1["lens"]
    lib = _os.path.join(_os.path.dirname(product_lib), "libimg.so")
    for k, (sx, sy) in enumerate(golden_c1["img_positions"]):
        im = Img(*lens[:5], sx, sy, lib_path=lib)
        im.get_images()
        roots = np.zeros(10, np.cdouble)
        flags = np.zeros(10, np.bool_)
        im.copy_images(roots, flags)
        mine = np.sort_complex(roots[flags])
        ref = np.sort_complex(golden_c1["img_roots"][k][golden_c1["img_isimg"][k]])
        assert len(mine) == len(ref), k
        assert np.max(np.abs(mine - ref)) < 1e-9, k


def test_lccuda_abi_routes_to_the_irs(product_lib):
    """liblccuda.so: LC_cuda's get_lc_cuda gives the IRS curve of get_lc_irs,
    get_lc the point-source curve of get_lc."""
    import os as _os
    from triplelens_gb300.img import LC_cuda
    from triplelens_gb300.lcirs import LC_irs
    lens, traj, n = workloads.config1()
    lib = _os.path.join(_os.path.dirname(product_lib), "liblccuda.so")
    a = LC_cuda(*lens[:5], lens[5], n, int(lens[7]), lib_path=lib)
    a.lib_cuda.lcirs_set_verbose(a.obj, 0)
    a.set_limb_darkening("linear", 0.5)
    a.get_lc_cuda(*traj)
    out_a = np.zeros(n)
    a.copy_lc(out_a)
    b = _lc(product_lib, np.r_[lens[:6], 0.5, lens[7]], n, 1)
    b.get_lc_irs(*traj)
    out_b = np.zeros(n)
    b.copy_lc(out_b)
    assert np.max(np.abs(out_a - out_b) / out_b) < LD_RTOL_SPLIT
    a.get_lc(*traj)
    b.get_lc(*traj)
    a.copy_lc(out_a)
    b.copy_lc(out_b)
    assert np.max(np.abs(out_a - out_b) / np.abs(out_b)) < 1e-12


def test_concurrent_objects_equal_lone_calls(product_lib):
    """get_lc_irs on several objects from several host threads (batched into
    shared launches) leaves every object with the counts and magnifications
    of a lone call, and with the same warm-start state for its next call."""
    from concurrent.futures import ThreadPoolExecutor
    lenses, trajs, _ = workloads.config2(seed=9, n_curves=6, n_points=120)
    n = 120
    lone = []
    for k in range(6):
        lc = _lc(product_lib, lenses[k], n, 1)
        lc.get_lc_irs(*trajs[k])
        lc.get_lc_irs(*trajs[(k + 1) % 6])
        lone.append((lc.counts(), lc.lc_full()))
    objs = [_lc(product_lib, lenses[k], n, 1) for k in range(6)]

    def run(k):
        objs[k].get_lc_irs(*trajs[k])
        objs[k].get_lc_irs(*trajs[(k + 1) % 6])
        return objs[k].counts(), objs[k].lc_full()

    with ThreadPoolExecutor(max_workers=6) as ex:
        got = list(ex.map(run, range(6)))
    for k in range(6):
        assert np.array_equal(got[k][0], lone[k][0]), k
        _assert_ld_close(got[k][1], lone[k][1], LD_RTOL_SPLIT)
