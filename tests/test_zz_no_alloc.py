"""lcirs_fill_device_noalloc (include/lcirs.h) against lcirs_fill_from_seeds.

The entry point serves callers that cannot call cudaMalloc while they compute
magnifications (programs whose device memory belongs to their own pool, and
loops that cannot take cudaFree's device-wide synchronisation): it runs the
fill kernel with a static 80 MiB scratch array instead of allocated tables.
Given the same seed pixels and source positions it must give the same ray
counts (exactly) and magnifications (within the limb-darkening tolerance of
the other GPU tests) as the allocating fill entry point, and on config 1 the
reference's own counts (tests/golden/config1.npz).  Two calls in a row
on different lenses and trajectories check that the shared array's leftovers
from one call do not reach the next; device free memory around the second
call checks that nothing is allocated.

This file is collected last, so a stopping run has already run every other
test when it gets here.
"""
import ctypes

import numpy as np
import pytest

from triplelens_gb300 import workloads

pytestmark = pytest.mark.gpu

LD_RTOL = 1e-6        # limb-darkened magnifications (FP32 per-tile sums)
MAX_POINTS = 8192     # LCIRS_NOALLOC_MAX_POINTS


def _bind(L):
    vp = ctypes.c_void_p
    L.lcirs_fill_device_noalloc.argtypes = [vp, ctypes.c_int, vp, vp, vp, vp, vp, vp, vp]
    L.lcirs_fill_device_noalloc.restype = ctypes.c_int
    return L.lcirs_fill_device_noalloc


def _object(product_lib, lens, n):
    from triplelens_gb300.lcirs import LC_irs
    lc = LC_irs(*lens[:5], lens[5], n, int(lens[7]), lib_path=product_lib)
    lc.set_verbose(0)
    lc.set_limb_darkening("linear", lens[6])
    return lc


def _positions(traj, n):
    # t = i/n as the engine's trajectory sampling (lcirs.cc:117-120)
    x0, y0, x1, y1 = traj
    t = np.arange(n + 1, dtype=np.float64) / float(n)
    return np.stack([x0 + (x1 - x0) * t, y0 + (y1 - y0) * t], axis=1)


def _case(product_lib, lens, traj, n):
    """Object, seeds from its own pipeline, and the allocating fill's output."""
    lc = _object(product_lib, lens, n)
    lc.get_lc_irs(*traj)
    seeds, nseeds = lc.seeds()
    lc.fill_from_seeds(*traj, seeds, nseeds)
    return lc, seeds, nseeds, lc.counts(), lc.lc_full(), lc.status()


def _run_noalloc(fn, lc, xy, seeds, nseeds):
    import torch
    dev = torch.device("cuda", 0)
    np_ = len(xy)
    d_xy = torch.from_numpy(np.ascontiguousarray(xy)).to(dev)
    d_seeds = torch.from_numpy(np.ascontiguousarray(seeds, np.int32)).to(dev)
    d_ns = torch.from_numpy(np.ascontiguousarray(nseeds, np.int32)).to(dev)
    d_mag = torch.full((np_,), -1.0, dtype=torch.float64, device=dev)
    d_cnt = torch.zeros(np_, dtype=torch.int64, device=dev)
    d_st = torch.zeros(np_, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    torch.cuda.synchronize(dev)
    free0 = torch.cuda.mem_get_info(dev)[0]
    r = fn(ctypes.c_void_p(lc.obj), np_, d_xy.data_ptr(), d_seeds.data_ptr(), d_ns.data_ptr(),
           d_mag.data_ptr(), d_cnt.data_ptr(), d_st.data_ptr(), ctypes.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize(dev)
    free1 = torch.cuda.mem_get_info(dev)[0]
    assert r == 0
    return (d_mag.cpu().numpy(), d_cnt.cpu().numpy().view(np.uint64),
            d_st.cpu().numpy().view(np.uint32), free0, free1)


def test_noalloc_matches_fill_from_seeds_twice(product_lib, golden_c1):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from triplelens_gb300.lcirs import load_lcirs
    fn = _bind(load_lcirs(product_lib))

    lens1, traj1, n1 = workloads.config1()
    lens1 = lens1.copy()
    lens1[6] = 0.5
    # includes a caustic-crossing point of magnification 55 (7e6 rays)
    lenses2, trajs2, n2 = workloads.config2(3, n_curves=1, n_points=64, rho=1e-3, ppr=200)
    cases = [(lens1, traj1, n1), (lenses2[0], trajs2[0], n2)]

    for k, (lens, traj, n) in enumerate(cases):
        lc, seeds, nseeds, counts, amps, status = _case(product_lib, lens, traj, n)
        # the allocating fill retries table overflows; the compared points need no retry
        assert int(np.bitwise_or.reduce(status)) & 0x4 == 0
        mag, cnt, st, free0, free1 = _run_noalloc(fn, lc, _positions(traj, n), seeds, nseeds)
        assert np.array_equal(st, status), "call %d: status words differ" % k
        assert np.array_equal(cnt, counts), "call %d: ray counts differ" % k
        if k == 0:
            # config 1: also the reference's own counts (strict IEEE build;
            # the counts do not depend on limb darkening)
            assert np.array_equal(cnt, golden_c1["counts_linear05_strict"])
        assert np.max(np.abs(mag - amps) / amps) < LD_RTOL, "call %d" % k
        if k > 0:
            # the array's address was looked up on the first call: later
            # calls take no device memory
            assert free1 == free0


def test_noalloc_rejects_too_many_points(product_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from triplelens_gb300.lcirs import load_lcirs
    fn = _bind(load_lcirs(product_lib))
    lens, traj, n = workloads.config1()
    lc = _object(product_lib, lens, n)
    dev = torch.device("cuda", 0)
    big = MAX_POINTS + 1
    d_xy = torch.zeros((big, 2), dtype=torch.float64, device=dev)
    d_seeds = torch.zeros((big, 64, 2), dtype=torch.int32, device=dev)
    d_ns = torch.zeros(big, dtype=torch.int32, device=dev)
    d_mag = torch.zeros(big, dtype=torch.float64, device=dev)
    r = fn(ctypes.c_void_p(lc.obj), big, d_xy.data_ptr(), d_seeds.data_ptr(), d_ns.data_ptr(),
           d_mag.data_ptr(), None, None, None)
    assert r == -3
    torch.cuda.synchronize(dev)


def test_noalloc_seed_counts_are_clamped(product_lib):
    """nseeds < 0 fills nothing; nseeds > 64 uses the 64 stored pixels."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from triplelens_gb300.lcirs import load_lcirs
    fn = _bind(load_lcirs(product_lib))
    lens, traj, n = workloads.config1()
    lens = lens.copy()
    lens[6] = 0.5
    lc, seeds, nseeds, counts, amps, status = _case(product_lib, lens, traj, n)
    xy = _positions(traj, n)
    # every slot past a point's count repeats its first seed pixel, so all 64
    # stored pixels seed the same components as the first nseeds
    full = np.array(seeds, dtype=np.int32, copy=True)
    for i, c in enumerate(nseeds):
        if 0 < c < 64:
            full[i, c:] = full[i, 0]
    mag, cnt, st, _, _ = _run_noalloc(fn, lc, xy, full, np.full(len(xy), 100, np.int32))
    has = np.asarray(nseeds) > 0
    assert np.array_equal(cnt[has], counts[has])
    assert np.max(np.abs(mag[has] - amps[has]) / amps[has]) < LD_RTOL
    mag, cnt, st, _, _ = _run_noalloc(fn, lc, xy, full, np.full(len(xy), -1, np.int32))
    assert np.all(cnt == 0) and np.all(mag == 0.0)
    assert np.all(st & 0x4 == 0)


def test_noalloc_table_overflow_sets_status_bit_4(product_lib):
    """A point whose images need more than the static table's blocks comes
    back with status bit 4 and a partial count; every other point is exact."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from triplelens_gb300.lcirs import load_lcirs
    fn = _bind(load_lcirs(product_lib))
    # the caustic crossing of magnification ~55, at 500 rays per radius:
    # ~4e7 rays around its images, more than 16384 blocks of 32 x 32
    lenses, trajs, n = workloads.config2(3, n_curves=1, n_points=64, rho=1e-3, ppr=500)
    lc, seeds, nseeds, counts, amps, status = _case(product_lib, lenses[0], trajs[0], n)
    assert int(np.bitwise_or.reduce(status)) & 0x4 == 0   # the allocating fill retries
    mag, cnt, st, _, _ = _run_noalloc(fn, lc, _positions(trajs[0], n), seeds, nseeds)
    full = (st & 0x4) != 0
    assert full.any(), "no point overflowed: max count %d" % int(counts.max())
    assert np.all(counts[full] > 12288 * 1024 // 2)
    assert np.all(cnt[full] < counts[full])
    ok = ~full
    assert np.array_equal(cnt[ok], counts[ok])
    assert np.array_equal(st[ok], status[ok])
