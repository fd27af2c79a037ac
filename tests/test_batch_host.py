"""The Python wrappers of the batched API (triplelens_gb300/batch.py) and of
the reference's class (triplelens_gb300/lcirs.py) check the shapes of what
they hand to the C functions, which read and write as many rows as the
counts they are given: wrong shapes raise ValueError before any pointer
crosses the boundary.  No GPU: module functions, and an LC_irs around a
stand-in library."""
import numpy as np
import pytest

from triplelens_gb300 import batch as B


def test_lens_rows():
    one = [1.0, 0.9, 1.0, 0.3, 0.0, 0.01, 0.0, 60.0]
    a = B._lens_rows(one)                       # one lens as one row
    assert a.shape == (1, 8) and a.dtype == np.float64 and a.flags.c_contiguous
    a = B._lens_rows(np.tile(one, (3, 1)).T.copy().T)   # non-contiguous input
    assert a.shape == (3, 8) and a.flags.c_contiguous
    for bad in ([1.0, 2.0], np.zeros((2, 7)), np.zeros((0, 8)), np.zeros((2, 8, 1))):
        with pytest.raises(ValueError):
            B._lens_rows(bad)
    # rows the lens set-up cannot use
    for k, v in ((5, 0.0), (5, -1e-3), (5, np.nan), (7, 0.0), (0, np.inf), (3, np.nan)):
        row = np.array(one)
        row[k] = v
        with pytest.raises(ValueError):
            B._lens_rows(np.stack([np.array(one), row]))


def test_traj_args_broadcast_and_check():
    t, li, nn = B._traj_args([0.0, 0.1, 1.0, 0.2], 0, 100)
    assert t.shape == (1, 4) and li.tolist() == [0] and nn.tolist() == [100]
    trajs = np.zeros((3, 4))
    t, li, nn = B._traj_args(trajs, [0, 1, 2], 50)
    assert li.dtype == np.int32 and nn.dtype == np.uint32 and nn.tolist() == [50, 50, 50]
    assert li.flags.c_contiguous and nn.flags.c_contiguous
    t, li, nn = B._traj_args(trajs, 0, [1, 2, 3])
    assert li.tolist() == [0, 0, 0] and nn.tolist() == [1, 2, 3]
    with pytest.raises(ValueError):
        B._traj_args(np.zeros((3, 3)), 0, 10)        # not 4 values per row
    with pytest.raises(ValueError):
        B._traj_args(trajs, [0, 1], 10)              # 2 lens indices for 3 curves
    with pytest.raises(ValueError):
        B._traj_args(trajs, 0, [10, 20])             # 2 counts for 3 curves
    with pytest.raises(ValueError):
        B._traj_args(trajs, 0, -1)                   # negative count
    with pytest.raises(ValueError):
        B._traj_args(np.zeros((0, 4)), 0, 1)


def test_output_arrays_are_checked():
    B._check_out("amp", None, np.float64, 10)    # skipped output
    B._check_out("amp", np.zeros(12), np.float64, 10)
    for bad in (np.zeros(9), np.zeros(10, np.float32), np.zeros((10, 2))[:, 0], [0.0] * 10):
        with pytest.raises(ValueError):
            B._check_out("amp", bad, np.float64, 10)
    ro = np.zeros(10)
    ro.flags.writeable = False
    with pytest.raises(ValueError):
        B._check_out("amp", ro, np.float64, 10)
    B._check_out("cnt", np.zeros(10, np.uint64), np.uint64, 10)
    with pytest.raises(ValueError):
        B._check_out("cnt", np.zeros(10, np.int64), np.uint64, 10)


class _FakeLib:
    """Stands in for liblcirs.so: records the calls that reach it."""

    def __init__(self):
        self.calls = []

    def __getattr__(self, name):
        def call(*args):
            self.calls.append(name)
        return call


def _lc_without_gpu(n):
    from triplelens_gb300.lcirs import LC_irs
    lc = object.__new__(LC_irs)
    lc.lib_lc, lc.lc_len, lc.obj = _FakeLib(), n, None
    return lc


def test_lc_irs_checks_sizes_before_the_c_calls():
    """LC_irs.copy_lc writes n values and fill_from_seeds reads (n+1) x 64 x 2
    seeds and n+1 counts (include/lcirs.h): shorter or misshapen arrays raise
    ValueError and never reach the library."""
    from triplelens_gb300.lcirs import MAX_SEEDS
    lc = _lc_without_gpu(10)
    lc.copy_lc(np.zeros(10))
    with pytest.raises(ValueError):
        lc.copy_lc(np.zeros(9))
    seeds = np.zeros((11, MAX_SEEDS, 2), np.int32)
    lc.fill_from_seeds(0.0, 0.0, 1.0, 1.0, seeds, np.zeros(11, np.int32))
    with pytest.raises(ValueError):
        lc.fill_from_seeds(0.0, 0.0, 1.0, 1.0, seeds[:10], np.zeros(11, np.int32))
    with pytest.raises(ValueError):
        lc.fill_from_seeds(0.0, 0.0, 1.0, 1.0, seeds, np.zeros(10, np.int32))
    assert lc.lib_lc.calls == ["copy_lc", "lcirs_fill_from_seeds"]


def test_tuning_json_round_trip(tmp_path):
    """The autotuner's choice saved as JSON (batch.save_tuning) comes back
    as (warp-fill threshold, team) for Batch.set_fill_stages."""
    path = tmp_path / "tuning.json"
    B.save_tuning(path, (3000, 1, 32768), [420.0, 401.5, 430.0, 431.0, 457.0], {"gpu": "x"})
    assert B.load_tuning(path) == (3000, True)
    import json
    d = json.loads(path.read_text())
    assert d["candidates_ms"]["warp<=3000+team"] == 401.5 and d["points_timed"] == 32768
    B.save_tuning(path, (0, 0, 10))
    assert B.load_tuning(path) == (0, False)
    with pytest.raises(ValueError):
        B.save_tuning(path, (-1, 0, 10))
