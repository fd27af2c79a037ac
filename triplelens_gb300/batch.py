"""ctypes view of the batched entry points (include/tl_batch.h): many lenses
and trajectories in one seeds launch and one persistent fill launch."""
import ctypes

import numpy as np
from numpy.ctypeslib import ndpointer

from .lcirs import load_lcirs

_bound = set()


def _bind(L):
    if id(L) in _bound:
        return L
    vp, d = ctypes.c_void_p, ctypes.c_double
    f64 = ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
    L.tlb_new.restype = vp
    L.tlb_new.argtypes = []
    L.tlb_delete.argtypes = [vp]
    L.tlb_set_lenses.argtypes = [vp, ctypes.c_int, f64]
    L.tlb_set_lenses.restype = ctypes.c_int
    L.tlb_set_trajectories.argtypes = [vp, ctypes.c_int, f64,
                                       ndpointer(dtype=np.int32, flags="C_CONTIGUOUS"),
                                       ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")]
    L.tlb_set_trajectories.restype = ctypes.c_long
    L.tlb_run_device.argtypes = [vp, ctypes.c_int, vp]
    L.tlb_run_device.restype = ctypes.c_int
    L.tlb_download.argtypes = [vp, vp, vp, vp, vp]
    L.tlb_download.restype = ctypes.c_int
    L.tlb_run_host.argtypes = [vp, ctypes.c_int, f64,
                               ndpointer(dtype=np.int32, flags="C_CONTIGUOUS"),
                               ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS"), vp, vp, vp, vp]
    L.tlb_run_host.restype = ctypes.c_long
    L.tlb_stats.argtypes = [vp, ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")]
    L.tlb_stats.restype = ctypes.c_int
    L.tlb_configure.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                ctypes.c_int]
    L.tlb_configure.restype = ctypes.c_int
    L.tlb_set_chain.argtypes = [vp, ctypes.c_int]
    L.tlb_set_chain.restype = ctypes.c_int
    L.tlb_point_lc.argtypes = [vp, f64]
    L.tlb_point_lc.restype = ctypes.c_long
    L.tlb_set_fill_stages.argtypes = [vp, ctypes.c_int, ctypes.c_int]
    L.tlb_set_fill_stages.restype = ctypes.c_int
    L.tlb_autotune.argtypes = [vp, ctypes.c_long, ndpointer(dtype=np.int32, flags="C_CONTIGUOUS"),
                               ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")]
    L.tlb_autotune.restype = ctypes.c_int
    L.tlb_graph_capture.argtypes = [vp]
    L.tlb_graph_capture.restype = ctypes.c_int
    L.tlb_graph_launch.argtypes = [vp, vp]
    L.tlb_graph_launch.restype = ctypes.c_int
    _bound.add(id(L))
    return L


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


# The C functions read and write as many rows as the counts they are given:
# the shapes are checked here, before any pointer crosses the boundary.
def _lens_rows(lenses):
    """Lenses as a contiguous (k, 8) float64 array (one row is one lens)."""
    a = np.ascontiguousarray(np.atleast_2d(np.asarray(lenses, np.float64)))
    if a.ndim != 2 or a.shape[1] != 8 or a.shape[0] == 0:
        raise ValueError("lenses: rows of 8 values (a, b, th, m2, m3, rho, ld_v, ppr), "
                         "got shape %s" % (a.shape,))
    bad = ~np.all(np.isfinite(a), axis=1) | ~(a[:, 5] > 0) | ~(a[:, 7] >= 1) | \
        ~(a[:, 7] <= 2 ** 31 - 1)
    if np.any(bad):
        raise ValueError("lenses: rows %s have non-finite values, rho <= 0 or rays per "
                         "radius outside 1..2^31-1" % np.nonzero(bad)[0][:10].tolist())
    return a


def _traj_args(trajs, lens_idx, n):
    """Trajectories as a contiguous (k, 4) float64 array, with the lens index
    and the point count of each curve (a scalar applies to every curve)."""
    t = np.ascontiguousarray(np.atleast_2d(np.asarray(trajs, np.float64)))
    if t.ndim != 2 or t.shape[1] != 4 or t.shape[0] == 0:
        raise ValueError("trajs: rows of 4 values (x0, y0, x1, y1), got shape %s" % (t.shape,))
    k = t.shape[0]
    try:
        li = np.broadcast_to(np.asarray(lens_idx), (k,))
        nn = np.broadcast_to(np.asarray(n), (k,))
    except ValueError:
        raise ValueError("lens_idx and n: one value per curve (%d) or one for all" % k)
    if np.any(nn < 0) or np.any(nn >= 2 ** 31):
        raise ValueError("n: point counts in [0, 2^31)")
    return t, np.ascontiguousarray(li, np.int32), np.ascontiguousarray(nn, np.uint32)


def _check_out(name, arr, dtype, points):
    """An output array the C side writes `points` entries of (None: skipped)."""
    if arr is None:
        return
    if not isinstance(arr, np.ndarray) or arr.dtype != dtype or not arr.flags.c_contiguous \
            or not arr.flags.writeable or arr.size < points:
        raise ValueError("%s: a writable contiguous %s array of at least %d entries"
                         % (name, np.dtype(dtype).name, points))


class Batch:
    """Lenses (rows a, b, th, m2, m3, rho, ld_v, ppr) and trajectories
    (rows x0, y0, x1, y1) on the GPU engine."""

    def __init__(self, lib_path=None):
        self.L = _bind(load_lcirs(lib_path))
        self.obj = self.L.tlb_new()
        self.npoints = 0

    def __del__(self):
        try:
            self.L.tlb_delete(self.obj)
        except Exception:
            pass

    def configure(self, precision=-1, fill_ctas=0, table_log2=0, threads=0, block_h=0):
        return self.L.tlb_configure(self.obj, precision, fill_ctas, table_log2, threads, block_h)

    def set_chain(self, points):
        """Warm-start chain length: > 0 restarts every `points` points
        (parallel, default 4); <= 0 one chain per curve (the reference's
        order, exact).  Applies from the next set_trajectories."""
        return self.L.tlb_set_chain(self.obj, int(points))

    def set_lenses(self, lenses):
        lenses = _lens_rows(lenses)
        r = self.L.tlb_set_lenses(self.obj, len(lenses), lenses.ravel())
        if r < 0:
            raise RuntimeError("tlb_set_lenses failed: %d" % r)

    def set_trajectories(self, trajs, lens_idx, n):
        trajs, li, nn = _traj_args(trajs, lens_idx, n)
        r = self.L.tlb_set_trajectories(self.obj, len(trajs), trajs.ravel(), li, nn)
        if r < 0:
            raise RuntimeError("tlb_set_trajectories failed: %d" % r)
        self.npoints = int(r)
        return self.npoints

    def run_device(self, phase=3, stream=None):
        r = self.L.tlb_run_device(self.obj, phase, stream)
        if r < 0:
            raise RuntimeError("tlb_run_device failed: %d" % r)

    def download(self, stream=None):
        amp = np.zeros(self.npoints)
        cnt = np.zeros(self.npoints, np.uint64)
        st = np.zeros(self.npoints, np.uint32)
        r = self.L.tlb_download(self.obj, _ptr(amp), _ptr(cnt), _ptr(st), stream)
        if r < 0:
            raise RuntimeError("tlb_download failed: %d" % r)
        return amp, cnt, st

    def run(self, trajs, lens_idx, n):
        self.set_trajectories(trajs, lens_idx, n)
        self.run_device(3)
        return self.download()

    def run_host(self, trajs, lens_idx, n, amp, cnt, st, stream=None):
        trajs, li, nn = _traj_args(trajs, lens_idx, n)
        points = int(np.sum(nn.astype(np.int64) + 1))
        _check_out("amp", amp, np.float64, points)
        _check_out("cnt", cnt, np.uint64, points)
        _check_out("st", st, np.uint32, points)
        r = self.L.tlb_run_host(self.obj, len(trajs), trajs.ravel(), li, nn, _ptr(amp),
                                _ptr(cnt), _ptr(st), stream)
        if r < 0:
            raise RuntimeError("tlb_run_host failed: %d" % r)
        self.npoints = int(r)
        return self.npoints

    def stats(self):
        out = np.zeros(4, np.uint64)
        self.L.tlb_stats(self.obj, out)
        return out

    def autotune(self, sample_points=0):
        """Fastest sharing of the points among the fill's stages, timed on a
        prefix of the current points: (warp-fill threshold in blocks, 0 for
        the CTA fill alone; 1 if the team fill takes the larger points;
        points timed), and the 5 timings (ms), in the order of
        include/tl_batch.h."""
        chosen = np.zeros(3, np.int32)
        times = np.zeros(5, np.float32)
        r = self.L.tlb_autotune(self.obj, sample_points, chosen, times)
        if r < 0:
            raise RuntimeError("tlb_autotune failed: %d" % r)
        return tuple(int(x) for x in chosen), times

    def set_fill_stages(self, warp_threshold_blocks, team):
        """Reapplies a choice of tlb_autotune (see save_tuning/load_tuning)."""
        r = self.L.tlb_set_fill_stages(self.obj, int(warp_threshold_blocks), int(team))
        if r < 0:
            raise RuntimeError("tlb_set_fill_stages failed: %d" % r)

    def graph_capture(self):
        r = self.L.tlb_graph_capture(self.obj)
        if r < 0:
            raise RuntimeError("tlb_graph_capture failed: %d" % r)

    def graph_launch(self, stream=None):
        r = self.L.tlb_graph_launch(self.obj, stream)
        if r < 0:
            raise RuntimeError("tlb_graph_launch failed: %d" % r)

    def point_lc(self):
        amp = np.zeros(self.npoints)
        r = self.L.tlb_point_lc(self.obj, amp)
        if r < 0:
            raise RuntimeError("tlb_point_lc failed: %d" % r)
        return amp


# The autotuner's choice as JSON, so that a later process can apply it without
# timing again (Batch.set_fill_stages).
CANDIDATES = ("warp<=7000+team", "warp<=3000+team", "warp<=1500+team", "warp<=7000+cta", "cta")


def save_tuning(path, chosen, times_ms=None, meta=None):
    """Writes (warp-fill threshold, team, points timed) of Batch.autotune and
    its candidate timings to a JSON file."""
    import json
    thr, team, points = (int(x) for x in chosen)
    if thr < 0:
        raise ValueError("warp-fill threshold must be >= 0")
    out = {"warp_fill_threshold_blocks": thr, "team_fill": bool(team), "points_timed": points}
    if times_ms is not None:
        out["candidates_ms"] = {k: float(t) for k, t in zip(CANDIDATES, times_ms)}
    if meta:
        out["meta"] = meta
    with open(path, "w") as f:
        json.dump(out, f, indent=1)


def load_tuning(path):
    """(warp-fill threshold, team) from save_tuning's file."""
    import json
    with open(path) as f:
        d = json.load(f)
    thr = int(d["warp_fill_threshold_blocks"])
    if thr < 0:
        raise ValueError("%s: negative warp-fill threshold" % path)
    return thr, bool(d["team_fill"])
