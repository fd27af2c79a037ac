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
        lenses = np.ascontiguousarray(lenses, np.float64)
        r = self.L.tlb_set_lenses(self.obj, len(lenses), lenses.ravel())
        if r < 0:
            raise RuntimeError("tlb_set_lenses failed: %d" % r)

    def set_trajectories(self, trajs, lens_idx, n):
        trajs = np.ascontiguousarray(trajs, np.float64)
        li = np.ascontiguousarray(lens_idx, np.int32)
        nn = np.ascontiguousarray(n, np.uint32)
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
        trajs = np.ascontiguousarray(trajs, np.float64)
        r = self.L.tlb_run_host(self.obj, len(trajs), trajs.ravel(),
                                np.ascontiguousarray(lens_idx, np.int32),
                                np.ascontiguousarray(n, np.uint32), _ptr(amp), _ptr(cnt),
                                _ptr(st), stream)
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
