"""ctypes mirror of the reference's ``LC_irs`` class
(Examples/ctypes_classes.py:128-193), bound to this repository's
``bin/liblcirs.so``.  Same method names, argument meaning and behaviour;
a few additive methods expose counts, status and statistics.

There is no CPU path: loading fails loudly when the CUDA library is absent.
"""
import ctypes
import os

import numpy as np
from numpy.ctypeslib import ndpointer

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_DIR = os.path.join(ROOT, "bin")

_libs = {}


def load_lcirs(path=None):
    path = path or os.path.join(LIB_DIR, "liblcirs.so")
    if path in _libs:
        return _libs[path]
    if not os.path.exists(path):
        raise RuntimeError(
            "liblcirs.so not built at %s: run `python -c 'import __graft_entry__ as g; g.build()'`"
            % path)
    L = ctypes.cdll.LoadLibrary(path)
    d, vp = ctypes.c_double, ctypes.c_void_p
    L.lcirs_new.argtypes = [d, d, d, d, d, d, ctypes.c_uint, ctypes.c_long]
    L.lcirs_new.restype = vp
    for name in ("get_lc", "get_lc_irs"):
        getattr(L, name).argtypes = [vp, d, d, d, d]
        getattr(L, name).restype = None
    L.copy_lc.argtypes = [vp, ndpointer(dtype=np.double, flags="C_CONTIGUOUS")]
    L.set_limb_darkening.argtypes = [vp, ctypes.c_char_p, d]
    L.set_amoeba_printout.argtypes = [vp, ctypes.c_char_p, ctypes.c_char_p]
    L.lcirs_delete.argtypes = [vp]
    L.lcirs_last_status.argtypes = [vp]
    L.lcirs_last_status.restype = ctypes.c_uint
    L.lcirs_copy_counts.argtypes = [vp, ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")]
    L.lcirs_copy_lc_full.argtypes = [vp, ndpointer(dtype=np.double, flags="C_CONTIGUOUS")]
    L.lcirs_copy_status.argtypes = [vp, ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")]
    L.lcirs_set_verbose.argtypes = [vp, ctypes.c_int]
    L.lcirs_grid.argtypes = [vp, ndpointer(dtype=np.double, flags="C_CONTIGUOUS")]
    L.lcirs_copy_seeds.argtypes = [vp, ndpointer(dtype=np.int32, flags="C_CONTIGUOUS"),
                                   ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")]
    L.lcirs_fill_from_seeds.argtypes = [vp, d, d, d, d,
                                        ndpointer(dtype=np.int32, flags="C_CONTIGUOUS"),
                                        ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")]
    L.lcirs_copy_stats.argtypes = [vp, ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")]
    L.lcirs_set_precision.argtypes = [vp, ctypes.c_int]
    L.lcirs_set_chain.argtypes = [vp, ctypes.c_int]
    L.lcirs_copy_diag.argtypes = [vp, ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")]
    L.lcirs_copy_transfer_bytes.argtypes = [ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")]
    L.lcirs_copy_transfer_bytes.restype = None
    _libs[path] = L
    return L


def transfer_bytes(lib_path=None):
    """(host -> device, device -> host) bytes the library's own copies have
    moved in this process so far (lcirs_copy_transfer_bytes): what an
    end-to-end run sends across the host boundary, counted by the library."""
    out = np.zeros(2, np.uint64)
    load_lcirs(lib_path).lcirs_copy_transfer_bytes(out)
    return int(out[0]), int(out[1])


MAX_SEEDS = 64


class LC_irs(object):
    """Extended-source light curve of a triple lens (reference LC_irs)."""

    def __init__(self, a, b, th, m2, m3, source_size, lc_len, img_plane_size, lib_path=None):
        self.lib_lc = load_lcirs(lib_path)
        self.lc_len = int(lc_len)
        self.obj = self.lib_lc.lcirs_new(a, b, th, m2, m3, source_size, lc_len, img_plane_size)

    def __del__(self):
        try:
            self.lib_lc.lcirs_delete(self.obj)
        except Exception:
            pass

    # --- reference methods ---
    def get_lc(self, iniX, iniY, finX, finY):
        self.lib_lc.get_lc(self.obj, iniX, iniY, finX, finY)

    def get_lc_irs(self, iniX, iniY, finX, finY):
        self.lib_lc.get_lc_irs(self.obj, iniX, iniY, finX, finY)

    def copy_lc(self, lc_vec):
        # copy_lc writes lc_len values (lcirs.cc:566-576)
        if isinstance(lc_vec, np.ndarray) and lc_vec.size < self.lc_len:
            raise ValueError("copy_lc writes %d values; the array holds %d"
                             % (self.lc_len, lc_vec.size))
        self.lib_lc.copy_lc(self.obj, lc_vec)

    def set_limb_darkening(self, model_type, model_parameter):
        if isinstance(model_type, str):
            model_type = model_type.encode()
        self.lib_lc.set_limb_darkening(self.obj, model_type, model_parameter)

    def set_amoeba_printout(self, amoeba_filename, par_filename):
        if isinstance(amoeba_filename, str):
            amoeba_filename = amoeba_filename.encode()
        if isinstance(par_filename, str):
            par_filename = par_filename.encode()
        self.lib_lc.set_amoeba_printout(self.obj, amoeba_filename, par_filename)

    # --- additive ---
    def set_verbose(self, v):
        self.lib_lc.lcirs_set_verbose(self.obj, int(v))

    def set_precision(self, mode):
        self.lib_lc.lcirs_set_precision(self.obj, int(mode))

    def set_chain(self, points):
        """0: one warm-start chain over the object's life (the reference's,
        exact); k > 0: restart every k points (parallel chunks)."""
        self.lib_lc.lcirs_set_chain(self.obj, int(points))

    def last_status(self):
        return int(self.lib_lc.lcirs_last_status(self.obj))

    def counts(self):
        out = np.zeros(self.lc_len + 1, np.uint64)
        self.lib_lc.lcirs_copy_counts(self.obj, out)
        return out

    def lc_full(self):
        out = np.zeros(self.lc_len + 1)
        self.lib_lc.lcirs_copy_lc_full(self.obj, out)
        return out

    def status(self):
        out = np.zeros(self.lc_len + 1, np.uint32)
        self.lib_lc.lcirs_copy_status(self.obj, out)
        return out

    def grid(self):
        out = np.zeros(8)
        self.lib_lc.lcirs_grid(self.obj, out)
        return out

    def seeds(self):
        s = np.zeros((self.lc_len + 1) * MAX_SEEDS * 2, np.int32)
        n = np.zeros(self.lc_len + 1, np.int32)
        self.lib_lc.lcirs_copy_seeds(self.obj, s, n)
        return s.reshape(self.lc_len + 1, MAX_SEEDS, 2), n

    def fill_from_seeds(self, iniX, iniY, finX, finY, seeds, nseeds):
        """The fill alone from given seed pixels: seeds (n+1, 64, 2) as
        seeds() returns them, nseeds (n+1) counts (clamped to 0..64)."""
        s = np.ascontiguousarray(seeds, np.int32).reshape(-1)
        n = np.ascontiguousarray(nseeds, np.int32).reshape(-1)
        if s.size != (self.lc_len + 1) * MAX_SEEDS * 2 or n.size != self.lc_len + 1:
            raise ValueError("fill_from_seeds: seeds of shape (%d, %d, 2) and %d counts"
                             % (self.lc_len + 1, MAX_SEEDS, self.lc_len + 1))
        self.lib_lc.lcirs_fill_from_seeds(self.obj, iniX, iniY, finX, finY, s, n)

    def diag(self):
        out = np.zeros(self.lc_len + 1, np.uint32)
        self.lib_lc.lcirs_copy_diag(self.obj, out)
        return out

    def stats(self):
        out = np.zeros(3, np.uint64)
        self.lib_lc.lcirs_copy_stats(self.obj, out)
        return out
