"""ctypes view of the C restatement of TripleLens' LightCurveIRS (the oracle).

Test infrastructure only: tests/, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py`` check and time against it.  The product path never
imports this module.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_ROOT = os.path.dirname(_HERE)
LIB_PATH = os.path.join(_HERE, "build", "liboracle.so")

_lib = None


def build(quiet=True):
    """Compile oracle/lcirs_oracle.c into oracle/build/liboracle.so."""
    cmd = ["make", "-s", "-f", os.path.join("oracle", "Makefile")]
    subprocess.run(cmd, cwd=_ROOT, check=True,
                   stdout=subprocess.DEVNULL if quiet else None)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        d, vp, i64p, dp = ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p
        L.orc_new.argtypes = [d, d, d, d, d, d, ctypes.c_uint, ctypes.c_long]
        L.orc_new.restype = vp
        L.orc_free.argtypes = [vp]
        L.orc_set_limb_darkening.argtypes = [vp, ctypes.c_char_p, d]
        L.orc_grid_params.argtypes = [vp, vp]
        L.orc_copy_cc_ca.argtypes = [vp, dp, dp]
        L.orc_lens.argtypes = [vp, dp, dp]
        L.orc_ld.argtypes = [vp, dp, dp, dp]
        L.orc_get_lc_irs.argtypes = [vp, d, d, d, d, dp, i64p]
        L.orc_lc_seeds.argtypes = [vp, d, d, d, d, ctypes.c_int, i64p, vp, vp]
        L.orc_set_chain_chunk.argtypes = [vp, ctypes.c_int]
        L.orc_set_fragile_band.argtypes = [vp, d]
        L.orc_lc_seeds.restype = ctypes.c_long
        L.orc_fill.argtypes = [vp, d, d, i64p, ctypes.c_int, dp, i64p]
        L.orc_last_amoeba.argtypes = [vp, i64p, ctypes.c_long]
        L.orc_last_amoeba.restype = ctypes.c_long
        L.orc_get_lc.argtypes = [vp, d, d, d, d, dp]
        L.orc_get_images.argtypes = [vp, d, d, dp]
        L.orc_get_images.restype = ctypes.c_int
        L.orc_images_cold.argtypes = [d, d, d, d, d, d, d, dp]
        L.orc_images_cold.restype = ctypes.c_int
        L.orc_irs.argtypes = [vp, d, d, d, d]
        L.orc_irs.restype = d
        L.orc_solve_roots.argtypes = [dp, ctypes.c_int, dp, dp]
        L.orc_laguerre.argtypes = [dp, ctypes.c_int, dp]
        L.orc_laguerre.restype = ctypes.c_int
        L.orc_lens_poly.argtypes = [vp, d, d, dp]
        L.orc_set_trace.argtypes = [vp, dp, ctypes.c_long]
        L.orc_trace_count.argtypes = [vp]
        L.orc_trace_count.restype = ctypes.c_long
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class Grid(ctypes.Structure):
    _fields_ = [("corner_x", ctypes.c_double), ("corner_y", ctypes.c_double),
                ("top_x", ctypes.c_double), ("top_y", ctypes.c_double),
                ("size_double", ctypes.c_double), ("h", ctypes.c_double),
                ("amp_scale", ctypes.c_double), ("n", ctypes.c_int64)]


class OracleIRS:
    """Mirror of the reference's LightCurveIRS object, on the oracle."""

    def __init__(self, a, b, th, m2, m3, rho, lc_len, ppr):
        self.L = lib()
        self.lc_len = int(lc_len)
        self.obj = self.L.orc_new(a, b, th, m2, m3, rho, lc_len, ppr)

    def __del__(self):
        try:
            self.L.orc_free(self.obj)
        except Exception:
            pass

    def set_limb_darkening(self, model, v):
        if isinstance(model, str):
            model = model.encode()
        self.L.orc_set_limb_darkening(self.obj, model, v)

    def grid(self):
        g = Grid()
        self.L.orc_grid_params(self.obj, ctypes.byref(g))
        return g

    def cc_ca(self):
        cc = np.zeros((6, 500, 2))
        ca = np.zeros((6, 500, 2))
        self.L.orc_copy_cc_ca(self.obj, _p(cc), _p(ca))
        return cc, ca

    def lc_irs(self, x0, y0, x1, y1):
        """n+1 magnifications and ray counts (lcirs.cc:117 loops i <= n)."""
        amps = np.zeros(self.lc_len + 1)
        counts = np.zeros(self.lc_len + 1, np.uint64)
        self.L.orc_get_lc_irs(self.obj, x0, y0, x1, y1, _p(amps), _p(counts))
        return amps, counts

    def set_chain_chunk(self, k):
        """Restart the warm-start chain every k points (0: one chain)."""
        self.L.orc_set_chain_chunk(self.obj, int(k))

    def trace_slots(self, cap):
        """Record the value each warm solve starts root 10 from (the heap
        slot the reference reads past the end of its root vector)."""
        self._trace = np.zeros(2 * cap)
        self.L.orc_set_trace(self.obj, _p(self._trace), cap)

    def traced_slots(self):
        n = self.L.orc_trace_count(self.obj)
        return self._trace[0:2 * n:2] + 1j * self._trace[1:2 * n:2]

    def set_fragile_band(self, r):
        self.L.orc_set_fragile_band(self.obj, float(r))

    def lc_seeds(self, x0, y0, x1, y1, max_seeds=64):
        """Seed pixels per point, their number, and the fragile flags."""
        seeds = np.zeros((self.lc_len + 1, max_seeds, 2), np.int64)
        cnt = np.zeros(self.lc_len + 1, np.int32)
        frag = np.zeros(self.lc_len + 1, np.int32)
        self.L.orc_lc_seeds(self.obj, x0, y0, x1, y1, max_seeds, _p(seeds), _p(cnt), _p(frag))
        return seeds, cnt, frag

    def fill(self, sx, sy, seeds):
        seeds = np.ascontiguousarray(seeds, np.int64).reshape(-1, 2)
        amp = ctypes.c_double()
        cnt = ctypes.c_uint64()
        self.L.orc_fill(self.obj, sx, sy, _p(seeds), len(seeds), ctypes.byref(amp),
                        ctypes.byref(cnt))
        return amp.value, cnt.value

    def last_amoeba(self):
        n = self.L.orc_last_amoeba(self.obj, None, 0)
        t = np.zeros((max(n, 1), 3), np.int64)
        self.L.orc_last_amoeba(self.obj, _p(t), n)
        t = t[:n]
        return t[np.lexsort((t[:, 1], t[:, 0]))]

    def lc_point(self, x0, y0, x1, y1):
        out = np.zeros(self.lc_len)
        self.L.orc_get_lc(self.obj, x0, y0, x1, y1, _p(out))
        return out

    def images(self, sx, sy):
        buf = np.zeros(20)
        n = self.L.orc_get_images(self.obj, sx, sy, _p(buf))
        return buf[:2 * n].reshape(n, 2)

    def irs(self, x, y, sx, sy):
        return self.L.orc_irs(self.obj, x, y, sx, sy)

    def lens_poly(self, sx, sy):
        c = np.zeros(22)
        self.L.orc_lens_poly(self.obj, sx, sy, _p(c))
        return c[0::2] + 1j * c[1::2]


def images_cold(a, b, th, m2, m3, sx, sy):
    buf = np.zeros(20)
    n = lib().orc_images_cold(a, b, th, m2, m3, sx, sy, _p(buf))
    return buf[:2 * n].reshape(n, 2)


def solve_roots(coeffs, init=None):
    """Laguerre with deflation (laguerre.cc:103-167); coeffs low->high."""
    c = np.asarray(coeffs, np.complex128)
    deg = len(c) - 1
    cf = np.ascontiguousarray(np.stack([c.real, c.imag], -1).ravel())
    out = np.zeros(2 * deg)
    if init is not None:
        ini = np.asarray(init, np.complex128)
        inf = np.ascontiguousarray(np.stack([ini.real, ini.imag], -1).ravel())
        lib().orc_solve_roots(_p(cf), deg, _p(inf), _p(out))
    else:
        lib().orc_solve_roots(_p(cf), deg, None, _p(out))
    return out[0::2] + 1j * out[1::2]


def laguerre(coeffs, x0):
    c = np.asarray(coeffs, np.complex128)
    cf = np.ascontiguousarray(np.stack([c.real, c.imag], -1).ravel())
    x = np.array([x0.real, x0.imag])
    ok = lib().orc_laguerre(_p(cf), len(c) - 1, _p(x))
    return complex(x[0], x[1]), bool(ok)
