"""ctypes mirror of the reference's ``CCC`` class
(Examples/ctypes_classes.py:13-75), bound to this repository's
``bin/libccc.so`` (critical curves and caustics on the GPU).  Same method
names and argument meaning."""
import ctypes
import os

import numpy as np
from numpy.ctypeslib import ndpointer

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def load_ccc(path=None):
    path = path or os.path.join(ROOT, "bin", "libccc.so")
    if not os.path.exists(path):
        raise RuntimeError("libccc.so not built at %s: run `python -c 'import __graft_entry__ as "
                           "g; g.build()'`" % path)
    L = ctypes.cdll.LoadLibrary(path)
    d, vp = ctypes.c_double, ctypes.c_void_p
    cplx = ndpointer(dtype=np.cdouble, flags="C_CONTIGUOUS")
    L.ccc_new.argtypes = [d] * 5 + [ctypes.c_int]
    L.ccc_new.restype = vp
    L.get_cc.argtypes = [vp]
    L.get_ca.argtypes = [vp]
    L.print_ccc.argtypes = [vp, ctypes.c_char_p]
    L.copy_cc_ca.argtypes = [vp, cplx, cplx]
    L.copy_lenses.argtypes = [vp, cplx]
    L.get_bounding_box.argtypes = [vp, cplx, cplx, cplx, cplx, d]
    L.ccc_delete.argtypes = [vp]
    return L


class CCC(object):
    def __init__(self, a, b, th, m2, m3, length, lib_path=None):
        self.lib_ccc = load_ccc(lib_path)
        self.obj = self.lib_ccc.ccc_new(a, b, th, m2, m3, length)

    def __del__(self):
        try:
            self.lib_ccc.ccc_delete(self.obj)
        except Exception:
            pass

    def get_cc(self):
        self.lib_ccc.get_cc(self.obj)

    def get_ca(self):
        self.lib_ccc.get_ca(self.obj)

    def print_ccc(self, file_name):
        if isinstance(file_name, str):
            file_name = file_name.encode()
        self.lib_ccc.print_ccc(self.obj, file_name)

    def copy_cc_ca(self, ccp, cap):
        self.lib_ccc.copy_cc_ca(self.obj, ccp, cap)

    def copy_lenses(self, lens_pos):
        self.lib_ccc.copy_lenses(self.obj, lens_pos)

    def get_bounding_box(self, cc_min, cc_max, ca_min, ca_max, scale):
        self.lib_ccc.get_bounding_box(self.obj, cc_min, cc_max, ca_min, ca_max, scale)
