"""ctypes mirrors of the reference's ``Img`` and ``LC_cuda`` classes
(Examples/ctypes_classes.py:78-125, 196-270), bound to this repository's
``bin/libimg.so`` and ``bin/liblccuda.so``.  Same method names and argument
meaning."""
import ctypes
import os

import numpy as np
from numpy.ctypeslib import ndpointer

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _load(name, path=None):
    path = path or os.path.join(ROOT, "bin", name)
    if not os.path.exists(path):
        raise RuntimeError("%s not built at %s: run `python -c 'import __graft_entry__ as g; "
                           "g.build()'`" % (name, path))
    return ctypes.cdll.LoadLibrary(path)


class Img(object):
    def __init__(self, a, b, th, m2, m3, pos_x, pos_y, lib_path=None):
        L = self.lib_img = _load("libimg.so", lib_path)
        d, vp = ctypes.c_double, ctypes.c_void_p
        L.img_new.argtypes = [d] * 7
        L.img_new.restype = vp
        L.get_roots.argtypes = [vp]
        L.get_images.argtypes = [vp]
        L.set_pos.argtypes = [vp, d, d]
        L.copy_images.argtypes = [vp, ndpointer(dtype=np.cdouble, flags="C_CONTIGUOUS"),
                                  ndpointer(dtype=np.bool_, flags="C_CONTIGUOUS")]
        L.img_delete.argtypes = [vp]
        self.obj = L.img_new(a, b, th, m2, m3, pos_x, pos_y)

    def __del__(self):
        try:
            self.lib_img.img_delete(self.obj)
        except Exception:
            pass

    def get_roots(self):
        self.lib_img.get_roots(self.obj)

    def get_images(self):
        self.lib_img.get_images(self.obj)

    def set_pos(self, pos_x, pos_y):
        self.lib_img.set_pos(self.obj, pos_x, pos_y)

    def copy_images(self, roots, is_img):
        self.lib_img.copy_images(self.obj, roots, is_img)


class LC_cuda(object):
    def __init__(self, a, b, th, m2, m3, source_size, lc_len, img_plane_size, lib_path=None):
        L = self.lib_cuda = _load("liblccuda.so", lib_path)
        d, vp = ctypes.c_double, ctypes.c_void_p
        L.lccuda_new.argtypes = [d] * 6 + [ctypes.c_uint, ctypes.c_long]
        L.lccuda_new.restype = vp
        L.get_lc.argtypes = [vp, d, d, d, d]
        L.get_lc_cuda.argtypes = [vp, d, d, d, d]
        L.copy_lc.argtypes = [vp, ndpointer(dtype=np.double, flags="C_CONTIGUOUS")]
        L.set_limb_darkening_cuda.argtypes = [vp, ctypes.c_char_p, d]
        L.lcirs_set_verbose.argtypes = [vp, ctypes.c_int]
        L.lcirs_delete.argtypes = [vp]
        self.obj = L.lccuda_new(a, b, th, m2, m3, source_size, lc_len, img_plane_size)

    def __del__(self):
        try:
            self.lib_cuda.lcirs_delete(self.obj)
        except Exception:
            pass

    def get_lc(self, iniX, iniY, finX, finY):
        self.lib_cuda.get_lc(self.obj, iniX, iniY, finX, finY)

    def get_lc_cuda(self, iniX, iniY, finX, finY):
        self.lib_cuda.get_lc_cuda(self.obj, iniX, iniY, finX, finY)

    def copy_lc(self, lc_vec):
        self.lib_cuda.copy_lc(self.obj, lc_vec)

    def set_limb_darkening(self, model_type, model_parameter):
        if isinstance(model_type, str):
            model_type = model_type.encode()
        self.lib_cuda.set_limb_darkening_cuda(self.obj, model_type, model_parameter)
