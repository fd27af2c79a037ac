"""C ABI of bin/liblcirs.so without a GPU: the library builds (nvcc cross-
compiles for sm_103a), loads, and exports every function that include/*.h
declares; the reference's six ctypes entry points (src/LightCurves/lcirs.cc:
515-609, bound by Examples/ctypes_classes.py:128-193) are among them.  No
entry point is called here (every one of them reaches the GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")

REFERENCE_ABI = ["lcirs_new", "get_lc", "get_lc_irs", "copy_lc", "set_limb_darkening",
                 "set_amoeba_printout", "ccc_new", "get_cc", "get_ca", "print_ccc", "copy_cc_ca",
                 "copy_lenses", "get_lens_pos", "get_bounding_box", "img_new", "get_roots",
                 "get_images", "set_pos", "copy_images", "lccuda_new", "get_lc_cuda",
                 "set_limb_darkening_cuda"]


def declared_functions(path):
    """Names of the functions declared in a C header (comments and
    preprocessor lines removed; one declaration per ';')."""
    with open(path) as f:
        src = f.read()
    src = re.sub(r"/\*.*?\*/", " ", src, flags=re.S)
    src = re.sub(r"//[^\n]*", " ", src)
    src = "\n".join(l for l in src.splitlines() if not l.lstrip().startswith("#"))
    src = src.replace('extern "C" {', " ").replace("}", " ")
    names = []
    for stmt in src.split(";"):
        stmt = " ".join(stmt.split())
        if "(" not in stmt or stmt.startswith("typedef"):
            continue
        m = re.match(r"^[\w\s\*]+?\b(\w+)\s*\(", stmt)
        if m:
            names.append(m.group(1))
    return names


def c_headers():
    return sorted(os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h"))


def test_headers_declare_the_reference_abi():
    names = set()
    for h in c_headers():
        names.update(declared_functions(h))
    for n in REFERENCE_ABI:
        assert n in names
    assert len(names) >= len(REFERENCE_ABI) + 10


# header -> library that exports it
LIBRARY_OF = {"ccc.h": "libccc.so", "img.h": "libimg.so", "lccuda.h": "liblccuda.so"}


@pytest.mark.parametrize("header", [os.path.basename(h) for h in c_headers()])
def test_library_exports_every_declared_function(product_lib, header):
    lib = ctypes.CDLL(os.path.join(os.path.dirname(product_lib),
                                   LIBRARY_OF.get(header, "liblcirs.so")))
    names = declared_functions(os.path.join(INCLUDE, header))
    assert names, header
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, "%s declares functions the library does not export: %s" % (header,
                                                                                     missing)


def test_product_path_has_no_oracle_dependency():
    """The shipped package never imports the oracle (it is test
    infrastructure)."""
    pkg = os.path.join(ROOT, "triplelens_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".h", ".cpp")):
                with open(os.path.join(dirpath, f)) as fh:
                    text = fh.read()
                assert "import oracle" not in text and "from oracle" not in text, f
                assert "liboracle" not in text, f


def test_entry_points_reject_bad_arguments_without_a_gpu(product_lib):
    """Argument errors return their documented codes before any CUDA call
    (include/tl_batch.h, include/lcirs.h, include/tl_surrogate.h)."""
    lib = ctypes.CDLL(product_lib)
    vp = ctypes.c_void_p
    f = lib.lcirs_fill_device_noalloc
    f.argtypes = [vp, ctypes.c_int] + [vp] * 7
    f.restype = ctypes.c_int
    assert f(None, 10, None, None, None, None, None, None, None) == -1
    for name, args in (("tlb_run_device", [None, 3, None]), ("tlb_stats", [None, None]),
                       ("tlb_graph_launch", [None, None]), ("tlb_graph_capture", [None]),
                       ("tlb_set_fill_stages", [None, 7000, 1])):
        fn = getattr(lib, name)
        fn.restype = ctypes.c_int
        fn.argtypes = [vp if not isinstance(a, int) else ctypes.c_int for a in args]
        assert fn(*args) == -1, name
    fn = lib.tls_predict
    fn.restype = ctypes.c_int
    assert fn(None, 0, None, None, None, ctypes.c_float(0), ctypes.c_float(0), ctypes.c_float(0),
              None, None, None, None, None) == -1
    assert lib.tls_param_count() == 16 * 256 + 256 + 3 * (256 * 256 + 256) + 256 + 1


def test_static_noalloc_scratch_lives_in_liblcirs_only(product_lib):
    """The allocation-free entry point's static device array is linked into
    liblcirs.so alone: a process that loads liblccuda.so as well holds it
    once."""
    lcirs = ctypes.CDLL(product_lib)
    lccuda = ctypes.CDLL(os.path.join(os.path.dirname(product_lib), "liblccuda.so"))
    assert hasattr(lcirs, "lcirs_fill_device_noalloc")
    assert not hasattr(lccuda, "lcirs_fill_device_noalloc")


def test_transfer_byte_counters_read_without_a_gpu(product_lib):
    """lcirs_copy_transfer_bytes reports the library's own host<->device copy
    totals (include/lcirs.h): readable with no GPU work, zero before any
    copy, and tolerant of a null output pointer."""
    from triplelens_gb300.lcirs import transfer_bytes
    lib = ctypes.CDLL(product_lib)
    lib.lcirs_copy_transfer_bytes.argtypes = [ctypes.c_void_p]
    lib.lcirs_copy_transfer_bytes.restype = None
    lib.lcirs_copy_transfer_bytes(None)
    h2d, d2h = transfer_bytes(product_lib)
    assert h2d >= 0 and d2h >= 0
    import torch
    if not torch.cuda.is_available():
        assert (h2d, d2h) == (0, 0)


CXX_CALLER = r"""
// a C++ caller of the reference's class (src/main.cc:165-176 pattern)
#include <cstdio>
#include <cmath>
#include "lcirs.hpp"

// never called here (no GPU): compiled and linked against liblcirs.so
void run_curve(double a, double b, double th, double m2, double m3, std::vector<double>* out) {
  LightCurveIRS lcIRS(a, b, th, m2, m3, 0.001, 100, 50);
  lcIRS.setLimbDarkeningModel(LimbDarkeningModel(0.5));
  lcIRS.setAmoebaPrintOut(false, "amoeba", "pars.json");
  lcIRS.getLCIRS({-1.0, -1.0}, {1.0, 1.0});
  *out = lcIRS.lcVec;
  lcIRS.getLC({-1.0, -1.0}, {1.0, 1.0});
}

static bool same(double x, double y) { return x == y; }

int main(int argc, char**) {
  if (argc > 5) { std::vector<double> v; run_curve(1, 1, 1, 0.1, 0.1, &v); }
  // limbdarkeningmodel.cc:8-37
  LimbDarkeningModel d, n(0.5), l(2.0, 0.4);
  const double i0 = 1.0 / (1.0 - 0.5 / 3.0);
  bool ok = same(d.getParA(), 0.6) && same(d.getParB(), 0.4) &&
            same(d.intensityCoeff, 1.0 / (0.6 + 2.0 / 3.0 * 0.4)) &&
            d.model == LimbDarkeningModel::linear &&
            same(n.getParA(), i0 * 0.5) && same(n.getParB(), i0 * 0.5) &&
            same(n.intensityCoeff, 1.0) && n.model == LimbDarkeningModel::linearNormalized &&
            same(l.getParA(), 2.0 * 0.6) && same(l.getParB(), 2.0 * 0.4) &&
            same(l.intensityCoeff, 1.0 / (2.0 * (1.0 - 0.4 / 3.0))) &&
            same(n.sourceBrightness(0.6), n.getParA() + n.getParB() * std::sqrt(1.0 - 0.36)) &&
            same(n.sourceBrightnessRSq(0.25), n.getParA() + n.getParB() * std::sqrt(0.75));
  printf(ok ? "OK\n" : "FAIL\n");
  return ok ? 0 : 1;
}
"""


def test_cpp_callers_compile_and_link_against_the_class(product_lib, tmp_path):
    """include/lcirs.hpp keeps the reference's C++ interface: a main.cc-style
    caller (constructor, setLimbDarkeningModel with the reference's
    LimbDarkeningModel, setAmoebaPrintOut, getLCIRS, getLC, lcVec) compiles
    and links against liblcirs.so; the model's three forms give the
    reference's coefficients (run without a GPU: the curve is not computed)."""
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    src = tmp_path / "caller.cc"
    src.write_text(CXX_CALLER)
    exe = tmp_path / "caller"
    libdir = os.path.dirname(product_lib)
    r = subprocess.run([gxx, "-std=c++17", "-O1", "-I", INCLUDE, str(src), "-o", str(exe),
                        "-L", libdir, "-llcirs", "-Wl,-rpath," + libdir,
                        "-Wl,--allow-shlib-undefined"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.strip() == "OK", r.stdout + r.stderr


@pytest.mark.parametrize("header", ["lcirs.h", "tl_batch.h", "tl_surrogate.h", "ccc.h", "img.h",
                                    "lccuda.h"])
def test_headers_compile_as_c(header, tmp_path):
    """The C-ABI headers are plain C (what a cgo, JNI or other FFI binding
    includes): each compiles as C11 with -pedantic and no warnings."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("no gcc")
    src = tmp_path / "use.c"
    src.write_text('#include "%s"\nint main(void) { return 0; }\n' % header)
    r = subprocess.run([gcc, "-std=c11", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I",
                        INCLUDE, "-c", str(src), "-o", str(tmp_path / "use.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_integration_guide_names_every_entry_point():
    """INTEGRATION.md names every function include/*.h declares, so a
    maintainer binding the libraries (ctypes, cgo, JNI) finds each one."""
    with open(os.path.join(ROOT, "INTEGRATION.md")) as f:
        guide = f.read()
    missing = []
    for h in sorted(os.listdir(INCLUDE)):
        if not h.endswith(".h"):
            continue
        with open(os.path.join(INCLUDE, h)) as f:
            src = f.read()
        for m in re.finditer(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(\w+)\s*\(", src, re.M):
            if m.group(1) not in guide:
                missing.append((h, m.group(1)))
    assert not missing, missing


@pytest.mark.parametrize("bad", [
    dict(rho=float("nan")), dict(rho=0.0), dict(rho=-1e-3), dict(ppr=0),
    dict(a=float("inf")), dict(m2=float("nan"))])
def test_bad_lens_parameters_come_back_as_status(product_lib, bad):
    """Lens parameters the set-up cannot use (non-finite values, rho <= 0,
    ppr < 1): lcirs_new still returns an object, as the reference's does, but
    it never reaches the GPU; every call leaves zero results and status bit
    32 (bad input) on every point.  Runs without a GPU for that reason."""
    import numpy as np
    from triplelens_gb300.lcirs import LC_irs, MAX_SEEDS
    p = dict(a=1.0, b=0.9, th=1.0, m2=0.2, m3=0.1, rho=1e-3, n=20, ppr=100)
    p.update(bad)
    lc = LC_irs(p["a"], p["b"], p["th"], p["m2"], p["m3"], p["rho"], p["n"], p["ppr"],
                lib_path=product_lib)
    assert lc.last_status() == 32
    lc.set_limb_darkening("linear", 0.5)
    lc.get_lc_irs(-1.0, 0.0, 1.0, 0.1)
    assert lc.last_status() == 32
    assert np.all(lc.status() == 32) and np.all(lc.counts() == 0)
    out = np.full(p["n"], -1.0)
    lc.copy_lc(out)
    assert np.all(out == 0.0)
    lc.get_lc(-1.0, 0.0, 1.0, 0.1)
    lc.copy_lc(out)
    assert np.all(out == 0.0) and lc.last_status() == 32
    seeds = np.zeros((p["n"] + 1, MAX_SEEDS, 2), np.int32)
    lc.fill_from_seeds(-1.0, 0.0, 1.0, 0.1, seeds, np.full(p["n"] + 1, 3, np.int32))
    assert np.all(lc.status() == 32) and np.all(lc.lc_full() == 0.0)
    # no image plane (the amplitude scale, grid[6], follows set_limb_darkening)
    assert np.all(lc.grid()[[0, 1, 2, 3, 4, 5, 7]] == 0.0)
    del lc
