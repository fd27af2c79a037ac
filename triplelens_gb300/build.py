"""Build recipe for the engine's shared libraries (nvcc, sm_103a only).

Outputs (in-tree, git-ignored):
  bin/liblcirs.so   LightCurveIRS C ABI + GPU engine
  bin/libccc.so     critical-curve / caustic C ABI (GPU set-up kernel)

Translation units compile in parallel; seeds.cu and chain.cu are
compiled with --fmad=false so their FP64 arithmetic matches a
-ffp-contract=off host build bit for bit.
"""
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "triplelens_gb300", "csrc")
INC = os.path.join(ROOT, "include")
BIN = os.path.join(ROOT, "bin")
OBJ = os.path.join(ROOT, "_build", "obj")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
          "-Xcompiler", "-ffp-contract=off", "-I" + INC, "-I" + CSRC]

# (source, extra flags)
UNITS = [
    ("seeds.cu", ["--fmad=false"]),
    ("chain.cu", ["--fmad=false"]),
    ("fill.cu", []),
    ("engine_host.cu", []),
    ("lcirs_abi.cu", []),
    ("batch_abi.cu", []),
    ("noalloc_abi.cu", []),
    ("surrogate.cu", []),
    ("ccc_abi.cu", ["--fmad=false"]),
    ("img_abi.cu", ["--fmad=false"]),
    ("lccuda_abi.cu", []),
]

LIBS = {
    "liblcirs.so": ["seeds.cu", "chain.cu", "fill.cu", "engine_host.cu", "lcirs_abi.cu", "batch_abi.cu",
                    "noalloc_abi.cu", "surrogate.cu"],
    "libccc.so": ["ccc_abi.cu"],
    "libimg.so": ["img_abi.cu"],
    # without noalloc_abi.cu: its static scratch array stays in liblcirs.so
    # alone, so a process that loads both libraries holds it once
    "liblccuda.so": ["seeds.cu", "chain.cu", "fill.cu", "engine_host.cu", "lcirs_abi.cu", "batch_abi.cu",
                     "surrogate.cu", "lccuda_abi.cu"],
}


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _compile(unit, verbose=False):
    src, extra = unit
    out = os.path.join(OBJ, src.replace(".cu", ".o"))
    deps = [os.path.join(CSRC, src)] + [os.path.join(CSRC, f) for f in os.listdir(CSRC)
                                        if f.endswith(".h")] + \
        [os.path.join(INC, f) for f in os.listdir(INC)]
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out
    cmd = [nvcc()] + ARCH + COMMON + extra + ["-c", os.path.join(CSRC, src), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    if verbose and r.stderr:
        print(r.stderr)
    return out


def build(verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(BIN, exist_ok=True)
    units = [u for u in UNITS if os.path.exists(os.path.join(CSRC, u[0]))]
    with ThreadPoolExecutor(max_workers=min(8, len(units))) as ex:
        objs = dict(zip([u[0] for u in units], ex.map(lambda u: _compile(u, verbose), units)))
    for lib, srcs in LIBS.items():
        if not all(s in objs for s in srcs):
            continue
        out = os.path.join(BIN, lib)
        ins = [objs[s] for s in srcs]
        if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(o) for o in ins):
            continue
        cmd = [nvcc()] + ARCH + ["-shared", "-o", out] + ins + ["-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed for %s:\n%s" % (lib, r.stderr))
    return BIN


if __name__ == "__main__":
    build(verbose=True)
    print("built", BIN)
