"""Generates the golden fixtures in tests/golden/ from the REFERENCE itself.

Runs only where the reference sources are present: it builds the reference
library with oracle/Makefile.ref (into oracle/_ref/, git-ignored) and drives
it through its own ctypes ABI (lcirs_new / set_limb_darkening / get_lc_irs /
copy_lc, ccc_new / get_ca / copy_cc_ca, img_new / get_images / copy_images).
Ray counts are read from the reference's per-point stdout line
"irs amplification: A and the count N ..." (lcirs.cc:176-177); the filled
sets from its amoeba dump files (amoeba.cc:90-108).

Three reference builds (oracle/Makefile.ref): "strict" (IEEE, -O2
-fno-fast-math -ffp-contract=off), the pinned parity target; "nfc" and
"fast", the makefile's -Ofast flags without and with FMA contraction, kept to
show the reference's own build-to-build spread.

    python tests/golden/make_golden.py --ref <TripleLens checkout> [--c2] [--bench]
        [--only-ccc | --only-bench | --only-config4 | --only-extra]

(--ref may be replaced by TRIPLELENS_REF in the environment.)  Each reference
run happens in a child process of its own (its stdout is C++ cout, and its
warm start depends on the process's heap history), several at a time.  The
committed outputs are small .npz files; this script is kept beside them.
"""
import argparse
import ctypes
import json
import os
import re
import subprocess
import sys
import tempfile
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from triplelens_gb300 import workloads  # noqa: E402

REF_LIBS = {
    "strict": os.path.join(ROOT, "oracle", "_ref", "liblcirs_ref_strict.so"),
    "nfc": os.path.join(ROOT, "oracle", "_ref", "liblcirs_ref_nfc.so"),
    "fast": os.path.join(ROOT, "oracle", "_ref", "liblcirs_ref.so"),
}
POOL = ThreadPoolExecutor(max_workers=os.cpu_count() or 4)


def worker(spec):
    """Child process: one reference light curve; counts go to stdout."""
    L = ctypes.cdll.LoadLibrary(spec["lib"])
    d = ctypes.c_double
    L.lcirs_new.argtypes = [d] * 6 + [ctypes.c_uint, ctypes.c_long]
    L.lcirs_new.restype = ctypes.c_void_p
    L.get_lc_irs.argtypes = [ctypes.c_void_p] + [d] * 4
    L.copy_lc.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    L.set_limb_darkening.argtypes = [ctypes.c_void_p, ctypes.c_char_p, d]
    L.set_amoeba_printout.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p]
    a, b, th, m2, m3, rho, v, ppr = spec["lens"]
    n = spec["n"]
    o = L.lcirs_new(a, b, th, m2, m3, rho, n, int(ppr))
    if v >= 0:
        L.set_limb_darkening(o, b"linear", v)
    else:
        L.set_limb_darkening(o, b"default", 0.0)
    if spec.get("amoeba"):
        L.set_amoeba_printout(o, spec["amoeba"].encode(), (spec["amoeba"] + "pars.json").encode())
    x0, y0, x1, y1 = spec["traj"]
    L.get_lc_irs(o, x0, y0, x1, y1)
    out = np.zeros(n)
    L.copy_lc(o, out.ctypes.data_as(ctypes.c_void_p))
    np.save(spec["amp_out"], out)


def _big_stack():
    import resource
    soft, hard = resource.getrlimit(resource.RLIMIT_STACK)
    want = 1 << 33
    if hard != resource.RLIM_INFINITY:
        want = min(want, hard)
    resource.setrlimit(resource.RLIMIT_STACK, (want, hard))


def run_curve(lib, lens, traj, n, amoeba=None):
    with tempfile.TemporaryDirectory() as td:
        spec = {"lib": lib, "lens": [float(x) for x in lens], "traj": [float(x) for x in traj],
                "n": int(n), "amp_out": os.path.join(td, "amp.npy"), "amoeba": amoeba}
        # the reference's flood fill recurses once per filled row
        # (lcirs.cc:446-463): the largest images need more than the default
        # 8 MiB of stack
        r = subprocess.run([sys.executable, __file__, "--worker", json.dumps(spec)],
                           capture_output=True, text=True, check=True, preexec_fn=_big_stack)
        counts = np.array([int(m) for m in re.findall(r"the count (\d+)", r.stdout)], np.uint64)
        amps = np.load(spec["amp_out"])
    assert len(counts) == n + 1, (len(counts), n)
    return counts, amps


def read_amoeba(path):
    t = np.loadtxt(path, delimiter=",", dtype=np.int64, ndmin=2).reshape(-1, 3)
    return t[np.lexsort((t[:, 1], t[:, 0]))]


# critical-curve / caustic cases for libccc.so: (a, b, th, m2, m3, length);
# m3 == 0 takes the reference's binary path
CCC_CASES = [
    (1.0, 0.9433981132056603, 1.0121970114513341, 0.2, 0.1, 500),
    (1.0, 0.9433981132056603, 1.0121970114513341, 0.2, 0.1, 333),
    (0.7, 1.4, 2.3, 0.05, 0.002, 500),
    (1.2, 0.0, 0.0, 0.3, 0.0, 500),
    (0.8, 1.0, 0.5, 0.1, 0.0, 400),
]


def ccc_worker(spec):
    """Child process: one reference CCC object (its stdout is C++ cout)."""
    L = ctypes.cdll.LoadLibrary(spec["lib"])
    d, vp = ctypes.c_double, ctypes.c_void_p
    L.ccc_new.argtypes = [d] * 5 + [ctypes.c_int]
    L.ccc_new.restype = vp
    L.get_cc.argtypes = [vp]
    L.get_ca.argtypes = [vp]
    L.print_ccc.argtypes = [vp, ctypes.c_char_p]
    L.copy_cc_ca.argtypes = [vp, vp, vp]
    L.copy_lenses.argtypes = [vp, vp]
    L.get_bounding_box.argtypes = [vp, vp, vp, vp, vp, d]
    a, b, th, m2, m3, length = spec["case"]
    o = L.ccc_new(a, b, th, m2, m3, length)
    # the reference's scripts call get_ca alone (run_amoebae*.py); a binary
    # lens must take that route (get_cc first leaves it with more critical-
    # curve than caustic branches, which copy_cc_ca then reads past)
    if m3 != 0.0:
        L.get_cc(o)
    L.get_ca(o)
    order = 4 if m3 == 0.0 else 6
    cc = np.zeros(order * length, np.complex128)
    ca = np.zeros(order * length, np.complex128)
    L.copy_cc_ca(o, cc.ctypes.data_as(vp), ca.ctypes.data_as(vp))
    lz = np.zeros(3, np.complex128)
    L.copy_lenses(o, lz.ctypes.data_as(vp))
    box = np.zeros(4, np.complex128)
    L.get_bounding_box(o, *[box[k:].ctypes.data_as(vp) for k in range(4)], 1.1)
    L.print_ccc(o, spec["file"].encode())
    np.savez(spec["out"], cc=cc, ca=ca, lenses=lz, box=box)


def point_worker(spec):
    """Child process: the reference's point-source curve (get_lc,
    lcbase.cc:40-52) of one lens and trajectory."""
    L = ctypes.cdll.LoadLibrary(spec["lib"])
    d, vp = ctypes.c_double, ctypes.c_void_p
    L.lcirs_new.argtypes = [d] * 6 + [ctypes.c_uint, ctypes.c_long]
    L.lcirs_new.restype = vp
    L.get_lc.argtypes = [vp] + [d] * 4
    L.copy_lc.argtypes = [vp, vp]
    a, b, th, m2, m3, rho, v, ppr = spec["lens"]
    n = spec["n"]
    o = L.lcirs_new(a, b, th, m2, m3, rho, n, int(ppr))
    L.get_lc(o, *spec["traj"])
    out = np.zeros(n)
    L.copy_lc(o, out.ctypes.data_as(vp))
    np.save(spec["out"], out)


def point_fixtures(lib):
    """Point-source curves of the config-1 lens and of three config-2 lenses."""
    lens, traj, n = workloads.config1()
    lenses, trajs, _ = workloads.config2(seed=11, n_curves=3)
    cases = [(lens, traj, n)] + [(lenses[k], trajs[k], 500) for k in range(3)]
    out = {}
    with tempfile.TemporaryDirectory() as td:
        for k, (L2, t, nn) in enumerate(cases):
            spec = {"lib": lib, "lens": [float(x) for x in L2], "traj": [float(x) for x in t],
                    "n": nn, "out": os.path.join(td, "p_%d.npy" % k)}
            subprocess.run([sys.executable, __file__, "--point-worker", json.dumps(spec)],
                           capture_output=True, text=True, check=True)
            out["lens_%d" % k] = np.asarray(L2)
            out["traj_%d" % k] = np.asarray(t)
            out["amps_%d" % k] = np.load(spec["out"])
    out["cases"] = np.array(len(cases))
    return out


def ccc_fixtures(lib):
    out = {"cases": np.array(CCC_CASES)}
    with tempfile.TemporaryDirectory() as td:
        for k, case in enumerate(CCC_CASES):
            spec = {"lib": lib, "case": case, "file": os.path.join(td, "ccc_%d.txt" % k),
                    "out": os.path.join(td, "ccc_%d.npz" % k)}
            r = subprocess.run([sys.executable, __file__, "--ccc-worker", json.dumps(spec)],
                               capture_output=True, text=True, check=True)
            z = np.load(spec["out"])
            for key in ("cc", "ca", "lenses", "box"):
                out["%s_%d" % (key, k)] = z[key]
            if k in (0, 3):   # one triple and one binary print_ccc file
                with open(spec["file"]) as f:
                    out["text_%d" % k] = np.array(f.read())
            out["stdout_%d" % k] = np.array(r.stdout)
    return out


def ccc_and_images(lib, lens, positions):
    L = ctypes.cdll.LoadLibrary(lib)
    d = ctypes.c_double
    L.ccc_new.argtypes = [d] * 5 + [ctypes.c_int]
    L.ccc_new.restype = ctypes.c_void_p
    L.get_ca.argtypes = [ctypes.c_void_p]
    L.copy_cc_ca.argtypes = [ctypes.c_void_p] * 3
    L.img_new.argtypes = [d] * 7
    L.img_new.restype = ctypes.c_void_p
    L.get_images.argtypes = [ctypes.c_void_p]
    L.copy_images.argtypes = [ctypes.c_void_p] * 3
    a, b, th, m2, m3 = lens[:5]
    obj = L.ccc_new(a, b, th, m2, m3, 500)
    L.get_ca(obj)
    cc = np.zeros(3000, np.complex128)
    ca = np.zeros(3000, np.complex128)
    L.copy_cc_ca(obj, cc.ctypes.data_as(ctypes.c_void_p), ca.ctypes.data_as(ctypes.c_void_p))
    roots = np.zeros((len(positions), 10), np.complex128)
    isimg = np.zeros((len(positions), 10), np.bool_)
    for k, (sx, sy) in enumerate(positions):
        im = L.img_new(a, b, th, m2, m3, sx, sy)
        L.get_images(im)
        r = np.zeros(10, np.complex128)
        f = np.zeros(10, np.bool_)
        L.copy_images(im, r.ctypes.data_as(ctypes.c_void_p), f.ctypes.data_as(ctypes.c_void_p))
        roots[k], isimg[k] = r, f
    return cc, ca, roots, isimg


# small cases that no other fixture covers: a binary lens (m3 == 0: the
# two-lens ray map, lcirs.cc:28-36, and the binary image count), a two-point
# curve (n = 1) and a curve far from the caustics.  The far curve has n = 6:
# at n = 5 the reference's own write past lcVec (lcirs.cc:117,181, quirk Q1)
# lands on the next heap chunk's header, because 5 doubles fill their malloc
# chunk exactly, and glibc aborts the process ("corrupted size vs. prev_size");
# for most n the write falls into the chunk's rounding slack
EXTRA_CASES = [
    ("binary", [1.2, 0.9, 1.0, 0.3, 0.0, 0.01, 0.0, 60.0], [-1.5, 0.05, 1.5, 0.15], 40),
    ("short", [1.0, 1.0, 1.2, 0.1, 0.05, 0.02, 0.3, 40.0], [0.1, 0.2, 0.3, 0.1], 1),
    ("far", [1.0, 1.0, 1.2, 0.1, 0.05, 0.02, 0.3, 40.0], [1.8, 1.9, 2.1, 1.7], 6),
]


def extra_fixtures():
    out = {}
    jobs = {}
    for name, lens, traj, n in EXTRA_CASES:
        out["lens_" + name] = np.array(lens)
        out["traj_" + name] = np.array(traj)
        out["n_" + name] = np.array(n)
        for build, lib in REF_LIBS.items():
            jobs[(name, build)] = POOL.submit(run_curve, lib, np.array(lens), np.array(traj), n)
    for (name, build), f in jobs.items():
        out["counts_%s_%s" % (name, build)], out["amps_%s_%s" % (name, build)] = f.result()
    return out


def config4_fixture(n_curves=8, n=20):
    """Config-4 curves (each its own lens, rho log-uniform in [1e-4, 3e-2],
    200/500/1000 rays per radius, v in [0.3, 0.7]): n + 1 points each."""
    lenses, trajs, _ = workloads.config4(seed=5, n_curves=n_curves)
    out = {"lenses": lenses, "trajs": trajs, "n": np.array(n)}
    for build in ("strict", "fast"):
        res = curves(REF_LIBS[build], lenses, trajs, n)
        out["counts_" + build] = np.array([c for c, _ in res])
        out["amps_" + build] = np.array([a for _, a in res])
    return out


def curves(lib, lenses, trajs, n):
    """Reference curves, several child processes at a time."""
    futs = [POOL.submit(run_curve, lib, lenses[k], trajs[k], n) for k in range(len(lenses))]
    return [f.result() for f in futs]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("TRIPLELENS_REF"))
    ap.add_argument("--worker")
    ap.add_argument("--c2", action="store_true", help="also the 5000-point config-2 curve")
    ap.add_argument("--bench", action="store_true",
                    help="also the benchmark's 8 curves (seed 2024, strict build only)")
    ap.add_argument("--ccc-worker")
    ap.add_argument("--point-worker")
    ap.add_argument("--only-ccc", action="store_true")
    ap.add_argument("--only-bench", action="store_true",
                    help="only the benchmark fixture (implies --bench)")
    ap.add_argument("--only-extra", action="store_true",
                    help="only extra_cases.npz (binary lens, short and far curves)")
    ap.add_argument("--only-config4", action="store_true",
                    help="only config4_sample.npz (config-4 lenses, radii and densities)")
    args = ap.parse_args()
    if args.worker:
        worker(json.loads(args.worker))
        return
    if args.ccc_worker:
        ccc_worker(json.loads(args.ccc_worker))
        return
    if args.point_worker:
        point_worker(json.loads(args.point_worker))
        return
    if not args.ref:
        ap.error("give --ref <TripleLens checkout> or set TRIPLELENS_REF")
    subprocess.run(["make", "-s", "-f", "oracle/Makefile.ref", "REF=" + args.ref], cwd=ROOT,
                   check=True)

    if args.only_bench:
        args.bench = True
        bench_fixture()
        return
    np.savez_compressed(os.path.join(HERE, "config4_sample.npz"), **config4_fixture())
    print("wrote config4_sample.npz")
    if args.only_config4:
        return
    np.savez_compressed(os.path.join(HERE, "extra_cases.npz"), **extra_fixtures())
    print("wrote extra_cases.npz")
    if args.only_extra:
        return
    np.savez_compressed(os.path.join(HERE, "ccc.npz"), **ccc_fixtures(REF_LIBS["fast"]))
    print("wrote ccc.npz")
    np.savez_compressed(os.path.join(HERE, "point_lc.npz"), **point_fixtures(REF_LIBS["strict"]))
    print("wrote point_lc.npz")
    if args.only_ccc:
        return

    lens, traj, n = workloads.config1()
    out = {"lens": lens, "traj": traj, "n": n}
    jobs = {}
    for tag, v in (("uniform", 0.0), ("default", -1.0), ("linear05", 0.5)):
        L2 = lens.copy()
        L2[6] = v
        for build, lib in REF_LIBS.items():
            jobs[(tag, build)] = POOL.submit(run_curve, lib, L2, traj, n)
    for (tag, build), f in jobs.items():
        out["counts_%s_%s" % (tag, build)], out["amps_%s_%s" % (tag, build)] = f.result()
    with tempfile.TemporaryDirectory() as td:
        L2 = lens.copy()
        L2[6] = 0.0
        run_curve(REF_LIBS["strict"], L2, traj, n, amoeba=os.path.join(td, "amo_"))
        pts = [0, 20, 50, 75, 100]
        out["amoeba_points"] = np.array(pts)
        for p in pts:
            out["amoeba_%d" % p] = read_amoeba(os.path.join(td, "amo_%d" % p))
        with open(os.path.join(td, "amo_pars.json")) as f:
            out["pars_json"] = np.array(f.read())
    rng = np.random.Generator(np.random.PCG64(7))
    positions = rng.uniform(-1.0, 1.5, size=(64, 2))
    cc, ca, roots, isimg = ccc_and_images(REF_LIBS["strict"], lens, positions)
    out.update(cc=cc, ca=ca, img_positions=positions, img_roots=roots, img_isimg=isimg)
    np.savez_compressed(os.path.join(HERE, "config1.npz"), **out)
    print("wrote config1.npz")

    # config-2 lenses, short curves (201 points over the same 4 theta_E)
    lenses, trajs, _ = workloads.config2(seed=11, n_curves=3)
    c2 = {"lenses": lenses, "trajs": trajs, "n": 200}
    for build, key in (("strict", "counts_%d"), ("nfc", "counts_nfc_%d"),
                       ("fast", "counts_fast_%d")):
        for k, (c, a) in enumerate(curves(REF_LIBS[build], lenses, trajs, 200)):
            c2[key % k] = c
            if build == "strict":
                c2["amps_%d" % k] = a
    np.savez_compressed(os.path.join(HERE, "config2_short.npz"), **c2)
    print("wrote config2_short.npz")

    if args.c2:
        lenses, trajs, n = workloads.config2(seed=0, n_curves=1)
        res = {b: POOL.submit(run_curve, REF_LIBS[b], lenses[0], trajs[0], n) for b in REF_LIBS}
        (c, a), (cn, _), (cf, _) = [res[b].result() for b in ("strict", "nfc", "fast")]
        np.savez_compressed(os.path.join(HERE, "config2_seed0.npz"), lenses=lenses, trajs=trajs,
                            n=n, counts=c, amps=a, counts_nfc=cn, counts_fast=cf)
        print("wrote config2_seed0.npz")

    if args.bench:
        bench_fixture()


def bench_fixture():
    """The benchmark's workload: 8 config-2 curves of seed 2024 (rank 0),
    strict build."""
    lenses, trajs, n = workloads.config2(seed=2024, n_curves=8)
    res = curves(REF_LIBS["strict"], lenses, trajs, n)
    np.savez_compressed(os.path.join(HERE, "bench_seed2024.npz"), lenses=lenses, trajs=trajs,
                        n=n, counts=np.stack([c for c, _ in res]),
                        amps=np.stack([a for _, a in res]))
    print("wrote bench_seed2024.npz")


if __name__ == "__main__":
    main()
