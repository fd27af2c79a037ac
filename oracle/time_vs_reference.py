"""Times the oracle (C restatement, oracle/build/liboracle.so) against the
reference's own builds (oracle/_ref/, from oracle/Makefile.ref) on the same
light curves, one core each, to show whether the oracle is a fair stand-in
for the reference's speed where only the oracle can run (the reference's
lcirs.cc needs x86 AVX).  Test infrastructure: runs where oracle/_ref/ was
built, never on the product path.

    python oracle/time_vs_reference.py [--curves 4] [--points 200]

Each reference run happens in a child process of its own (its per-point
stdout and its heap history stay there); the times cover get_lc_irs only
(lens set-up excluded on both sides).
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
# run as a script, this directory comes first on the path and would shadow
# the oracle package with its oracle.py module
sys.path = [p for p in sys.path if os.path.abspath(p or ".") != HERE]
sys.path.insert(0, ROOT)

BUILDS = {"fast": "liblcirs_ref.so", "nfc": "liblcirs_ref_nfc.so",
          "strict": "liblcirs_ref_strict.so"}


def _child(spec):
    L = ctypes.cdll.LoadLibrary(spec["lib"])
    d = ctypes.c_double
    L.lcirs_new.argtypes = [d] * 6 + [ctypes.c_uint, ctypes.c_long]
    L.lcirs_new.restype = ctypes.c_void_p
    L.get_lc_irs.argtypes = [ctypes.c_void_p] + [d] * 4
    L.set_limb_darkening.argtypes = [ctypes.c_void_p, ctypes.c_char_p, d]
    lens, traj, n = spec["lens"], spec["traj"], spec["n"]
    o = L.lcirs_new(*lens[:5], lens[5], n, int(lens[7]))
    L.set_limb_darkening(o, b"linear", lens[6])
    t0 = time.perf_counter()
    L.get_lc_irs(o, *traj)
    sys.stderr.write("TIME %.6f\n" % (time.perf_counter() - t0))


def _time_reference(lib, lens, traj, n):
    spec = {"lib": lib, "lens": [float(x) for x in lens], "traj": [float(x) for x in traj],
            "n": int(n)}
    r = subprocess.run([sys.executable, __file__, "--child", json.dumps(spec)],
                       capture_output=True, text=True, check=True)
    return float([ln for ln in r.stderr.splitlines() if ln.startswith("TIME")][0].split()[1])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--child")
    ap.add_argument("--curves", type=int, default=4)
    ap.add_argument("--points", type=int, default=200)
    ap.add_argument("--seed", type=int, default=2024)
    args = ap.parse_args()
    if args.child:
        _child(json.loads(args.child))
        return
    from oracle import oracle
    from triplelens_gb300 import workloads
    libs = {k: os.path.join(HERE, "_ref", v) for k, v in BUILDS.items()}
    missing = [v for v in libs.values() if not os.path.exists(v)]
    if missing:
        sys.exit("build the reference first (make -f oracle/Makefile.ref REF=...): missing %s"
                 % missing)
    lenses, trajs, _ = workloads.config2(args.seed, n_curves=args.curves, n_points=args.points)
    n = args.points
    totals = {k: 0.0 for k in list(libs) + ["oracle"]}
    for k in range(args.curves):
        L, t = lenses[k], trajs[k]
        row = {name: _time_reference(lib, L, t, n) for name, lib in libs.items()}
        o = oracle.OracleIRS(*L[:5], L[5], n, int(L[7]))
        o.set_limb_darkening("linear", L[6])
        t0 = time.perf_counter()
        o.lc_irs(*t)
        row["oracle"] = time.perf_counter() - t0
        for key, v in row.items():
            totals[key] += v
        print(json.dumps({"curve": k, "seconds": {a: round(b, 4) for a, b in row.items()}}))
    print(json.dumps({"curves": args.curves, "points_per_curve": n + 1,
                      "seconds": {a: round(b, 3) for a, b in totals.items()},
                      "reference_time_over_oracle_time": {
                          a: round(totals[a] / totals["oracle"], 3) for a in libs}}))


if __name__ == "__main__":
    main()
