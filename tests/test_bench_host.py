"""bench.py host-side helpers (no GPU): the HBM view of the fill's DRAM
traffic, the CPU legs' point sample and the reference arm's JSON line
shape."""
import json
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_hbm_view():
    import bench
    v = bench.hbm_view(2.0e11, 0.5, {"hbm_gbs": 8000.0})
    assert abs(v["achieved"] - 400.0) < 1e-9 and abs(v["frac"] - 0.05) < 1e-12
    assert v["peak_source"].startswith("MEASURED")
    assert bench.hbm_view(None, 0.5, {}) is None
    assert bench.hbm_view(1.0, 0.0, {}) is None


def test_mufu_view():
    import bench
    v = bench.mufu_view(1.0e12, 4.0, 2070.0, 152)
    assert abs(v["achieved"] - 0.25) < 1e-12
    assert abs(v["peak"] - 16 * 152 * 2.07e9 / 1e12) < 1e-9
    assert abs(v["frac"] - 0.25 / v["peak"]) < 1e-12
    assert bench.mufu_view(0, 4.0, 2070.0, 152) is None
    assert bench.mufu_view(1.0e12, 0.0, 2070.0, 152) is None
    import numpy as np
    assert bench.mufu_view(np.uint64(10 ** 12), 4.0, 2070.0, 152)["achieved"] > 0


def test_reference_arm_prints_one_json_line():
    """`bench.py --impl reference` (the oracle on the host cores) prints the
    contract's line with impl, cpu_baseline and e2e."""
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "0", "--cpu-sample", "16"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "points/s" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0


def test_parity_vs_fixture_counts_mismatches():
    """The bench's parity check reads the reference's counts of its first
    curves from the committed fixture and counts differing points."""
    import numpy as np
    import bench
    z = np.load(os.path.join(ROOT, "tests", "golden", "bench_seed2024.npz"))
    n = int(z["n"])
    cnt = np.concatenate([z["counts"].ravel(), np.zeros(3 * (n + 1), np.uint64)])
    p = bench.parity_vs_fixture(cnt, n, 11, 2024, 0)
    assert p["points"] == 8 * (n + 1) and p["mismatches"] == 0
    cnt[5] += 1
    assert bench.parity_vs_fixture(cnt, n, 11, 2024, 0)["mismatches"] == 1
    assert bench.parity_vs_fixture(cnt, n, 11, 7, 0) is None


def test_cpu_sample_covers_the_whole_curve():
    """The CPU legs sample points along the whole trajectory: one point per
    curve over 152 curves lands in every tenth of the curve, several points
    per curve are distinct and in range, and n+1 points take every point."""
    import bench
    n = 5000
    one = np.array([bench.sample_indices(k, 1, n)[0] for k in range(152)])
    hist = np.histogram(one, bins=10, range=(0, n + 1))[0]
    assert hist.min() >= 10 and one.min() >= 0 and one.max() <= n
    for k in range(20):
        s = bench.sample_indices(k, 7, n)
        assert len(set(s.tolist())) == 7 and s.min() >= 0 and s.max() <= n
    assert sorted(bench.sample_indices(3, n + 1, n).tolist()) == list(range(n + 1))
