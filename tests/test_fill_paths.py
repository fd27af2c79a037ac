"""The engine's fill paths against the reference's ray counts.

The fill has three stages (triplelens_gb300/csrc/fill.cu): the warp fill (one
warp per point), the team fill (8 warps per large point, in rounds) and the
CTA fill levels (larger tables).  Each point normally goes through the first
stage that can hold it, so most points never see the later ones.  Here every
path runs alone over the first curves of the bench workload (exact warm-start
chain), in child processes with the engine's switches set, and each must give
the reference's ray counts (strict IEEE build, tests/golden/bench_seed2024.npz)
on every point, also when the chain runs in segments beside the fill, and the
same magnifications within the limb-darkening tolerance of the other GPU
tests.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
pytestmark = pytest.mark.gpu

LD_RTOL = 1e-6
CURVES = 2

_CHILD = r"""
import sys, json
import numpy as np
sys.path.insert(0, %(root)r)
from triplelens_gb300 import workloads
from triplelens_gb300.batch import Batch
lenses, trajs, n = workloads.config2(2024, n_curves=%(curves)d, n_points=5000)
b = Batch()
b.set_chain(0)
b.set_lenses(lenses)
b.set_trajectories(trajs, np.arange(len(trajs)), np.full(len(trajs), n))
b.run_device(%(phase)d)
amp, cnt, st = b.download()
np.savez(%(out)r, amp=amp, cnt=cnt, st=st)
"""

PATHS = {
    "default": {},
    "overlapped": {"_phase": "4"},                      # chain in segments beside the fill
    "team": {"TL_WFILL_THR": "0"},                       # every point to the team fill
    "cta": {"TL_FILL_KERNEL": "cta"},                    # the CTA fill alone
    "cta_levels": {"TL_WFILL_THR": "0", "TL_TEAM_FILL": "0"},   # warp fill skips all
}


def _run(env_extra, out, product_lib):
    env = dict(os.environ)
    env.update({k: v for k, v in env_extra.items() if not k.startswith("_")})
    phase = int(env_extra.get("_phase", "3"))
    code = _CHILD % {"root": ROOT, "curves": CURVES, "out": out, "phase": phase}
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    z = np.load(out)
    return z["amp"], z["cnt"], z["st"]


def test_every_fill_path_gives_the_reference_counts(product_lib, tmp_path):
    z = np.load(os.path.join(ROOT, "tests", "golden", "bench_seed2024.npz"))
    n = int(z["n"])
    ref = z["counts"][:CURVES].ravel()
    res = {}
    for name, env in PATHS.items():
        amp, cnt, st = _run(env, str(tmp_path / (name + ".npz")), product_lib)
        assert len(cnt) == CURVES * (n + 1)
        assert np.all((st & 0xC) == 0), name            # complete: no table-full or timeout
        assert np.array_equal(cnt, ref), "%s: %d points differ" % (name, int(np.sum(cnt != ref)))
        res[name] = amp
    base = res["default"]
    for name, amp in res.items():
        assert np.max(np.abs(amp - base) / base) < LD_RTOL, name
