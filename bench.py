"""Benchmark: finite-source light-curve points/s on one GB300 (plain GPU IRS).

Workload (the configuration the metric is quoted on): random triple lenses
from a seed, masses from ratios log-uniform in [1e-3, 1], separations
log-uniform in [0.5, 2], trajectories of 4 theta_E with impact parameter
uniform in [-0.5, 0.5], 5000 points each (5001 computed, the reference's
sampling), rho = 1e-3, 500 rays per source radius, linear limb darkening
v = 0.5.  A step = one batch of --curves light curves (default 152, one per
SM) through the seeds kernels and the persistent fill kernel, every curve
with one warm-start chain in the reference's order, so the ray counts are the
reference's (the first 8 curves are checked against its counts).  Synthetic,
seeded data.

JSON keys: value = points/s with inputs resident in HBM (device-timed with
CUDA events on the launching stream, L2 flushed between steps); e2e = the same
metric through the reference's C ABI (lcirs_new / get_lc_irs / copy_lc per
curve from host threads, host buffers, copies and lens set-up inside the
timed region); parity = counts against the reference's; roofline = the fill
kernel against the FP32 pipe; fast_chain = the same workload with chunked
warm-start chains; cpu_baseline = the oracle (C restatement of the
reference's CPU IRS, bit-identical to its strict build) on the host's cores
over a bounded sample of the same points.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "finite-source light-curve points/s at <=1e-3 rel. error: IRS vs surrogate-gated"
UNIT = "points/s"
FLOP_PER_RAY = 32.0       # triple map + disc test per evaluated ray
FLOP_PER_WEIGHT = 6.0     # limb-darkened weight per accepted ray


# ---------------------------------------------------------------------------
# CPU baseline: the oracle over a bounded sample of points
# ---------------------------------------------------------------------------
def _cpu_worker(args):
    lens, traj, n, idx = args
    from oracle import oracle
    o = oracle.OracleIRS(*lens[:5], lens[5], n, int(lens[7]))
    o.set_limb_darkening("linear", lens[6])
    # the seeds need the whole warm-start chain up to each sampled point; its
    # time is charged to the sample in proportion to the points it covers
    t0 = time.perf_counter()
    seeds, cnt, _ = o.lc_seeds(*traj)
    t_seeds = (time.perf_counter() - t0) * len(idx) / (n + 1.0)
    t0 = time.perf_counter()
    rays = 0
    for p in idx:
        x = traj[0] + (traj[2] - traj[0]) * (p / n)
        y = traj[1] + (traj[3] - traj[1]) * (p / n)
        _, c = o.fill(x, y, seeds[p, :cnt[p]])
        rays += c
    return time.perf_counter() - t0 + t_seeds, len(idx), rays, t_seeds


def sample_indices(k, per_curve, n):
    """Point indices of curve k in the CPU sample: `per_curve` points evenly
    spaced along the curve, shifted by a golden-ratio offset per curve, so
    that with one point per curve the sample still covers every position
    along the trajectories (near and far from the lenses) instead of the
    curves' first points alone."""
    step = (n + 1) / float(per_curve)
    off = ((k + 0.5) * 0.6180339887498949) % 1.0
    return np.minimum(((np.arange(per_curve) + off) * step).astype(np.int64), n)


def cpu_baseline(pool, procs, lenses, trajs, n, sample_points):
    """Times the oracle (image chain + fill) on `sample_points` points spread
    over the curves, split over `procs` concurrent processes; returns
    (points/s all cores, points/s one core, rays/s all cores, description,
    busy seconds).

    A point costs its fill plus its 1/(n+1) share of its curve's warm-start
    chain (the reference computes every point of a curve in one chain).  A
    sampled point still needs the chain up to it, so each task runs its
    curve's whole chain but is charged only the sampled points' shares; the
    rates divide the sampled points by the charged CPU seconds (each
    measured inside its process while the others run), times the processes
    that ran, not by the wall time, which would count the uncharged chain
    work."""
    ncurves = len(lenses)
    use = min(ncurves, max(1, sample_points))
    per_curve = max(1, sample_points // use)
    tasks = []
    for k in range(use):
        pts = sample_indices(k, per_curve, n)
        for chunk in np.array_split(pts, max(1, procs // use)):
            if len(chunk):
                tasks.append((lenses[k], trajs[k], n, chunk.tolist()))
    res = pool.map(_cpu_worker, tasks)
    busy = sum(r[0] for r in res)
    npts = sum(r[1] for r in res)
    rays = sum(r[2] for r in res)
    t_seed = sum(r[3] for r in res)
    par = min(procs, len(tasks))
    desc = ("%d points spread along %d curves (%d per curve): oracle fill + each point's share "
            "of its curve's image chain (%.3f s of %.2f s charged CPU time), %d concurrent "
            "processes; points/s = points x processes / charged CPU seconds"
            % (npts, use, per_curve, t_seed, busy, par))
    return npts * par / busy, npts / busy, rays * par / busy, desc, busy


class quiet_stdout:
    """Sends fd 1 to /dev/null: the reference ABI reports on stdout ("model
    is linear", per-point lines), and this script prints one JSON line."""

    def __enter__(self):
        import ctypes
        self.libc = ctypes.CDLL(None)
        sys.stdout.flush()
        self.libc.fflush(None)
        self.saved = os.dup(1)
        nul = os.open(os.devnull, os.O_WRONLY)
        os.dup2(nul, 1)
        os.close(nul)
        return self

    def __exit__(self, *a):
        self.libc.fflush(None)
        os.dup2(self.saved, 1)
        os.close(self.saved)


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    def __init__(self, path):
        self.path = path
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + q, "--format=csv",
                                          "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self, gpu_index=0):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        try:
            lines = open(self.path).read().strip().splitlines()[1:]
        except Exception:
            return out
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9 or f[0] != str(gpu_index):
                continue
            try:
                sm.append(float(f[1].split()[0]))
                mx = float(f[2].split()[0])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if sm:
            busy = [s for s in sm if s > 0.5 * max(sm)]
            out["sm_mhz"] = float(np.median(busy))
            out["sm_max_mhz"] = mx
            out["reasons"] = sorted(reasons)
            out["samples"] = len(sm)
        return out


def fp32_peak_tflops(sm_max_mhz):
    """FP32 FMA peak: 152 SMs x 128 lanes x 2 flop at the SM clock."""
    try:
        import torch
        sms = torch.cuda.get_device_properties(0).multi_processor_count
    except Exception:
        sms = 152
    return 2.0 * 128 * sms * sm_max_mhz * 1e6 / 1e12, sms


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


def hbm_view(traffic_bytes, fill_s, peaks):
    """The fill's DRAM traffic per launch (from the ncu calibration) as a
    bandwidth against the measured HBM copy peak: how far the kernel is from
    being memory-bound."""
    peak = peaks.get("hbm_gbs") or 6800.0
    if not traffic_bytes or not fill_s or fill_s <= 0:
        return None
    gbs = traffic_bytes / fill_s / 1e9
    return {"achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
            "peak_source": "MEASURED_PEAKS hbm_gbs" if peaks.get("hbm_gbs") else "fallback"}


def mufu_view(evaluated_rays, fill_s, sm_mhz, sms):
    """The fill's special-function work as a rate against the nominal MUFU
    rate (16 operations per clock per SM): the split map has no divisions,
    and each evaluated ray takes one square root (its limb-darkening
    weight)."""
    if not evaluated_rays or not fill_s or fill_s <= 0 or not sm_mhz or not sms:
        return None
    achieved = float(evaluated_rays) / fill_s / 1e12
    peak = 16.0 * sms * sm_mhz * 1e6 / 1e12
    return {"achieved": achieved, "peak": peak, "unit": "Tops/s", "frac": achieved / peak,
            "ops_per_ray": 1, "peak_source": "16 MUFU ops/clock/SM x %d SMs x %.0f MHz (nominal)"
                                            % (sms, sm_mhz)}


# ---------------------------------------------------------------------------
def config4_leg(seed, curves, reps):
    """Config 4 (sub-sample): `curves` light curves of 2000 points, each its
    own random lens with rho log-uniform in [1e-4, 3e-2], 200/500/1000 rays
    per radius and v in [0.3, 0.7]; the fill stages' sharing of the points
    from the autotuner; seeds + fill replayed as one CUDA graph
    (device-resident inputs)."""
    import torch
    from triplelens_gb300 import workloads
    from triplelens_gb300.batch import Batch
    lenses, trajs, n = workloads.config4(seed + 3, n_curves=curves)
    b = Batch()
    b.set_chain(0)
    b.set_lenses(lenses)
    npts = b.set_trajectories(trajs, np.arange(curves), np.full(curves, n))
    t0 = time.perf_counter()
    chosen, times = b.autotune(sample_points=0)   # every point: the largest decide
    t_tune = time.perf_counter() - t0
    stream = torch.cuda.Stream()
    b.graph_capture()
    b.graph_launch(stream.cuda_stream)
    stream.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        b.graph_launch(stream.cuda_stream)
    e1.record(stream)
    e1.synchronize()
    ms_graph = e0.elapsed_time(e1) / reps
    e0.record(stream)
    b.run_device(3, stream.cuda_stream)
    e1.record(stream)
    e1.synchronize()
    ms_plain = e0.elapsed_time(e1)
    _, cnt, st = b.download(stream.cuda_stream)
    stats = b.stats()
    parity = config4_fixture_parity()
    return {"workload": "config 4 sub-sample: %d curves x %d points, own lens each" % (curves, n + 1),
            "points": int(npts), "ms_per_replay": ms_graph, "points_per_s": npts / (ms_graph / 1e3),
            "rays_evaluated_per_s": float(stats[0]) / (ms_graph / 1e3),
            "ms_plain_launches": ms_plain,
            "autotune": {"warp_fill_threshold_blocks": chosen[0], "team_fill": bool(chosen[1]),
                         "points_timed": chosen[2],
                         "candidates_ms": {"warp<=7000+team": float(times[0]),
                                           "warp<=3000+team": float(times[1]),
                                           "warp<=1500+team": float(times[2]),
                                           "warp<=7000+cta": float(times[3]),
                                           "cta": float(times[4])},
                         "seconds": round(t_tune, 2)},
            "status_or": int(np.bitwise_or.reduce(st)),
            # points whose magnification is incomplete (table full or a wait ran out)
            "incomplete_points": int(((st & 0xC) != 0).sum()),
            "status_counts": status_counts(st),
            "parity_vs_reference_fixture": parity}


def config4_fixture_parity():
    """Ray counts of the reference's strict build on 8 config-4 curves x 21
    points (tests/golden/config4_sample.npz: radii 3e-4 to 2e-2, 200 to 1000
    rays per radius) against the engine's (exact chain), reported rather
    than asserted."""
    from triplelens_gb300.batch import Batch
    try:
        z = np.load(os.path.join(ROOT, "tests", "golden", "config4_sample.npz"))
        n, lenses, trajs = int(z["n"]), z["lenses"], z["trajs"]
        b = Batch()
        b.set_chain(0)
        b.set_lenses(lenses)
        _, cnt, st = b.run(trajs, np.arange(len(trajs)), n)
        ref = z["counts_strict"].ravel()
        return {"points": int(len(ref)), "mismatches": int(np.sum(cnt != ref)),
                "incomplete_points": int(((st & 0xC) != 0).sum()),
                "fixture": "tests/golden/config4_sample.npz (the reference's strict build)"}
    except Exception as e:   # reported, never fatal to the leg
        return {"error": repr(e)[:300]}


def surrogate_leg(seed, train_lenses, eval_lenses):
    """Finite-source surrogate: train on GPU-IRS labels, then time the plain
    IRS and the gated path on the same fresh queries (host buffers; the lens
    set-up both share is outside the timing)."""
    import torch
    from triplelens_gb300 import surrogate as S
    t_start = time.perf_counter()

    def log(what):
        print("[bench surrogate %.1fs] %s" % (time.perf_counter() - t_start, what),
              file=sys.stderr, flush=True)

    with quiet_stdout():
        model, tinfo = S.fit(seed + 7, train_lenses, 64)
        log("trained: %s" % tinfo)
        q = S.QuerySet(*S.sample_config5(seed + 8, eval_lenses, 64))
        n_drawn = q.n
        q.restrict()
        q.irs_points(torch.arange(min(q.n, 4096), device=q.dev))   # warm-up
        torch.cuda.synchronize()
        log("queries %d of %d" % (q.n, n_drawn))
        t0 = time.perf_counter()
        truth, st = q.label()
        t_irs = time.perf_counter() - t0
        log("plain IRS %.2fs" % t_irs)
        S.evaluate(model, q)                                        # warm-up
        mag, gated, tm = S.evaluate(model, q)
        log("gated %s" % tm)
    ok = (truth > 0) & ((st & 0x2f) == 0)
    err = np.abs(mag[ok] / truth[ok] - 1.0)
    aps = q.aps.cpu().numpy()
    dc = q.dc.cpu().numpy()
    # the method without the network at the same error target: A_point beyond
    # 5 source radii of the caustic, IRS within
    ps_gate = dc < 5.0
    err_ps = np.abs(np.where(ps_gate, truth, aps)[ok] / truth[ok] - 1.0)
    return {
        "queries": int(q.n), "queries_drawn": int(n_drawn),
        "train_points": tinfo["train_points"],
        "label_s": round(tinfo["label_s"], 2), "train_s": round(tinfo["train_s"], 2),
        "train_steps": tinfo["steps"],
        "plain_irs_points_per_s": q.n / t_irs,
        "gated_points_per_s": q.n / tm["total_s"],
        "speedup_vs_plain_irs": t_irs / tm["total_s"],
        "fallback_fraction": len(gated) / q.n,
        "median_rel_err": float(np.median(err)), "p99_rel_err": float(np.percentile(err, 99)),
        "plain_irs_status_counts": {"table_full": int(((st & 4) != 0).sum()),
                                    "timeout": int(((st & 8) != 0).sum()),
                                    "edge": int(((st & 2) != 0).sum()),
                                    "image_count": int(((st & 16) != 0).sum())},
        "gated_time_s": {k: round(v, 4) for k, v in tm.items()},
        "gate": S.GATE,
        "point_source_only": {"fallback_fraction": float(ps_gate.mean()),
                              "median_rel_err": float(np.median(err_ps)),
                              "p99_rel_err": float(np.percentile(err_ps, 99))},
        "workload": "lenses as config 2, rho log-uniform [1e-4, 3e-2], v uniform [0.3, 0.7], "
                    "500 rays/radius; queries: caustic sample + offset uniform in a 3 theta_E "
                    "disc; training sources 2-300 rho from a caustic; queries with A_point > "
                    "300 (sources within ~rho of a cusp at small rho) left out of both arms",
    }


def noalloc_leg(lens, traj, n, reps=3):
    """lcirs_fill_device_noalloc (static 80 MiB scratch, 8 fill CTAs) on one
    curve's points, with the seeds of the object's own get_lc_irs; counts are
    compared with that run."""
    import ctypes
    import torch
    from triplelens_gb300.lcirs import LC_irs, load_lcirs
    L = load_lcirs()
    fn = L.lcirs_fill_device_noalloc
    vp = ctypes.c_void_p
    fn.argtypes = [vp, ctypes.c_int, vp, vp, vp, vp, vp, vp, vp]
    fn.restype = ctypes.c_int
    with quiet_stdout():
        lc = LC_irs(*lens[:5], lens[5], n, int(lens[7]))
        lc.set_verbose(0)
        lc.set_limb_darkening("linear", lens[6])
        lc.get_lc_irs(*traj)
    seeds, nseeds = lc.seeds()
    t = np.arange(n + 1, dtype=np.float64) / float(n)
    xy = np.stack([traj[0] + (traj[2] - traj[0]) * t, traj[1] + (traj[3] - traj[1]) * t], 1)
    dev = torch.device("cuda")
    d_xy = torch.from_numpy(xy).to(dev)
    d_seeds = torch.from_numpy(np.ascontiguousarray(seeds, np.int32)).to(dev)
    d_ns = torch.from_numpy(np.ascontiguousarray(nseeds, np.int32)).to(dev)
    d_mag = torch.zeros(n + 1, dtype=torch.float64, device=dev)
    d_cnt = torch.zeros(n + 1, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream()
    args = (vp(lc.obj), n + 1, d_xy.data_ptr(), d_seeds.data_ptr(), d_ns.data_ptr(),
            d_mag.data_ptr(), d_cnt.data_ptr(), None, vp(stream.cuda_stream))
    assert fn(*args) == 0
    torch.cuda.synchronize()
    ms = []
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn(*args)
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    cnt = d_cnt.cpu().numpy().view(np.uint64)
    return {"points": n + 1, "ms_per_call": float(np.median(ms)),
            "points_per_s": (n + 1) / (float(np.median(ms)) / 1e3),
            "counts_equal_get_lc_irs": bool(np.array_equal(cnt, lc.counts())),
            "path": "lcirs_fill_device_noalloc, device arrays, static scratch (8 fill CTAs)"}


_T0 = time.perf_counter()


def leg(what):
    """Progress of the bench's legs on stderr (the JSON line stays alone on
    stdout)."""
    print("[bench %.1fs] %s" % (time.perf_counter() - _T0, what), file=sys.stderr, flush=True)


def child_leg(argv, timeout):
    """Runs one leg (`bench.py --leg ...`) in a child process on the same GPU
    and returns its JSON object; a leg that does not finish within `timeout`
    seconds is killed and reported as such, so the headline line is always
    printed."""
    cmd = [sys.executable, os.path.abspath(__file__)] + argv
    try:
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=None, timeout=timeout,
                           text=True)
    except subprocess.TimeoutExpired:
        return {"unavailable": "did not finish within %d s (child killed)" % timeout}
    if r.returncode != 0:
        return {"unavailable": "exited with status %d" % r.returncode}
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    if not lines:
        return {"unavailable": "printed no result"}
    return json.loads(lines[-1])


def rank_seed(seed, rank):
    """Weak scaling: every rank draws its own curves (independent objects,
    no data-path collective)."""
    return seed + 1000 * rank


def max_over_ranks(value, dist, device):
    """The slowest rank's step time (the only collective of the bench)."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def parity_vs_fixture(cnt, n, ncurves, seed, rank, ppr=500):
    """Ray counts of the benchmark's first curves against the reference's own
    counts for them (tests/golden/bench_seed2024.npz, strict IEEE build of
    the reference, 8 curves of seed 2024)."""
    path = os.path.join(ROOT, "tests", "golden", "bench_seed2024.npz")
    if rank != 0 or seed != 2024 or ppr != 500 or not os.path.exists(path):
        return None
    z = np.load(path)
    if int(z["n"]) != n:
        return None
    k = min(ncurves, len(z["counts"]))
    ref = z["counts"][:k].ravel()
    got = cnt[:k * (n + 1)]
    return {"points": int(len(ref)), "mismatches": int(np.sum(got != ref)),
            "reference": "ray counts of the reference's own IRS (strict IEEE build), "
                         "first %d curves" % k}


def status_counts(st):
    return {"table_full": int(((st & 4) != 0).sum()), "timeout": int(((st & 8) != 0).sum()),
            "edge": int(((st & 2) != 0).sum()), "image_count": int(((st & 16) != 0).sum()),
            "seed_overflow": int(((st & 1) != 0).sum())}


def e2e_objects(lenses, trajs, n, chain, threads):
    """The reference-facing C ABI (lcirs_new / set_limb_darkening /
    get_lc_irs / copy_lc) with host buffers, one object per curve, the curves
    driven from a pool of host threads as independent objects (their seeds
    run concurrently; their fills take turns).  Returns (seconds, outputs)."""
    from concurrent.futures import ThreadPoolExecutor
    from triplelens_gb300.lcirs import LC_irs
    outs = np.zeros((len(lenses), n))

    def one(k):
        L = lenses[k]
        lc = LC_irs(*L[:5], L[5], n, int(L[7]))
        lc.set_verbose(0)
        lc.set_chain(chain)
        lc.set_limb_darkening("linear", L[6])
        lc.get_lc_irs(*trajs[k])
        lc.copy_lc(outs[k])
        return lc

    with ThreadPoolExecutor(max_workers=threads) as ex:
        t0 = time.perf_counter()
        objs = list(ex.map(one, range(len(lenses))))
        t = time.perf_counter() - t0
    del objs
    return t, outs


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--curves", type=int, default=152, help="light curves per step per GPU")
    ap.add_argument("--points", type=int, default=5000)
    ap.add_argument("--ppr", type=int, default=500, help="rays per source radius")
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--chain", type=int, default=0,
                    help="warm-start chain: 0 = one per curve (the reference's, exact), "
                         "k > 0 = restart every k points")
    ap.add_argument("--cpu-sample", type=int, default=608,
                    help="points timed on the CPU (spread over the curves)")
    ap.add_argument("--e2e-threads", type=int, default=0,
                    help="host threads of the e2e leg (0: one per curve)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fast", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-surrogate", action="store_true")
    ap.add_argument("--no-config4", action="store_true")
    ap.add_argument("--no-noalloc", action="store_true")
    ap.add_argument("--no-pipeline", action="store_true",
                    help="exact chain: seeds then fill, not overlapped")
    ap.add_argument("--leg", choices=["config4", "surrogate"], default=None,
                    help="run one side leg alone and print its JSON object")
    ap.add_argument("--leg-timeout", type=int, default=300,
                    help="seconds allowed to each side leg run as a child process")
    ap.add_argument("--c4-curves", type=int, default=64,
                    help="config-4 sub-sample: curves of 2000 points, each its own lens")
    ap.add_argument("--sur-train-lenses", type=int, default=1024,
                    help="surrogate training lenses (64 sources each)")
    ap.add_argument("--sur-eval-lenses", type=int, default=16384,
                    help="surrogate evaluation lenses (64 queries each)")
    args = ap.parse_args()
    # a step that stalls shows where: every thread's Python stack on stderr
    # every 240 s (stdout keeps the one JSON line)
    import faulthandler
    faulthandler.dump_traceback_later(240, repeat=True, file=sys.stderr)

    if args.leg is not None:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        if args.leg == "config4":
            out = config4_leg(args.seed, args.c4_curves, args.steps)
        else:
            out = surrogate_leg(args.seed, args.sur_train_lenses, args.sur_eval_lenses)
        print(json.dumps(out))
        return

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    from triplelens_gb300 import workloads
    # weak scaling: every rank its own curves
    lenses, trajs, n = workloads.config2(rank_seed(args.seed, rank), n_curves=args.curves,
                                        n_points=args.points, ppr=args.ppr)
    chain_desc = ("one warm-start chain per curve (the reference's order)" if args.chain <= 0
                  else "warm-start chain restarted every %d points" % args.chain)
    config = {"workload": "config2: %d random triple lenses x %d-point curves, rho=1e-3, "
                          "%d rays/radius, linear LD v=0.5" % (args.curves, n, args.ppr),
              "curves_per_gpu": args.curves, "points_per_curve": n + 1, "rho": 1e-3,
              "rays_per_radius": args.ppr, "ld_v": 0.5, "seed": args.seed, "chain": chain_desc,
              "l2": "flushed between steps (256 MiB write)",
              "overlap": ("exact chain in 8 segments, each segment's fill overlapped with the "
                          "next segment's chain" if args.chain <= 0 else "none"),
              "parallelism": "curves sharded over %d GPU(s)" % world}
    ncpu = os.cpu_count() or 1

    if args.impl == "reference":
        if rank != 0:
            return
        import multiprocessing as mp
        pool = mp.get_context("spawn").Pool(ncpu)
        vals = []
        for step in range(args.warmup + args.steps):
            pts_s, pts_s1, rays_s, desc, busy = cpu_baseline(pool, ncpu, lenses, trajs, n,
                                                             args.cpu_sample)
            if step >= args.warmup:
                vals.append(pts_s)
        pool.close()
        v = float(np.mean(vals))
        line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": config, "impl": "reference",
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": ncpu, "kind": "port",
                                 "sample": desc + " per step"},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0},
                "note": "the reference's CPU IRS compiles only for x86 (lcirs.cc uses AVX "
                        "intrinsics) and its sources are not on this host; its C restatement "
                        "(oracle/), which reproduces its strict IEEE build bit for bit, is timed"}
        print(json.dumps(line))
        return

    # CPU pool before any GPU work (spawned workers)
    pool = None
    if rank == 0 and not args.no_cpu:
        import multiprocessing as mp
        pool = mp.get_context("spawn").Pool(ncpu)

    import torch
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    from triplelens_gb300.batch import Batch

    b = Batch()
    b.set_chain(args.chain)
    b.set_lenses(lenses)
    npts = b.set_trajectories(trajs, np.arange(len(trajs)), np.full(len(trajs), n))
    # a dedicated stream: the library launches on it and the events are
    # recorded on it (the legacy default stream does not order against the
    # library's non-blocking stream)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sptr = stream.cuda_stream
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def step_device(bb):
        bb.run_device(1, sptr)
        e1 = torch.cuda.Event(enable_timing=True)
        e1.record(stream)
        bb.run_device(2, sptr)
        return e1

    # the exact chain runs in segments overlapped with the fill (one call);
    # the seeds/fill split for the roofline comes from a sequential step
    pipelined = args.chain <= 0 and not args.no_pipeline

    def step_timed(bb):
        if pipelined:
            bb.run_device(4, sptr)
            return None
        return step_device(bb)

    leg("inputs set: %d points" % npts)
    for _ in range(args.warmup):
        step_timed(b)
    torch.cuda.synchronize()
    leg("warm-up steps")
    amp, cnt, st = b.download(sptr)
    stats = b.stats()

    tot_ms = 0.0
    fill_ms = 0.0
    # raw nvidia-smi samples (TL_CLOCKS_DIR, default the temp directory)
    import tempfile
    clock_path = os.path.join(os.environ.get("TL_CLOCKS_DIR", tempfile.gettempdir()),
                              "bench_clocks_r%d.csv" % rank)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(clock_path) as clk:
        time.sleep(0.3)
        for _ in range(args.steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e2 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            e1 = step_timed(b)
            e2.record(stream)
            e2.synchronize()
            tot_ms += e0.elapsed_time(e2)
            if e1 is not None:
                fill_ms += e1.elapsed_time(e2)
        time.sleep(0.3)
    torch.cuda.synchronize()
    seq_ms = None
    if pipelined:
        # one sequential step (seeds, then fill) for the seeds/fill split
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e2 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        e1 = step_device(b)
        e2.record(stream)
        e2.synchronize()
        seq_ms = e0.elapsed_time(e2)
        fill_ms = e1.elapsed_time(e2) * args.steps
        amp_seq, cnt_seq, _ = b.download(sptr)
    if dist:
        tot_ms = max_over_ranks(tot_ms, dist, "cuda")
        dist.barrier()
    ms_step = tot_ms / args.steps
    value = npts * world / (ms_step / 1e3)
    leg("timed steps: %.1f ms per step" % ms_step)
    incomplete = int(np.sum((st & 0xC) != 0))

    # the same workload with chunked warm-start chains (parallel seeds)
    fast = None
    if not args.no_fast and args.chain <= 0:
        bf = Batch()
        bf.set_chain(4)
        bf.set_lenses(lenses)
        bf.set_trajectories(trajs, np.arange(len(trajs)), np.full(len(trajs), n))
        step_device(bf)
        torch.cuda.synchronize()
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e2 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        e1 = step_device(bf)
        e2.record(stream)
        e2.synchronize()
        _, fcnt, _ = bf.download(sptr)
        fast = {"chain": "restarted every 4 points", "ms_per_step": e0.elapsed_time(e2),
                "seeds_ms": e0.elapsed_time(e1),
                "points_per_s": npts / (e0.elapsed_time(e2) / 1e3),
                "count_mismatches_vs_exact": int(np.sum(fcnt != cnt)),
                "parity": parity_vs_fixture(fcnt, n, len(lenses), args.seed, rank, args.ppr)}
        del bf
        leg("chunked-chain leg")

    e2e = None
    if not args.no_e2e:
        threads = len(lenses) if args.e2e_threads <= 0 else min(len(lenses), args.e2e_threads)
        with quiet_stdout():
            e2e_objects(lenses, trajs, n, args.chain, threads)          # warm-up pass
            torch.cuda.synchronize()
            from triplelens_gb300.lcirs import transfer_bytes
            x0 = transfer_bytes()
            t_e2e, outs = e2e_objects(lenses, trajs, n, args.chain, threads)
            x1 = transfer_bytes()
        ref_amp = amp.reshape(len(lenses), n + 1)[:, :n]
        rel = float(np.max(np.abs(outs - ref_amp) / ref_amp))
        # bytes across the host boundary per step, as the library counts its
        # own copies (parameters, jobs and point lists in; per-point results
        # and seeds out); the caller's own buffers hold the parameters and
        # the n magnifications per curve
        e2e = {"value": npts * world / t_e2e, "unit": UNIT,
               "h2d_bytes_per_step": x1[0] - x0[0],
               "d2h_bytes_per_step": x1[1] - x0[1],
               "caller_bytes_per_step": {"in": len(lenses) * (8 * 8 + 4 * 8),
                                         "out": len(lenses) * n * 8},
               "path": "lcirs_new/set_limb_darkening/get_lc_irs/copy_lc per curve (reference C "
                       "ABI), %d host threads, lens set-up included" % threads,
               "max_rel_diff_vs_device_run": rel}
        # the batched C ABI from host buffers (tl_batch.h: one call per batch)
        bh = Batch()
        bh.set_chain(args.chain)
        ampb = np.zeros(npts)
        cntb = np.zeros(npts, np.uint64)
        stb = np.zeros(npts, np.uint32)
        for it in range(2):
            x0 = transfer_bytes()
            t0 = time.perf_counter()
            bh.set_lenses(lenses)
            bh.run_host(trajs, np.arange(len(trajs)), np.full(len(trajs), n), ampb, cntb, stb)
            t_b = time.perf_counter() - t0
            x1 = transfer_bytes()
        e2e["batch_api"] = {"value": npts * world / t_b, "unit": UNIT,
                            "h2d_bytes_per_step": x1[0] - x0[0],
                            "d2h_bytes_per_step": x1[1] - x0[1],
                            "path": "tlb_set_lenses + tlb_run_host (host buffers in and out)",
                            "counts_equal_device_run": bool(np.array_equal(cntb, cnt))}
        del bh
        leg("e2e legs")

    peaks = measured_peaks()
    clocks = clk.summary(local_rank)
    sm_max = peaks.get("sm_max_mhz") or clocks.get("sm_max_mhz") or 2070.0
    peak_tf, sms = fp32_peak_tflops(sm_max)
    fill_s = fill_ms / args.steps / 1e3
    flops = FLOP_PER_RAY * float(stats[0]) + FLOP_PER_WEIGHT * float(stats[3])
    achieved = flops / fill_s / 1e12
    traffic = None
    tr_path = os.path.join(ROOT, "profiles", "fill_traffic.json")
    if os.path.exists(tr_path):
        with open(tr_path) as f:
            tr = json.load(f)
        # scale the captured per-ray traffic to this launch
        traffic = tr.get("bytes_per_evaluated_ray", 0.0) * float(stats[0])

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded random lenses and trajectories)", "config": config,
        "e2e": e2e,
        "parity": parity_vs_fixture(cnt, n, len(lenses), args.seed, rank, args.ppr),
        "incomplete_points": incomplete,
        "status_counts": status_counts(st),
        "seeds_ms_per_step": (seq_ms if pipelined else ms_step) - fill_ms / args.steps,
        "pipeline": ({"segments": 8, "sequential_ms_per_step": seq_ms,
                      "counts_equal_sequential": bool(np.array_equal(cnt, cnt_seq))}
                     if pipelined else None),
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak_tf, "unit": "TFLOP/s",
                     "frac": achieved / peak_tf, "traffic": traffic,
                     "kernel": "wfill_kernel (+ fill_kernel for points above its table)",
                     "flop_per_ray": FLOP_PER_RAY, "flop_per_accepted_ray": FLOP_PER_WEIGHT,
                     "peak_source": "2 x 128 FP32 lanes x %d SMs x sm_max_mhz %.0f (MEASURED_PEAKS)"
                                    % (sms, sm_max),
                     "fill_ms_per_step": fill_ms / args.steps,
                     "hbm_view": hbm_view(traffic, fill_s, peaks),
                     "mufu_view": mufu_view(stats[0], fill_s, sm_max, sms)},
        "rays": {"accepted_per_step": int(stats[3]), "evaluated_per_step": int(stats[0]),
                 "fp64_per_step": int(stats[1]), "tiles_per_step": int(stats[2]),
                 "accepted_per_s": float(stats[3]) * world / (ms_step / 1e3),
                 "status_or": int(np.bitwise_or.reduce(st))},
        "fast_chain": fast,
        "clocks": clocks,
        # per overlapped step: caustic scan, point prep, chain reset, 8 chain
        # segments with 8 warp fills, the team fill and two CTA-fill levels
        # (collect + fill each) = 25; per sequential step: scan, prep and chain
        # (or scan and chunked seeds), 3 ordering kernels, the warp fill, the
        # team fill and two CTA levels (collect + fill each) = 13 (12)
        "gpu_launches": (25 if pipelined else (13 if args.chain <= 0 else 12)) * args.steps,
    }
    if rank == 0 and not args.no_noalloc:
        line["noalloc"] = noalloc_leg(lenses[0], trajs[0], n)
        leg("noalloc leg")
    if rank == 0 and not args.no_config4:
        line["config4"] = child_leg(["--leg", "config4", "--seed", str(args.seed),
                                     "--c4-curves", str(args.c4_curves),
                                     "--steps", str(max(1, min(args.steps, 3)))],
                                    args.leg_timeout)
        leg("config4 leg")
    if rank == 0 and not args.no_surrogate:
        line["surrogate"] = child_leg(["--leg", "surrogate", "--seed", str(args.seed),
                                       "--sur-train-lenses", str(args.sur_train_lenses),
                                       "--sur-eval-lenses", str(args.sur_eval_lenses)],
                                      args.leg_timeout)
        leg("surrogate leg")
    if pool is not None and rank == 0:
        pts_s, pts_s1, rays_s, desc, busy = cpu_baseline(pool, ncpu, lenses, trajs, n,
                                                         args.cpu_sample)
        line["cpu_baseline"] = {"value": pts_s, "unit": UNIT, "cores": ncpu, "kind": "port",
                                "sample": desc, "value_1core": pts_s1, "rays_per_s": rays_s}
        pool.close()
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
