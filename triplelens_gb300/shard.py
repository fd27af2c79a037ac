"""Light curves sharded over ranks, balanced by predicted rays.

The reference computes one light curve per object and per process
(src/LightCurves/lcirs.cc:103-191; several curves run as independent
processes, Examples/run_asynccudalib.py).  Curves are independent, so many
of them split over GPUs with no exchange on the data path: every rank fills
the curves of its share with the engine (one process per GPU), and results
move only when the caller asks for them in one place (`gather`).

Balance.  The cost of a curve is its rays, and the rays of a point are about
A_point * pi * ppr^2 (the source disc's pixels times the point-source
magnification; the finite-source magnification differs from A_point by
< 1e-4 on the bench workload).  Costs are predicted from the point-source
magnifications (tlb_point_lc, cheap next to the fill): each rank predicts a
strided subset of the curves and the costs are all-gathered, then every rank
computes the same plan, longest-processing-time first (sorted by cost, each
curve to the rank with the least load; ties to the lower index), whose
largest load is within 4/3 of the best possible.

Everything above the engine is host logic and runs on CPU ranks (gloo) in
the tests with a fake predictor and runner; on GPUs the default predictor and
runner are the batched engine (triplelens_gb300.batch.Batch).
"""
import math

import numpy as np


def plan(costs, world):
    """Curve indices per rank: longest-processing-time first, deterministic.

    costs: per-curve predicted work (non-negative); world: number of ranks.
    Returns a list of `world` sorted index arrays covering every curve once.
    """
    costs = np.asarray(costs, dtype=np.float64)
    if world < 1:
        raise ValueError("world must be >= 1")
    if np.any(~np.isfinite(costs)) or np.any(costs < 0):
        raise ValueError("costs must be finite and non-negative")
    order = np.lexsort((np.arange(len(costs)), -costs))    # cost descending, index ascending
    loads = [0.0] * world
    shares = [[] for _ in range(world)]
    for i in order:
        # least loaded rank; on equal loads the one with fewer curves (zero
        # or equal costs then go round-robin, not all to the first rank)
        r = min(range(world), key=lambda k: (loads[k], len(shares[k]), k))
        shares[r].append(int(i))
        loads[r] += float(costs[i])
    return [np.array(sorted(s), dtype=np.int64) for s in shares]


def loads(costs, shares):
    """Predicted work per rank of a plan."""
    costs = np.asarray(costs, dtype=np.float64)
    return np.array([costs[s].sum() for s in shares])


def predicted_rays(lenses, lens_idx, n, point_amps):
    """Predicted rays per curve from point-source magnifications.

    lenses: rows (a, b, th, m2, m3, rho, ld_v, ppr); lens_idx, n: per curve;
    point_amps: the concatenated point-source magnifications, n[c] values per
    curve, either packed or in tlb_point_lc's layout (n[c] + 1 slots per
    curve, the last one unused).  Returns sum_i A_i * pi * ppr^2 per curve.
    """
    lenses = np.asarray(lenses, dtype=np.float64)
    n = np.asarray(n, dtype=np.int64)
    point_amps = np.asarray(point_amps, dtype=np.float64)
    if point_amps.size == int(n.sum()):
        slots = n
    elif point_amps.size == int((n + 1).sum()):
        slots = n + 1
    else:
        raise ValueError("point_amps holds %d values, curves need %d (or %d slots)"
                         % (point_amps.size, int(n.sum()), int((n + 1).sum())))
    base = np.concatenate([[0], np.cumsum(slots)])
    out = np.empty(len(n))
    for c in range(len(n)):
        ppr = lenses[lens_idx[c], 7]
        a = point_amps[base[c]:base[c] + n[c]]
        a = a[np.isfinite(a)]
        out[c] = float(np.sum(np.abs(a))) * math.pi * ppr * ppr
    return out


def engine_predictor(lenses, trajs, lens_idx, n):
    """Predicted rays of the given curves, from the engine's point-source
    magnifications (one GPU)."""
    from triplelens_gb300.batch import Batch
    b = Batch()
    b.set_lenses(lenses)
    b.set_trajectories(trajs, lens_idx, n)
    return predicted_rays(lenses, lens_idx, n, b.point_lc())


def engine_runner(lenses, trajs, lens_idx, n, chain=0):
    """IRS magnifications, ray counts and status words of the given curves
    (n + 1 points each, concatenated) on this rank's GPU."""
    from triplelens_gb300.batch import Batch
    b = Batch()
    b.set_chain(chain)
    b.set_lenses(lenses)
    return b.run(trajs, lens_idx, n)


class ShardedCurves:
    """Curves of one job split over the ranks of a process group.

    lenses: rows (a, b, th, m2, m3, rho, ld_v, ppr); trajs: rows (x0, y0, x1,
    y1); lens_idx, n: per curve.  rank/world default to torch.distributed's
    (1 rank without a process group).  predictor(lenses, trajs, lens_idx, n)
    -> per-curve cost and runner(lenses, trajs, lens_idx, n) -> (amp, cnt,
    st) of n + 1 points per curve default to the engine.
    """

    def __init__(self, lenses, trajs, lens_idx, n, rank=None, world=None, group=None,
                 predictor=None, runner=None):
        self.lenses = np.ascontiguousarray(lenses, np.float64)
        self.trajs = np.ascontiguousarray(trajs, np.float64)
        self.lens_idx = np.ascontiguousarray(lens_idx, np.int32)
        self.n = np.ascontiguousarray(n, np.int64)
        if not (len(self.trajs) == len(self.lens_idx) == len(self.n)):
            raise ValueError("trajs, lens_idx and n must have one entry per curve")
        self.group = group
        self.dist = None
        if rank is None or world is None:
            try:
                import torch.distributed as dist
                if dist.is_available() and dist.is_initialized():
                    self.dist = dist
                    rank = dist.get_rank(group)
                    world = dist.get_world_size(group)
            except ImportError:
                pass
        else:
            try:
                import torch.distributed as dist
                if dist.is_available() and dist.is_initialized():
                    self.dist = dist
            except ImportError:
                pass
        self.rank = 0 if rank is None else int(rank)
        self.world = 1 if world is None else int(world)
        self.predictor = predictor or engine_predictor
        self.runner = runner or engine_runner
        self.costs = None
        self.shares = None

    def _all_gather(self, obj):
        if self.world == 1 or self.dist is None:
            return [obj]
        out = [None] * self.world
        self.dist.all_gather_object(out, obj, group=self.group)
        return out

    def make_plan(self):
        """Predicts this rank's strided subset of the costs, all-gathers them,
        and computes the plan (the same on every rank)."""
        mine = np.arange(self.rank, len(self.n), self.world)
        part = (self.predictor(self.lenses, self.trajs[mine], self.lens_idx[mine], self.n[mine])
                if len(mine) else np.zeros(0))
        costs = np.zeros(len(self.n))
        for r, vals in enumerate(self._all_gather(np.asarray(part, np.float64))):
            costs[np.arange(r, len(self.n), self.world)] = vals
        self.costs = costs
        self.shares = plan(costs, self.world)
        return self.shares

    def my_curves(self):
        if self.shares is None:
            self.make_plan()
        return self.shares[self.rank]

    def run(self):
        """This rank's curves: (curve indices, amp, cnt, st), n + 1 points per
        curve concatenated in index order.  No collective."""
        idx = self.my_curves()
        if len(idx) == 0:
            return idx, np.zeros(0), np.zeros(0, np.uint64), np.zeros(0, np.uint32)
        amp, cnt, st = self.runner(self.lenses, self.trajs[idx], self.lens_idx[idx], self.n[idx])
        return idx, np.asarray(amp), np.asarray(cnt), np.asarray(st)

    def gather(self, result):
        """Every rank's `run` result -> full (amp, cnt, st) in the input's curve
        order, on every rank."""
        parts = self._all_gather(result)
        npts = self.n + 1
        base = np.concatenate([[0], np.cumsum(npts)])
        total = int(base[-1])
        amp = np.zeros(total)
        cnt = np.zeros(total, np.uint64)
        st = np.zeros(total, np.uint32)
        seen = np.zeros(len(self.n), bool)
        for idx, a, c, s in parts:
            off = 0
            for k in idx:
                m = int(npts[k])
                if seen[k]:
                    raise RuntimeError("curve %d returned by two ranks" % k)
                seen[k] = True
                amp[base[k]:base[k] + m] = a[off:off + m]
                cnt[base[k]:base[k] + m] = c[off:off + m]
                st[base[k]:base[k] + m] = s[off:off + m]
                off += m
            if off != len(a):
                raise RuntimeError("a rank returned %d points for %d expected" % (len(a), off))
        if not seen.all():
            raise RuntimeError("curves %s were not run" % np.nonzero(~seen)[0][:8].tolist())
        return amp, cnt, st
