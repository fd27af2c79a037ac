"""Library-level sharding of curves over ranks (triplelens_gb300/shard.py)
without a GPU: the plan covers every curve once and balances predicted rays;
two gloo ranks predict their strided costs, agree on the plan, run only their
own curves and gather results equal to a one-rank run.  The engine stands
behind the predictor and runner on GPUs; here they are deterministic fakes.
"""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from triplelens_gb300 import shard  # noqa: E402


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_plan_covers_every_curve_once_and_balances(world):
    rng = np.random.default_rng(world)
    # heavy-tailed costs, as magnifications near caustics make them
    costs = rng.pareto(1.5, size=500) * 1e7 + 1e6
    shares = shard.plan(costs, world)
    allidx = np.sort(np.concatenate(shares))
    assert np.array_equal(allidx, np.arange(len(costs)))
    ld = shard.loads(costs, shares)
    lower = max(costs.sum() / world, costs.max())
    assert ld.max() <= 4.0 / 3.0 * lower + 1e-6 * lower


def test_plan_is_deterministic_and_rejects_bad_costs():
    costs = [5.0, 5.0, 3.0, 3.0, 1.0]
    a = shard.plan(costs, 2)
    b = shard.plan(list(costs), 2)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    assert [x.tolist() for x in a] == [[0, 2, 4], [1, 3]]
    with pytest.raises(ValueError):
        shard.plan([1.0, -1.0], 2)
    with pytest.raises(ValueError):
        shard.plan([1.0, float("nan")], 2)
    with pytest.raises(ValueError):
        shard.plan([1.0], 0)


def test_plan_with_more_ranks_than_curves_and_zero_costs():
    """Ranks beyond the number of curves get empty shares (ShardedCurves
    skips their predictor and runner calls); zero-cost curves are still
    assigned, and every curve exactly once."""
    shares = shard.plan([3.0, 0.0, 1.0], 8)
    assert len(shares) == 8
    assert sorted(np.concatenate(shares).tolist()) == [0, 1, 2]
    assert sum(len(s) == 0 for s in shares) == 5
    shares = shard.plan(np.zeros(10), 3)
    assert sorted(np.concatenate(shares).tolist()) == list(range(10))
    assert [len(s) for s in shares] == [4, 3, 3]
    assert shard.plan([], 2)[0].size == 0


def test_predicted_rays_from_point_magnifications():
    lenses = np.array([[1, 1, 0, 0.1, 0.1, 1e-3, 0.5, 500.0],
                       [1, 1, 0, 0.1, 0.1, 1e-3, 0.5, 100.0]])
    n = np.array([3, 2])
    amps = np.array([1.0, 2.0, 3.0, 10.0, 10.0])
    r = shard.predicted_rays(lenses, np.array([0, 1]), n, amps)
    assert np.allclose(r, [6.0 * np.pi * 500 ** 2, 20.0 * np.pi * 100 ** 2])
    # the batched API's layout: n + 1 slots per curve, the last one unused
    slots = np.array([1.0, 2.0, 3.0, 0.0, 10.0, 10.0, 0.0])
    assert np.allclose(shard.predicted_rays(lenses, np.array([0, 1]), n, slots), r)
    with pytest.raises(ValueError):
        shard.predicted_rays(lenses, np.array([0, 1]), n, amps[:4])


def _fake_predictor(lenses, trajs, lens_idx, n):
    # deterministic, uneven: longer curves through stronger lenses cost more
    return (n + 1) * (1.0 + 10.0 * lenses[lens_idx, 3]) * (1.0 + np.abs(trajs[:, 0]))


def _fake_runner(lenses, trajs, lens_idx, n):
    amp, cnt, st = [], [], []
    for t, li, m in zip(trajs, lens_idx, n):
        x = np.linspace(t[0], t[2], int(m) + 1)
        amp.append(1.0 + lenses[li, 3] * np.cos(x))
        cnt.append((np.abs(x) * 1e6).astype(np.uint64))
        st.append(np.full(int(m) + 1, li % 3, np.uint32))
    return np.concatenate(amp), np.concatenate(cnt), np.concatenate(st)


def _job():
    rng = np.random.default_rng(7)
    lenses = np.column_stack([np.ones(5), np.ones(5), np.zeros(5), rng.uniform(0, 1, 5),
                              rng.uniform(0, 1, 5), np.full(5, 1e-3), np.full(5, 0.5),
                              np.full(5, 500.0)])
    ncurves = 23
    trajs = rng.uniform(-2, 2, (ncurves, 4))
    lens_idx = rng.integers(0, 5, ncurves)
    n = rng.integers(5, 40, ncurves)
    return lenses, trajs, lens_idx, n


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    from triplelens_gb300 import shard as sh
    dist.init_process_group("gloo", rank=rank, world_size=world)
    lenses, trajs, lens_idx, n = _job()
    ran = []

    def runner(L, T, LI, N):
        ran.append(len(T))
        return _fake_runner(L, T, LI, N)

    job = sh.ShardedCurves(lenses, trajs, lens_idx, n, predictor=_fake_predictor, runner=runner)
    res = job.run()
    amp, cnt, st = job.gather(res)
    out.put((rank, job.world, [s.tolist() for s in job.shares], res[0].tolist(), sum(ran),
             amp, cnt, st))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_run_their_share_and_gather_the_whole_job():
    pytest.importorskip("torch")
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted([q.get(timeout=120) for _ in procs], key=lambda r: r[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    lenses, trajs, lens_idx, n = _job()
    # the plan both ranks computed is the one of the full cost vector
    want = shard.plan(_fake_predictor(lenses, trajs, lens_idx, n), 2)
    ramp, rcnt, rst = _fake_runner(lenses, trajs, lens_idx, n)
    for rank, world, shares, mine, nran, amp, cnt, st in res:
        assert world == 2
        assert shares == [s.tolist() for s in want]
        assert mine == want[rank].tolist()
        assert nran == len(mine)             # only this rank's curves ran here
        assert np.array_equal(amp, ramp) and np.array_equal(cnt, rcnt)
        assert np.array_equal(st, rst)
    # the predicted loads of the two ranks are within the largest curve
    costs = _fake_predictor(lenses, trajs, lens_idx, n)
    ld = shard.loads(costs, want)
    assert abs(ld[0] - ld[1]) <= costs.max()


def test_one_rank_without_a_process_group():
    lenses, trajs, lens_idx, n = _job()
    job = shard.ShardedCurves(lenses, trajs, lens_idx, n, rank=0, world=1,
                              predictor=_fake_predictor, runner=_fake_runner)
    amp, cnt, st = job.gather(job.run())
    ramp, rcnt, rst = _fake_runner(lenses, trajs, lens_idx, n)
    assert np.array_equal(amp, ramp) and np.array_equal(cnt, rcnt) and np.array_equal(st, rst)


@pytest.mark.gpu
def test_engine_predictor_and_runner_on_one_gpu(product_lib):
    """The default predictor and runner are the engine: predicted rays track
    the counts, and the sharded run equals a plain batched run."""
    from triplelens_gb300 import workloads
    from triplelens_gb300.batch import Batch
    lenses, trajs, n = workloads.config2(11, n_curves=6, n_points=200)
    idx = np.arange(len(trajs))
    nn = np.full(len(trajs), n)
    job = shard.ShardedCurves(lenses, trajs, idx, nn, rank=0, world=1)
    amp, cnt, st = job.gather(job.run())
    b = Batch()
    b.set_chain(0)
    b.set_lenses(lenses)
    ramp, rcnt, rst = b.run(trajs, idx, nn)
    assert np.array_equal(cnt, rcnt) and np.array_equal(st, rst)
    assert np.max(np.abs(amp - ramp) / ramp) < 1e-6
    per_curve = cnt.reshape(len(trajs), n + 1).sum(axis=1).astype(np.float64)
    # predicted rays (A_point * pi * ppr^2) against the accepted rays; a
    # sample next to a fold can overshoot, so the bound is loose
    ratio = job.costs / per_curve
    assert np.all((ratio > 0.5) & (ratio < 2.0)), ratio
