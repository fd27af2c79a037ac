"""The seeded workloads (triplelens_gb300/workloads.py) against their
specification, without a GPU: config 1's pinned lens and trajectory, the
distributions of config 2 (the bench workload) and config 4, seeded
determinism, and the caustic-crossing test config 3 resamples with."""
import math

import numpy as np

from triplelens_gb300 import workloads


def test_config1_is_the_pinned_case():
    """Masses (0.7, 0.2, 0.1), z2 = (1, 0), z3 = (0.5, 0.8); 4 theta_E at 30
    degrees whose closest approach to the origin (z1) is 0.1; rho = 0.01,
    100 rays per radius, uniform source, 100 points."""
    lens, traj, n = workloads.config1()
    a, b, th, m2, m3, rho, v, ppr = lens
    assert (a, m2, m3, rho, v, ppr, n) == (1.0, 0.2, 0.1, 0.01, 0.0, 100.0, 100)
    assert abs(b * math.cos(th) - 0.5) < 1e-15 and abs(b * math.sin(th) - 0.8) < 1e-15
    p0, p1 = traj[:2], traj[2:]
    d = p1 - p0
    assert abs(np.hypot(*d) - 4.0) < 1e-14
    assert abs(math.atan2(d[1], d[0]) - math.radians(30.0)) < 1e-14
    # closest approach: the midpoint, at distance 0.1, on the left of the motion
    mid = 0.5 * (p0 + p1)
    assert abs(np.hypot(*mid) - 0.1) < 1e-15 and abs(mid @ d) < 1e-14
    assert d[0] * mid[1] - d[1] * mid[0] > 0


def _check_lenses(lenses):
    a, b, th, m2, m3 = lenses[:, :5].T
    m1 = 1.0 - m2 - m3
    for q in (m2 / m1, m3 / m1):          # mass ratios log-uniform in [1e-3, 1]
        assert q.min() >= 1e-3 * (1 - 1e-12) and q.max() <= 1.0 + 1e-12
        lq = np.log10(q)
        assert abs(lq.mean() + 1.5) < 0.1 and abs(lq.std() - 3 / math.sqrt(12)) < 0.1
    for s in (a, b):                      # separations log-uniform in [0.5, 2]
        assert s.min() >= 0.5 and s.max() <= 2.0
        assert abs(np.log10(s).mean()) < 0.03
    assert th.min() >= 0.0 and th.max() < 2 * math.pi and abs(th.mean() - math.pi) < 0.15


def _check_trajs(trajs):
    p0, p1 = trajs[:, :2], trajs[:, 2:]
    d = p1 - p0
    assert np.allclose(np.hypot(d[:, 0], d[:, 1]), 4.0, rtol=0, atol=1e-12)
    # impact parameter about the origin, uniform in [-0.5, 0.5]
    u0 = (d[:, 0] * p0[:, 1] - d[:, 1] * p0[:, 0]) / 4.0
    assert np.abs(u0).max() <= 0.5 + 1e-12 and abs(u0.mean()) < 0.03
    mid = 0.5 * (p0 + p1)
    assert np.allclose(np.hypot(mid[:, 0], mid[:, 1]), np.abs(u0), atol=1e-12)


def test_config2_distributions_and_determinism():
    lenses, trajs, n = workloads.config2(2024, n_curves=2000)
    assert n == 5000 and lenses.shape == (2000, 8) and trajs.shape == (2000, 4)
    assert np.all(lenses[:, 5] == 1e-3) and np.all(lenses[:, 6] == 0.5)
    assert np.all(lenses[:, 7] == 500.0)
    _check_lenses(lenses)
    _check_trajs(trajs)
    # the same seed gives the same curves; the first curves of a larger draw
    # are the curves of a smaller one (the bench's fixture relies on both)
    l2, t2, _ = workloads.config2(2024, n_curves=8)
    assert np.array_equal(l2, lenses[:8]) and np.array_equal(t2, trajs[:8])
    l3, _, _ = workloads.config2(2025, n_curves=8)
    assert not np.array_equal(l3, l2)


def test_config4_distributions():
    lenses, trajs, n = workloads.config4(7, n_curves=3000)
    assert n == 2000
    _check_lenses(lenses)
    _check_trajs(trajs)
    rho = lenses[:, 5]
    assert rho.min() >= 1e-4 and rho.max() <= 3e-2
    lr = np.log10(rho)
    assert abs(lr.mean() - 0.5 * (-4.0 + math.log10(3e-2))) < 0.05
    assert set(np.unique(lenses[:, 7])) == {200.0, 500.0, 1000.0}
    v = lenses[:, 6]
    assert v.min() >= 0.3 and v.max() <= 0.7 and abs(v.mean() - 0.5) < 0.01


def test_crossings_of_a_polyline():
    # a closed square of side 2 around the origin, 4 samples per side
    side = np.linspace(-1.0, 1.0, 5)[:-1]
    sq = np.concatenate([side - 1j, 1 + 1j * side, -side + 1j, -1 - 1j * side])[None, :]
    t = workloads.crossings(np.array([-3.0, 0.1, 3.0, 0.1]), sq)
    assert np.allclose(t, [1.0 / 3.0, 2.0 / 3.0])
    assert len(workloads.crossings(np.array([-3.0, 2.0, 3.0, 2.0]), sq)) == 0
    # ends inside: one crossing
    t = workloads.crossings(np.array([0.0, 0.0, 4.0, 0.0]), sq)
    assert np.allclose(t, [0.25])
