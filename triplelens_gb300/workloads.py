"""Seeded synthetic workloads for the extended-source light-curve path.

No public dataset is involved: every input is drawn from a seed.

config1  the CPU-runnable case: masses (0.7, 0.2, 0.1), z1 = 0, z2 = (1, 0),
         z3 = (0.5, 0.8); straight trajectory of 4 theta_E at 30 degrees with
         impact parameter 0.1 about the origin, 100 points; rho = 0.01,
         100 rays per source radius, uniform source (linear LD with v = 0).
config2  random triple lenses: mass ratios log-uniform in [1e-3, 1] (masses
         proportional to (1, q2, q3)), separations a, b log-uniform in
         [0.5, 2], angle uniform; trajectory angle uniform, impact parameter
         uniform in [-0.5, 0.5], 4 theta_E, 5000 points; rho = 1e-3,
         500 rays per radius, linear limb darkening v = 0.5.
config3  config2 lenses resampled until the trajectory crosses a caustic
         (the caustics come from libccc.so).
config4  many curves, each its own config2 lens, rho log-uniform in
         [1e-4, 3e-2], rays per radius in {200, 500, 1000}, v in [0.3, 0.7].

Lens rows are (a, b, th, m2, m3, rho, ld_v, ppr) - the layout of
tl_batch.h; trajectory rows are (x0, y0, x1, y1).
"""
import math

import numpy as np


def config1():
    a, b, th = 1.0, math.sqrt(0.5 ** 2 + 0.8 ** 2), math.atan2(0.8, 0.5)
    ang = math.radians(30.0)
    c = np.array([-0.1 * math.sin(ang), 0.1 * math.cos(ang)])
    d = np.array([math.cos(ang), math.sin(ang)])
    s, e = c - 2 * d, c + 2 * d
    lens = np.array([a, b, th, 0.2, 0.1, 0.01, 0.0, 100.0])
    traj = np.array([s[0], s[1], e[0], e[1]])
    return lens, traj, 100


def _random_lens(rng):
    q2 = 10.0 ** rng.uniform(-3.0, 0.0)
    q3 = 10.0 ** rng.uniform(-3.0, 0.0)
    tot = 1.0 + q2 + q3
    m2, m3 = q2 / tot, q3 / tot
    a = 10.0 ** rng.uniform(math.log10(0.5), math.log10(2.0))
    b = 10.0 ** rng.uniform(math.log10(0.5), math.log10(2.0))
    th = rng.uniform(0.0, 2.0 * math.pi)
    return a, b, th, m2, m3


def _random_traj(rng, length=4.0):
    alpha = rng.uniform(0.0, 2.0 * math.pi)
    u0 = rng.uniform(-0.5, 0.5)
    c = u0 * np.array([-math.sin(alpha), math.cos(alpha)])
    d = np.array([math.cos(alpha), math.sin(alpha)])
    s, e = c - 0.5 * length * d, c + 0.5 * length * d
    return np.array([s[0], s[1], e[0], e[1]])


def config2(seed, n_curves=1, n_points=5000, rho=1e-3, ppr=500, ld_v=0.5):
    """n_curves random lenses, one trajectory each."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lenses, trajs = [], []
    for _ in range(n_curves):
        a, b, th, m2, m3 = _random_lens(rng)
        lenses.append([a, b, th, m2, m3, rho, ld_v, float(ppr)])
        trajs.append(_random_traj(rng))
    return np.array(lenses), np.array(trajs), n_points


def crossings(traj, ca):
    """Parameters t in [0, 1] (sorted) at which the trajectory x0,y0 -> x1,y1
    crosses the caustic polylines ca (branches, samples; complex, closed)."""
    ca = np.asarray(ca)
    p0, p1 = np.asarray(traj[:2]), np.asarray(traj[2:])
    q = np.stack([ca.real, ca.imag], axis=-1)
    q0 = q.reshape(-1, 2)
    q1 = np.roll(q, -1, axis=1).reshape(-1, 2)
    d = p1 - p0
    e = q1 - q0
    den = d[0] * e[:, 1] - d[1] * e[:, 0]
    w = q0 - p0
    with np.errstate(divide="ignore", invalid="ignore"):
        t = (w[:, 0] * e[:, 1] - w[:, 1] * e[:, 0]) / den
        u = (w[:, 0] * d[1] - w[:, 1] * d[0]) / den
    hit = (den != 0) & (t >= 0) & (t <= 1) & (u >= 0) & (u <= 1)
    return np.sort(t[hit])


def config3(seed, caustics, n_curves=1, n_points=5000, rho=1e-3, ppr=500, ld_v=0.5):
    """config2 lenses and trajectories, resampled until the trajectory crosses
    a caustic branch.  caustics(a, b, th, m2, m3) returns the caustic samples
    as an array (branches, samples) of complex numbers (e.g. from libccc.so)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lenses, trajs = [], []
    while len(lenses) < n_curves:
        a, b, th, m2, m3 = _random_lens(rng)
        traj = _random_traj(rng)
        if len(crossings(traj, caustics(a, b, th, m2, m3))):
            lenses.append([a, b, th, m2, m3, rho, ld_v, float(ppr)])
            trajs.append(traj)
    return np.array(lenses), np.array(trajs), n_points


def config4(seed, n_curves=4096, n_points=2000):
    rng = np.random.Generator(np.random.PCG64(seed))
    lenses, trajs = [], []
    for _ in range(n_curves):
        a, b, th, m2, m3 = _random_lens(rng)
        rho = 10.0 ** rng.uniform(-4.0, math.log10(3e-2))
        ppr = float(rng.choice([200, 500, 1000]))
        v = rng.uniform(0.3, 0.7)
        lenses.append([a, b, th, m2, m3, rho, v, ppr])
        trajs.append(_random_traj(rng))
    return np.array(lenses), np.array(trajs), n_points
