"""Surrogate network (include/tl_surrogate.h): the library's BF16 tensor-core
forward pass and gradients against the FP64 CPU restatement (oracle/mlp.py),
and a small train-and-evaluate run showing what the trained network gains
over the method without it (A_finite = A_point)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# BF16 operands and BF16-stored activations: per-layer gradient blocks agree
# with the FP64 oracle to a few per cent in norm, and in direction to 1e-3
GRAD_REL = 5e-2
GRAD_COS = 0.998


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _blocks(g):
    from oracle import mlp
    out, o = [], 0
    for fan_in in (mlp.IN_PAD, mlp.W, mlp.W, mlp.W):
        out.append(g[o:o + mlp.W * fan_in])
        o += mlp.W * fan_in
        out.append(g[o:o + mlp.W])
        o += mlp.W
    out.append(g[o:o + mlp.W])
    out.append(g[o + mlp.W:])
    return out


def _case(seed, m=512):
    rng = np.random.default_rng(seed)
    feat = rng.normal(0.0, 1.0, (m, 14)).astype(np.float32)
    target = (0.3 * np.tanh(feat[:, 0]) - 0.2 * feat[:, 3] ** 2).astype(np.float32)
    return feat, target


def test_gradients_match_cpu_oracle(product_lib):
    torch = _torch()
    from oracle import mlp
    from triplelens_gb300 import surrogate as S
    from triplelens_gb300.lcirs import load_lcirs
    model = S.Model(members=1, seed=3, lib=load_lcirs(product_lib))
    mean, std = np.zeros(14, np.float32), np.ones(14, np.float32)
    model.set_normalisation(mean, std)
    feat, target = _case(1)
    p = model.get_params(0)
    g_gpu, loss_gpu = model.gradients(0, torch.from_numpy(feat).cuda(),
                                      torch.from_numpy(target).cuda())
    loss_cpu, _, g_cpu = mlp.forward_backward(p, feat, target, mean, std)
    assert abs(loss_gpu - loss_cpu) <= 2e-2 * loss_cpu
    for bg, bc in zip(_blocks(g_gpu.astype(np.float64)), _blocks(g_cpu)):
        if np.linalg.norm(bc) == 0.0:
            assert np.linalg.norm(bg) < 1e-6
            continue
        rel = np.linalg.norm(bg - bc) / np.linalg.norm(bc)
        cos = float(bg @ bc / (np.linalg.norm(bg) * np.linalg.norm(bc)))
        assert rel < GRAD_REL and cos > GRAD_COS, (rel, cos)


def test_forward_matches_cpu_oracle(product_lib):
    torch = _torch()
    from oracle import mlp
    from triplelens_gb300 import surrogate as S
    from triplelens_gb300.lcirs import load_lcirs
    model = S.Model(members=1, seed=5, lib=load_lcirs(product_lib))
    mean = np.linspace(-0.5, 0.5, 14).astype(np.float32)
    std = np.linspace(0.5, 2.0, 14).astype(np.float32)
    model.set_normalisation(mean, std)
    feat, target = _case(2, m=1000)
    y = torch.empty(len(feat), dtype=torch.float32, device="cuda")
    model.forward(0, torch.from_numpy(feat).cuda(), y)
    torch.cuda.synchronize()
    _, y_cpu, _ = mlp.forward_backward(model.get_params(0), feat, target, mean, std)
    y_gpu = y.cpu().numpy()
    scale = np.abs(y_cpu).max()
    assert np.max(np.abs(y_gpu - y_cpu)) < 2e-2 * scale


def test_training_step_lowers_the_loss(product_lib):
    torch = _torch()
    from triplelens_gb300 import surrogate as S
    from triplelens_gb300.lcirs import load_lcirs
    model = S.Model(members=1, seed=7, lib=load_lcirs(product_lib))
    feat, target = _case(3, m=4096)
    f, t = torch.from_numpy(feat).cuda(), torch.from_numpy(target).cuda()
    _, l0 = model.gradients(0, f, t)
    for _ in range(200):
        model.train_step(0, f, t, 2e-3)
    _, l1 = model.gradients(0, f, t)
    assert l1 < 0.2 * l0


def test_gated_surrogate_meets_error_target(product_lib):
    """Train on IRS labels of sources 2-300 source radii from a caustic, then
    evaluate the gated path on fresh lenses with the light-curve query
    distribution (caustic sample + offset in a 3 theta_E disc): the
    magnifications meet median <= 1e-3 and p99 <= 1e-2 relative error
    against the IRS while only a small fraction of the points needs the IRS
    (the method without the network runs the IRS on every point)."""
    _torch()
    from triplelens_gb300 import surrogate as S
    from triplelens_gb300.lcirs import load_lcirs
    model, _ = S.fit(11, 256, 64, members=4, epochs=30, batch=1024,
                     lib=load_lcirs(product_lib))
    te = S.QuerySet(*S.sample_config5(12, 64, 64)).restrict()
    te.label()
    mag, gated, _ = S.evaluate(model, te)
    ok = (te.irs > 0) & ((te.irs_status & 0x2f) == 0)
    err = np.abs(mag[ok] / te.irs[ok] - 1.0)
    assert np.median(err) <= 1e-3
    assert np.percentile(err, 99) <= 1e-2
    assert len(gated) <= 0.1 * te.n
