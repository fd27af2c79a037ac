"""Host-side logic of the surrogate (no GPU): the parameter layout of the
initialiser agrees with the FP64 restatement's, the sampler draws the
configured distributions, the training-row selection keeps only clean
IRS labels away from the caustic, the model's tensor checks reject wrong
arguments before any launch, and the FP64 gradient restatement agrees with
finite differences of its own loss."""
import math
import types

import numpy as np
import pytest


def test_init_params_layout_matches_oracle():
    from oracle import mlp
    from triplelens_gb300 import surrogate as S
    n = 16 * 256 + 256 + 3 * (256 * 256 + 256) + 256 + 1
    p = S.init_params(np.random.default_rng(0), n)
    layers, w5, b5 = mlp.unpack(p)
    assert layers[0][0].shape == (256, 16)
    assert np.all(layers[0][0][:, 14:] == 0.0)        # padding inputs
    for w, b in layers:
        assert np.all(b == 0.0) and np.std(w) > 0.0
    assert w5.shape == (256,) and b5 == 0.0


def test_sampler_distributions():
    from triplelens_gb300 import surrogate as S
    lenses, li, br, ix, off = S.sample_config5(3, 400, 16)
    rho, v = lenses[:, 5], lenses[:, 6]
    assert np.all((rho >= 1e-4) & (rho <= 3e-2))
    assert abs(np.median(np.log10(rho)) - 0.5 * (-4 + math.log10(3e-2))) < 0.2
    assert np.all((v >= 0.3) & (v <= 0.7)) and np.all(lenses[:, 7] == 500)
    assert np.all((br >= 0) & (br < 6)) and np.all((ix >= 0) & (ix < 500))
    r = np.hypot(off[:, 0], off[:, 1])
    assert r.max() <= 3.0 and abs(np.median(r) - 3.0 / math.sqrt(2)) < 0.1   # uniform disc
    _, li2, _, _, off2 = S.sample_config5(3, 400, 16, band=S.TRAIN_BAND)
    d = np.hypot(off2[:, 0], off2[:, 1]) / lenses[li2, 5]
    assert d.min() >= 2.0 * 0.999 and d.max() <= 10 ** 2.5 * 1.001


def test_training_rows():
    from triplelens_gb300 import surrogate as S

    class T:
        def __init__(self, a):
            self.a = a

        def cpu(self):
            return self

        def numpy(self):
            return self.a

    q = types.SimpleNamespace(
        n=5,
        irs=np.array([2.0, 2.0, 0.0, 3.0, 1.5]),
        irs_status=np.array([0, 16, 0, 4, 0], np.uint32),
        aps=T(np.array([1.9, 1.9, 1.0, 2.9, 1.4])),
        dc=T(np.array([5.0, 5.0, 5.0, 5.0, 1.0], np.float32)))
    y, ok = S.training_targets(q)
    # clean, image-count warning kept; empty IRS, table-full and near-caustic dropped
    assert list(ok) == [True, True, False, False, False]
    assert abs(y[0] - math.log(2.0 / 1.9)) < 1e-6


def test_device_tensor_checks_reject_before_any_launch():
    """Model methods check their device tensors (shape, type, contiguity,
    device) and host arrays (sizes) before a kernel is told how many rows to
    read: wrong ones raise ValueError.  On a machine without a GPU every
    tensor is a host tensor, which is rejected too."""
    torch = pytest.importorskip("torch")
    from triplelens_gb300 import surrogate as S
    feat = torch.zeros((8, S.N_FEATURES), dtype=torch.float32)
    with pytest.raises(ValueError):
        S._rows(feat)                                    # host tensor
    with pytest.raises(ValueError):
        S._rows(torch.zeros(8))                          # not 2-D
    with pytest.raises(ValueError):
        S._tensor("y", torch.zeros(8, dtype=torch.float64), (8,), torch.float32)
    with pytest.raises(ValueError):
        S._tensor("y", np.zeros(8, np.float32), (8,), torch.float32)
    assert S._host("mean", [0.0] * S.N_FEATURES, S.N_FEATURES).dtype == np.float32
    with pytest.raises(ValueError):
        S._host("mean", [0.0] * 13, S.N_FEATURES)
    with pytest.raises(ValueError):
        S._host("params", np.zeros(10), 11)


def test_gradient_oracle_matches_finite_differences(monkeypatch):
    """The FP64 gradient restatement the GPU gradients are checked against
    (oracle/mlp.py) is itself right: with the BF16 operand rounding switched
    off (it makes the loss piecewise constant in the weights), its gradient
    equals central finite differences of its loss on sampled weights and on
    every bias and output weight."""
    from oracle import mlp
    monkeypatch.setattr(mlp, "bf16", lambda a: np.asarray(a, np.float64))
    rng = np.random.Generator(np.random.PCG64(21))
    n_params = 16 * 256 + 256 + 3 * (256 * 256 + 256) + 256 + 1
    p = rng.normal(0.0, 0.08, n_params)
    feat = rng.normal(0.0, 1.0, (6, 14))
    target = rng.normal(0.0, 0.5, 6)
    mean, std = np.zeros(14), np.ones(14)
    _, _, g = mlp.forward_backward(p, feat, target, mean, std)
    assert g.shape == (n_params,)
    # a sample of weights, and every bias, output weight and the output bias
    offs, o = [], 0
    for fan_in in (16, 256, 256, 256):
        o += 256 * fan_in
        offs += list(range(o, o + 256))
        o += 256
    coords = np.concatenate([rng.choice(n_params, 300, replace=False), offs,
                             np.arange(o, n_params)])
    # inputs 14 and 15 of the first layer are padding: their weights see zeros
    pad = [r * 16 + c for r in range(256) for c in (14, 15)]
    assert np.all(g[pad] == 0.0)
    h = 1e-6
    num = np.empty(len(coords))
    for i, c in enumerate(coords):
        pp, pm = p.copy(), p.copy()
        pp[c] += h
        pm[c] -= h
        num[i] = (mlp.forward_backward(pp, feat, target, mean, std)[0] -
                  mlp.forward_backward(pm, feat, target, mean, std)[0]) / (2 * h)
    scale = np.abs(g[coords]).max()
    assert np.max(np.abs(num - g[coords])) < 1e-6 * scale


def test_checkpoint_round_trip_and_rejections(tmp_path):
    """Surrogate checkpoints (flat binary with a header): a round trip keeps
    every parameter, the standardisation and the metadata bit for bit; other
    files, bad headers and short files raise ValueError."""
    from triplelens_gb300 import surrogate as S
    rng = np.random.Generator(np.random.PCG64(3))
    params = rng.normal(0.0, 1.0, (4, 1000)).astype(np.float32)
    mean = rng.normal(0.0, 1.0, S.N_FEATURES).astype(np.float32)
    std = rng.uniform(0.5, 2.0, S.N_FEATURES).astype(np.float32)
    path = tmp_path / "model.tls"
    S.save_checkpoint(path, params, mean, std, {"gate": S.GATE, "train_points": 55000})
    p2, m2, s2, meta = S.load_checkpoint(path)
    assert p2.dtype == np.float32 and np.array_equal(p2, params)
    assert np.array_equal(m2, mean) and np.array_equal(s2, std)
    assert meta == {"gate": S.GATE, "train_points": 55000}
    raw = path.read_bytes()
    bad = tmp_path / "bad"
    for content in (b"not a checkpoint at all......", raw[:-4], raw + b"\0\0\0\0",
                    raw[:8] + np.array([4, 1000, 13, 0], "<i4").tobytes() + raw[24:]):
        bad.write_bytes(content)
        with pytest.raises(ValueError):
            S.load_checkpoint(bad)
    with pytest.raises(ValueError):
        S.save_checkpoint(path, params[0], mean, std)          # one row per member
    with pytest.raises(ValueError):
        S.save_checkpoint(path, params, mean[:10], std)
