"""The learned finite-source correction (include/tl_surrogate.h) and its
gated evaluation against the GPU IRS.

Workload (finite-source surrogate, training and evaluation sets): triple
lenses drawn as the random light-curve lenses (mass ratios log-uniform in
[1e-3, 1], separations log-uniform in [0.5, 2], angle uniform); per lens a
source radius log-uniform in [1e-4, 3e-2] and a linear limb-darkening
coefficient uniform in [0.3, 0.7]; source positions = a uniform caustic
sample plus a uniform offset in a disc of radius 3 theta_E.  Labels are
y = ln(A_IRS / A_point) from the GPU IRS at 500 rays per source radius.

The network (4 members of 14 -> 256 x 4 SiLU -> 1) runs in the library's own
BF16 tensor-core kernels; this module only samples inputs, holds device
buffers (torch tensors as plumbing) and drives training and evaluation.
"""
import ctypes
import math
import time

import numpy as np

from .batch import Batch, _ptr
from .workloads import _random_lens

N_FEATURES = 14
PPR = 500
# gate: IRS within `near` source radii of the caustic, or closer than `far`
# when the members' spread of y exceeds `max_std`; A_point alone beyond `far`
# (chosen on held-out near-caustic queries: median error 2e-5, p99 9e-3)
GATE = {"near": 2.0, "max_std": 3e-3, "far": 30.0}
TRAIN_BAND = (math.log10(2.0), 2.5)   # training sources 2-300 rho from a caustic
# queries with a larger point-source magnification (more than ~2.4e8 rays at
# 500 rays per source radius: sources within about rho of a cusp at small rho)
# are left out of both the training and the evaluation sets
A_MAX = 300.0


def _bind(L):
    if getattr(L, "_tls_bound", False):
        return L
    vp, i, f = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
    L.tls_param_count.restype = i
    L.tls_new.argtypes = [i]
    L.tls_new.restype = vp
    L.tls_delete.argtypes = [vp]
    L.tls_set_params.argtypes = [vp, i, vp]
    L.tls_get_params.argtypes = [vp, i, vp]
    L.tls_set_normalisation.argtypes = [vp, vp, vp]
    L.tls_train_step.argtypes = [vp, i, i, vp, vp, f, vp, vp]
    L.tls_gradients.argtypes = [vp, i, i, vp, vp, vp, vp]
    L.tls_forward.argtypes = [vp, i, i, vp, vp, vp]
    L.tls_predict.argtypes = [vp, i, vp, vp, vp, f, f, f, vp, vp, vp, vp, vp]
    L.tls_features.argtypes = [vp, i, vp, vp, vp, vp, vp, vp]
    L.tlb_caustic_points.argtypes = [vp, i, vp, vp, vp, vp, vp]
    for n in ("tls_set_params", "tls_get_params", "tls_set_normalisation", "tls_train_step",
              "tls_gradients", "tls_forward", "tls_predict", "tls_features",
              "tlb_caustic_points"):
        getattr(L, n).restype = i
    L._tls_bound = True
    return L


def _dp(t):
    return ctypes.c_void_p(t.data_ptr())


def _check(r, what):
    if r != 0:
        raise RuntimeError("%s failed: %d" % (what, r))


# The kernels read and write as many rows as they are told: the device
# tensors are checked here, so that a wrong shape, type or device raises
# instead of sending a kernel past the end of a buffer.
def _tensor(name, t, shape, dtype):
    import torch
    if not isinstance(t, torch.Tensor) or t.device.type != "cuda" or t.dtype != dtype \
            or not t.is_contiguous() or tuple(t.shape) != tuple(shape):
        raise ValueError("%s: a contiguous CUDA tensor of %s and shape %s, got %s"
                         % (name, dtype, tuple(shape),
                            (tuple(t.shape), t.dtype, str(t.device))
                            if isinstance(t, torch.Tensor) else type(t).__name__))


def _rows(feat):
    """Rows of a feature tensor (M x N_FEATURES float32 on the GPU)."""
    import torch
    m = feat.shape[0] if isinstance(feat, torch.Tensor) and feat.dim() == 2 else -1
    _tensor("feat", feat, (m, N_FEATURES), torch.float32)
    return m


def _host(name, a, n):
    """A float32 host array of exactly n values, contiguous."""
    a = np.ascontiguousarray(a, np.float32).reshape(-1)
    if a.size != n:
        raise ValueError("%s: %d values, got %d" % (name, n, a.size))
    return a


def init_params(rng, n_params):
    """He-uniform weights, zero biases, in the library's parameter layout."""
    p = np.zeros(n_params, np.float32)
    w, inp = 256, 16
    o = 0
    for fan_in in (inp, w, w, w):
        fan_out = w
        lim = math.sqrt(6.0 / fan_in)
        n = fan_out * fan_in
        p[o:o + n] = rng.uniform(-lim, lim, n)
        if fan_in == inp:
            p[o:o + n].reshape(w, inp)[:, N_FEATURES:] = 0.0
        o += n + fan_out   # weights, then biases (zero)
    lim = math.sqrt(3.0 / w)
    p[o:o + w] = rng.uniform(-lim, lim, w) * 0.1
    assert o + w + 1 == n_params
    return p


CHECKPOINT_MAGIC = b"TLSURR01"


def save_checkpoint(path, params, mean, std, meta=None):
    """Writes an ensemble as a flat binary with a header: the 8-byte magic,
    four little-endian int32 (members, parameters per member, features,
    metadata bytes), the metadata (UTF-8 JSON), then float32 arrays: the
    feature mean and standard deviation, and every member's parameters in
    the library's layout.  Adam's moments are not kept: tls_set_params
    starts them from zero, so training resumes with fresh moments."""
    import json
    params = np.ascontiguousarray(params, np.float32)
    if params.ndim != 2:
        raise ValueError("params: one row per member")
    mean = _host("mean", mean, N_FEATURES)
    std = _host("std", std, N_FEATURES)
    blob = json.dumps(meta or {}).encode()
    head = np.array([params.shape[0], params.shape[1], N_FEATURES, len(blob)], "<i4")
    with open(path, "wb") as f:
        f.write(CHECKPOINT_MAGIC)
        f.write(head.tobytes())
        f.write(blob)
        for a in (mean, std, params):
            f.write(a.astype("<f4").tobytes())


def load_checkpoint(path):
    """(params (members x n), mean, std, meta) from save_checkpoint's file;
    ValueError on another format or a short file."""
    import json
    with open(path, "rb") as f:
        data = f.read()
    if data[:8] != CHECKPOINT_MAGIC or len(data) < 24:
        raise ValueError("%s: not a surrogate checkpoint" % path)
    members, n, nf, nmeta = (int(x) for x in np.frombuffer(data[8:24], "<i4"))
    if members <= 0 or n <= 0 or nf != N_FEATURES or nmeta < 0:
        raise ValueError("%s: bad header" % path)
    o = 24 + nmeta
    need = o + 4 * (2 * nf + members * n)
    if len(data) != need:
        raise ValueError("%s: %d bytes, the header says %d" % (path, len(data), need))
    meta = json.loads(data[24:o].decode() or "{}")
    floats = np.frombuffer(data[o:], "<f4").astype(np.float32)
    return floats[2 * nf:].reshape(members, n), floats[:nf], floats[nf:2 * nf], meta


class Model:
    """Ensemble of MLPs in the library (BF16 GEMMs, FP32 Adam)."""

    def __init__(self, members=4, seed=0, lib=None):
        from .lcirs import load_lcirs
        self.L = _bind(lib or load_lcirs())
        self.members = members
        self.obj = self.L.tls_new(members)
        if not self.obj:
            raise RuntimeError("tls_new failed")
        self.n_params = self.L.tls_param_count()
        # the library's initial standardisation (identity)
        self.mean = np.zeros(N_FEATURES, np.float32)
        self.std = np.ones(N_FEATURES, np.float32)
        rng = np.random.Generator(np.random.PCG64(seed))
        for k in range(members):
            self.set_params(k, init_params(rng, self.n_params))

    def __del__(self):
        try:
            self.L.tls_delete(self.obj)
        except Exception:
            pass

    def set_params(self, k, p):
        p = _host("params", p, self.n_params)
        _check(self.L.tls_set_params(self.obj, k, p.ctypes.data_as(ctypes.c_void_p)), "set_params")

    def get_params(self, k):
        p = np.zeros(self.n_params, np.float32)
        _check(self.L.tls_get_params(self.obj, k, p.ctypes.data_as(ctypes.c_void_p)), "get_params")
        return p

    def set_normalisation(self, mean, std):
        mean = _host("mean", mean, N_FEATURES)
        std = _host("std", std, N_FEATURES)
        _check(self.L.tls_set_normalisation(self.obj, mean.ctypes.data_as(ctypes.c_void_p),
                                            std.ctypes.data_as(ctypes.c_void_p)), "normalisation")
        self.mean, self.std = mean.copy(), std.copy()

    def save(self, path, meta=None):
        """The ensemble's weights and standardisation (save_checkpoint)."""
        save_checkpoint(path, np.stack([self.get_params(k) for k in range(self.members)]),
                        self.mean, self.std, meta)

    @classmethod
    def load(cls, path, lib=None):
        """An ensemble from save_checkpoint's file, and its metadata."""
        params, mean, std, meta = load_checkpoint(path)
        m = cls(members=params.shape[0], lib=lib)
        if params.shape[1] != m.n_params:
            raise ValueError("%s: %d parameters per member, the library has %d"
                             % (path, params.shape[1], m.n_params))
        for k in range(m.members):
            m.set_params(k, params[k])
        m.set_normalisation(mean, std)
        return m, meta

    def gradients(self, k, feat, target):
        import torch
        _tensor("target", target, (_rows(feat),), torch.float32)
        g = np.zeros(self.n_params, np.float32)
        loss = np.zeros(1, np.float32)
        _check(self.L.tls_gradients(self.obj, k, feat.shape[0], _dp(feat), _dp(target),
                                    g.ctypes.data_as(ctypes.c_void_p),
                                    loss.ctypes.data_as(ctypes.c_void_p)), "gradients")
        return g, float(loss[0])

    def train_step(self, k, feat, target, lr, loss_dev=None, stream=None):
        import torch
        _tensor("target", target, (_rows(feat),), torch.float32)
        if loss_dev is not None:
            _tensor("loss_dev", loss_dev, (1,), torch.float32)
        _check(self.L.tls_train_step(self.obj, k, feat.shape[0], _dp(feat), _dp(target), lr,
                                     _dp(loss_dev) if loss_dev is not None else None, stream),
               "train_step")

    def forward(self, k, feat, y, stream=None):
        import torch
        _tensor("y", y, (_rows(feat),), torch.float32)
        _check(self.L.tls_forward(self.obj, k, feat.shape[0], _dp(feat), _dp(y), stream), "forward")

    def predict(self, feat, aps, dc_rho, max_std, min_dc_rho, out, far_dc_rho=GATE["far"],
                stream=None):
        """out: dict of device tensors mean, std (float32), mag (float64),
        gated (int32)."""
        import torch
        m = _rows(feat)
        _tensor("aps", aps, (m,), torch.float64)
        _tensor("dc_rho", dc_rho, (m,), torch.float32)
        for key, dt in (("mean", torch.float32), ("std", torch.float32), ("mag", torch.float64),
                        ("gated", torch.int32)):
            _tensor("out['%s']" % key, out[key], (m,), dt)
        _check(self.L.tls_predict(self.obj, feat.shape[0], _dp(feat), _dp(aps), _dp(dc_rho),
                                  float(max_std), float(min_dc_rho), float(far_dc_rho),
                                  _dp(out["mean"]),
                                  _dp(out["std"]), _dp(out["mag"]), _dp(out["gated"]), stream),
               "predict")


def sample_config5(seed, n_lens, per_lens, radius=3.0, band=None):
    """Lens rows (a, b, th, m2, m3, rho, v, ppr) and, per sample, its lens,
    caustic branch and sample index and the offset from that sample.
    Offsets are uniform in a disc of `radius` theta_E, or, with band = (lo,
    hi), at distances rho * 10^U(lo, hi) in a uniform direction (the band
    around the caustics where the finite-source correction matters)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lenses = np.zeros((n_lens, 8))
    for i in range(n_lens):
        a, b, th, m2, m3 = _random_lens(rng)
        rho = 10.0 ** rng.uniform(-4.0, math.log10(3e-2))
        v = rng.uniform(0.3, 0.7)
        lenses[i] = (a, b, th, m2, m3, rho, v, PPR)
    n = n_lens * per_lens
    lens_idx = np.repeat(np.arange(n_lens, dtype=np.int32), per_lens)
    branch = rng.integers(0, 6, n).astype(np.int32)
    index = rng.integers(0, 500, n).astype(np.int32)
    if band is None:
        r = radius * np.sqrt(rng.uniform(0.0, 1.0, n))
    else:
        r = lenses[lens_idx, 5] * 10.0 ** rng.uniform(band[0], band[1], n)
    ang = rng.uniform(0.0, 2.0 * math.pi, n)
    off = np.stack([r * np.cos(ang), r * np.sin(ang)], axis=1)
    return lenses, lens_idx, branch, index, off


class QuerySet:
    """Source positions on a batch of lenses, their features, and (on
    request) their IRS magnifications."""

    def __init__(self, lenses, lens_idx, branch, index, offsets, batch=None):
        import torch
        self.dev = torch.device("cuda")
        self.b = batch or Batch()
        self.L = _bind(self.b.L)
        self.b.set_lenses(lenses)
        self.lenses = lenses
        n = len(lens_idx)
        self.n = n
        t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a)).to(self.dev, dt)
        self.lens_idx = t(lens_idx, torch.int32)
        br, ix = t(branch, torch.int32), t(index, torch.int32)
        self.xy = torch.empty((n, 2), dtype=torch.float64, device=self.dev)
        _check(self.L.tlb_caustic_points(self.b.obj, n, _dp(self.lens_idx), _dp(br), _dp(ix),
                                         _dp(self.xy), None), "caustic points")
        self.xy += t(offsets, torch.float64)
        self.feat = torch.empty((n, N_FEATURES), dtype=torch.float32, device=self.dev)
        self.aps = torch.empty(n, dtype=torch.float64, device=self.dev)
        self.dc = torch.empty(n, dtype=torch.float32, device=self.dev)
        self.irs = None

    def features(self, stream=None):
        _check(self.L.tls_features(self.b.obj, self.n, _dp(self.xy), _dp(self.lens_idx),
                                   _dp(self.feat), _dp(self.aps), _dp(self.dc), stream),
               "features")

    def restrict(self, a_max=A_MAX):
        """Keep the queries whose point-source magnification is at most
        a_max (computes the features)."""
        import torch
        self.features()
        keep = torch.nonzero(self.aps <= a_max).flatten()
        self.xy = self.xy[keep].contiguous()
        self.lens_idx = self.lens_idx[keep].contiguous()
        self.feat = self.feat[keep].contiguous()
        self.aps = self.aps[keep].contiguous()
        self.dc = self.dc[keep].contiguous()
        self.n = int(keep.numel())
        return self

    def irs_points(self, sel=None):
        """IRS magnifications (and status) of all or the selected points,
        through the batch API (single-position trajectories)."""
        import torch
        idx = torch.arange(self.n, device=self.dev) if sel is None else sel
        xy = self.xy[idx].cpu().numpy()
        li = self.lens_idx[idx].cpu().numpy()
        m = len(li)
        if m == 0:
            return np.zeros(0), np.zeros(0, np.uint32)
        trajs = np.concatenate([xy, xy], axis=1)
        amp = np.zeros(m)
        cnt = np.zeros(m, np.uint64)
        st = np.zeros(m, np.uint32)
        self.b.run_host(trajs, li, np.zeros(m, np.uint32), amp, cnt, st)
        return amp, st

    def label(self):
        amp, st = self.irs_points()
        self.irs = amp
        self.irs_status = st
        return amp, st


def training_targets(q, min_dc_rho=2.0):
    """Network targets y = ln(A_IRS / A_point) and the rows usable for
    training (clean IRS status, at least min_dc_rho source radii from the
    caustic)."""
    aps = q.aps.cpu().numpy()
    dc = q.dc.cpu().numpy()
    ok = (q.irs > 0) & (aps > 0) & np.isfinite(aps) & ((q.irs_status & 0x2f) == 0)
    ok &= dc >= min_dc_rho
    y = np.zeros(q.n, np.float32)
    y[ok] = np.log(q.irs[ok] / aps[ok])
    return y, ok


def train(model, feat, y, epochs=20, batch=8192, lr=1e-3, seed=0, log=None):
    """Adam over shuffled mini-batches, every member on its own order.  The
    targets are standardised for training; the output layer is rescaled
    afterwards so that the members predict y itself."""
    import torch
    n = feat.shape[0]
    y_scale = float(y.std().item()) or 1.0
    y = (y / y_scale).contiguous()
    batch = min(batch, n)
    loss = torch.zeros(1, dtype=torch.float32, device=feat.device)
    g = torch.Generator(device="cpu")
    g.manual_seed(seed)
    steps = 0
    for ep in range(epochs):
        lr_ep = lr * 0.5 * (1.0 + math.cos(math.pi * ep / epochs))
        for k in range(model.members):
            perm = torch.randperm(n, generator=g).to(feat.device)
            for s in range(0, n - batch + 1, batch):
                idx = perm[s:s + batch]
                model.train_step(k, feat[idx].contiguous(), y[idx].contiguous(), lr_ep, loss)
                steps += 1
        if log:
            log(ep, float(loss.item()))
    for k in range(model.members):
        p = model.get_params(k)
        p[-257:] *= y_scale   # w5, b5
        model.set_params(k, p)
    return steps


def new_outputs(n, dev):
    import torch
    return {"mean": torch.empty(n, dtype=torch.float32, device=dev),
            "std": torch.empty(n, dtype=torch.float32, device=dev),
            "mag": torch.empty(n, dtype=torch.float64, device=dev),
            "gated": torch.empty(n, dtype=torch.int32, device=dev)}


def fit(seed, n_lens, per_lens, members=4, epochs=40, batch=2048, lr=2e-3, lib=None):
    """Label a training set (sources in TRAIN_BAND) with the GPU IRS and
    train an ensemble on it.  Returns the model and timings."""
    import torch
    t0 = time.perf_counter()
    tr = QuerySet(*sample_config5(seed, n_lens, per_lens, band=TRAIN_BAND)).restrict()
    tr.label()
    t1 = time.perf_counter()
    y, ok = training_targets(tr)
    rows = torch.from_numpy(np.nonzero(ok)[0]).to(tr.dev)
    feat = tr.feat[rows].contiguous()
    fn = feat.cpu().numpy()
    model = Model(members=members, seed=seed, lib=lib)
    model.set_normalisation(fn.mean(0), fn.std(0) + 1e-6)
    steps = train(model, feat, torch.from_numpy(y[ok]).to(tr.dev), epochs=epochs, batch=batch,
                  lr=lr)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    return model, {"train_points": int(ok.sum()), "label_s": t1 - t0, "train_s": t2 - t1,
                   "steps": steps}


def evaluate(model, q, max_std=GATE["max_std"], min_dc_rho=GATE["near"]):
    """Gated magnifications of a query set: surrogate where trusted, IRS
    elsewhere.  Returns the magnifications, the gated mask and timings."""
    import torch
    n = q.n
    out = new_outputs(n, q.dev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    q.features()
    model.predict(q.feat, q.aps, q.dc, max_std, min_dc_rho, out)
    gated = torch.nonzero(out["gated"]).flatten()
    mag = out["mag"].cpu().numpy()
    t1 = time.perf_counter()
    irs_amp, _ = q.irs_points(gated)
    g = gated.cpu().numpy()
    mag[g] = irs_amp
    t2 = time.perf_counter()
    return mag, g, {"surrogate_s": t1 - t0, "irs_fallback_s": t2 - t1, "total_s": t2 - t0}
