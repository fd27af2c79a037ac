"""CPU restatement (NumPy, FP64) of the surrogate network of
triplelens_gb300/csrc/surrogate.cu: 14 (padded to 16) -> 256 x 4 SiLU -> 1,
mean squared error.  TEST INFRASTRUCTURE ONLY: the GPU tests compare the
library's BF16 tensor-core forward pass and gradients with it.  It rounds
weights and inputs to BF16 as the library's GEMM operands are, and keeps every
other quantity in FP64.  The network is this project's own (the reference has
no learned part).
"""
import numpy as np

W, IN, IN_PAD, HIDDEN = 256, 14, 16, 4


def bf16(a):
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    """Layer weights and biases from the library's flat parameter layout."""
    p = np.asarray(p, np.float64)
    out, o = [], 0
    for fan_in in (IN_PAD, W, W, W):
        w = p[o:o + W * fan_in].reshape(W, fan_in)
        o += W * fan_in
        b = p[o:o + W]
        o += W
        out.append((w, b))
    w5 = p[o:o + W]
    b5 = p[o + W]
    return out, w5, b5


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward_backward(p, feat, target, mean, std):
    """Loss, predictions and the flat gradient (library layout)."""
    layers, w5, b5 = unpack(p)
    x = np.zeros((feat.shape[0], IN_PAD))
    x[:, :IN] = (np.asarray(feat, np.float64) - mean) / std
    x = bf16(x)
    acts, zs = [x], []
    h = x
    for w, b in layers:
        z = h @ bf16(w).T + b
        zs.append(z)
        h = silu(z)
        acts.append(h)
    y = h @ w5 + b5
    m = feat.shape[0]
    diff = y - target
    loss = float(np.mean(diff * diff))
    dy = 2.0 * diff / m
    grads = []
    gw5 = acts[-1].T @ dy
    gb5 = dy.sum()
    dh = np.outer(dy, w5)
    for l in range(HIDDEN - 1, -1, -1):
        dz = dh * dsilu(zs[l])
        gw = dz.T @ acts[l]
        gb = dz.sum(axis=0)
        grads.append((gw, gb))
        dh = dz @ bf16(layers[l][0])
    flat = []
    for gw, gb in reversed(grads):
        flat += [gw.ravel(), gb]
    flat += [gw5, np.array([gb5])]
    return loss, y, np.concatenate(flat)
