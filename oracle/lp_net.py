"""Test infrastructure: numpy restatement of the learned preconditioner's
network (forward, loss and backward) used as the checker of the device
training and inference kernels (nuclearcgm_gb300/csrc/k_learned.cu).

The reference has no learned preconditioner; its GCG uses the Jacobi
(diagonal) preconditioner of Eigen's ConjugateGradient
(src/solver/solver.cpp:664-666,733-743). This module defines the network
exactly as the device kernels compute it, in float64, so that the device
forward pass and gradients can be compared with it, and its own gradients
are checked against finite differences on the CPU.

Network (per instance: one real component of one residual column):
  input x: 3 channels on the n^3 lattice (residual r/s, (U+shift)/50,
  (f/h^2)/82.8); levels D0 = n, D(l+1) = (Dl + 1) // 2.
    e0 = relu(conv3(x;  W0 3->16))            D0
    e1 = relu(conv3(pool(e0); W1 16->16))     D1
    e2 = relu(conv3(pool(e1); W2 16->32))     D2
    e3 = relu(conv1(pool(e2); W3 32->64))     D3
    g3 = relu(conv1(e3; W4 64->32))           D3
    g2 = relu(conv3(e2 + up(g3); W5 32->16))  D2
    g1 = relu(conv3(e1 + up(g2); W6 16->16))  D1
    y  = conv3(e0 + up(g1); W7 16->1)         D0
conv3: 3x3x3 taps, zero outside the lattice; pool: sum of the (up to 8)
children 2q + {0,1}^3 inside the finer lattice, times 1/8; up: nearest
(fine p takes coarse p // 2). Weights are rounded to bfloat16 (round to
nearest even) before use; the FP32 master copy is what the optimiser
updates.
Loss over a batch of B instances: mean_b |y_b - t_b|^2 / (|t_b|^2 + 1e-30).
"""
import numpy as np

# (name, Cin, Cout, K) in parameter order; each layer stores W then bias
LAYERS = [("W0", 3, 16, 3), ("W1", 16, 16, 3), ("W2", 16, 32, 3),
          ("W3", 32, 64, 1), ("W4", 64, 32, 1), ("W5", 32, 16, 3),
          ("W6", 16, 16, 3), ("W7", 16, 1, 3)]


def num_params():
    return sum(co * ci * k ** 3 + co for _, ci, co, k in LAYERS)


def split(theta):
    """Flat parameter vector -> {name: (W[co, ci, k, k, k], b[co])}."""
    out, o = {}, 0
    for name, ci, co, k in LAYERS:
        nw = co * ci * k ** 3
        out[name] = (theta[o:o + nw].reshape(co, ci, k, k, k),
                     theta[o + nw:o + nw + co])
        o += nw + co
    return out


def bf16(a):
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    a = np.asarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def init(seed):
    """He-normal initial weights, zero biases, the device initialiser's
    distribution (not its random stream)."""
    rng = np.random.default_rng(seed)
    parts = []
    for _, ci, co, k in LAYERS:
        fan = ci * k ** 3
        parts.append(rng.normal(0, np.sqrt(2.0 / fan), co * fan))
        parts.append(np.zeros(co))
    return np.concatenate(parts).astype(np.float32)


def _shift(x, d):
    """x[..., k+dk, j+dj, i+di] with zeros outside (x: [..., D, D, D])."""
    dk, dj, di = d
    out = np.zeros_like(x)
    D = x.shape[-1]

    def sl(o):
        return (slice(max(0, -o), D - max(0, o)), slice(max(0, o), D + min(0, o)))
    (ak, bk), (aj, bj), (ai, bi) = sl(dk), sl(dj), sl(di)
    out[..., ak, aj, ai] = x[..., bk, bj, bi]
    return out


TAPS = [(dk, dj, di) for dk in (-1, 0, 1) for dj in (-1, 0, 1)
        for di in (-1, 0, 1)]


def conv(x, W, b):
    """x [B, ci, D, D, D], W [co, ci, k, k, k] -> [B, co, D, D, D]."""
    k = W.shape[-1]
    y = np.zeros((x.shape[0], W.shape[0]) + x.shape[2:])
    if k == 1:
        y += np.einsum("oc,bc...->bo...", W[:, :, 0, 0, 0], x)
    else:
        for t, d in enumerate(TAPS):
            y += np.einsum("oc,bc...->bo...", W[:, :, d[0] + 1, d[1] + 1,
                                                d[2] + 1], _shift(x, d))
    return y + b[None, :, None, None, None]


def _corr(dy, x):
    """sum over batch and lattice of dy[b, o, p] x[b, c, p] -> [o, c]."""
    B, co, ci = dy.shape[0], dy.shape[1], x.shape[1]
    return np.einsum("bop,bcp->oc", dy.reshape(B, co, -1), x.reshape(B, ci, -1))


def conv_bwd(x, W, dy):
    """Gradients of conv: (dx, dW, db)."""
    k = W.shape[-1]
    dW = np.zeros_like(W)
    db = dy.sum(axis=(0, 2, 3, 4))
    if k == 1:
        dW[:, :, 0, 0, 0] = _corr(dy, x)
        dx = np.einsum("oc,bo...->bc...", W[:, :, 0, 0, 0], dy)
        return dx, dW, db
    dx = np.zeros_like(x)
    for d in TAPS:
        xs = _shift(x, d)
        dW[:, :, d[0] + 1, d[1] + 1, d[2] + 1] = _corr(dy, xs)
        g = np.einsum("oc,bo...->bc...", W[:, :, d[0] + 1, d[1] + 1, d[2] + 1],
                      dy)
        dx += _shift(g, (-d[0], -d[1], -d[2]))
    return dx, dW, db


def coarse(D):
    return (D + 1) // 2


def pool(x):
    D = x.shape[-1]
    Dc = coarse(D)
    pad = np.zeros(x.shape[:2] + (2 * Dc,) * 3)
    pad[..., :D, :D, :D] = x
    return pad.reshape(x.shape[:2] + (Dc, 2, Dc, 2, Dc, 2)).sum(
        axis=(3, 5, 7)) / 8.0


def pool_bwd(dy, D):
    Dc = dy.shape[-1]
    g = np.repeat(np.repeat(np.repeat(dy, 2, 2), 2, 3), 2, 4) / 8.0
    return g[..., :D, :D, :D]


def up(x, D):
    g = np.repeat(np.repeat(np.repeat(x, 2, 2), 2, 3), 2, 4)
    return g[..., :D, :D, :D]


def up_bwd(dy, Dc):
    D = dy.shape[-1]
    pad = np.zeros(dy.shape[:2] + (2 * Dc,) * 3)
    pad[..., :D, :D, :D] = dy
    return pad.reshape(dy.shape[:2] + (Dc, 2, Dc, 2, Dc, 2)).sum(
        axis=(3, 5, 7))


def relu(x):
    return np.maximum(x, 0.0)


def forward(theta, x, keep=False, quant=True):
    """x [B, 3, n, n, n] -> y [B, 1, n, n, n] (and the activations).
    quant=False keeps float64 weights (finite-difference checks)."""
    q = bf16 if quant else (lambda w: np.asarray(w, np.float64))
    th = np.asarray(theta, np.float32 if quant else np.float64)
    P = {k: (q(W), np.asarray(b, np.float64)) for k, (W, b) in
         split(th).items()}
    a = {}
    a["x"] = x = np.asarray(x, np.float64)
    a["e0"] = relu(conv(x, *P["W0"]))
    a["p1"] = pool(a["e0"])
    a["e1"] = relu(conv(a["p1"], *P["W1"]))
    a["p2"] = pool(a["e1"])
    a["e2"] = relu(conv(a["p2"], *P["W2"]))
    a["p3"] = pool(a["e2"])
    a["e3"] = relu(conv(a["p3"], *P["W3"]))
    a["g3"] = relu(conv(a["e3"], *P["W4"]))
    a["d2"] = a["e2"] + up(a["g3"], a["e2"].shape[-1])
    a["g2"] = relu(conv(a["d2"], *P["W5"]))
    a["d1"] = a["e1"] + up(a["g2"], a["e1"].shape[-1])
    a["g1"] = relu(conv(a["d1"], *P["W6"]))
    a["d0"] = a["e0"] + up(a["g1"], a["e0"].shape[-1])
    a["y"] = conv(a["d0"], *P["W7"])
    return (a["y"], a, P) if keep else a["y"]


def loss(y, t):
    B = y.shape[0]
    num = ((y - t) ** 2).reshape(B, -1).sum(1)
    den = (t ** 2).reshape(B, -1).sum(1) + 1e-30
    return float((num / den).mean()), 2.0 * (y - t) / (den[:, None, None,
                                                              None, None] * B)


def backward(theta, x, t, quant=True):
    """Loss and its gradient with respect to the FP32 master parameters
    (the bf16 rounding is treated as the identity, straight-through, as the
    device optimiser does)."""
    y, a, P = forward(theta, x, keep=True, quant=quant)
    L, dy = loss(y, t)
    g = {}
    dd0, g["W7"], gb7 = conv_bwd(a["d0"], P["W7"][0], dy)
    g["b7"] = gb7
    de0 = dd0.copy()
    dg1 = up_bwd(dd0, a["g1"].shape[-1]) * (a["g1"] > 0)
    dd1, g["W6"], g["b6"] = conv_bwd(a["d1"], P["W6"][0], dg1)
    de1 = dd1.copy()
    dg2 = up_bwd(dd1, a["g2"].shape[-1]) * (a["g2"] > 0)
    dd2, g["W5"], g["b5"] = conv_bwd(a["d2"], P["W5"][0], dg2)
    de2 = dd2.copy()
    dg3 = up_bwd(dd2, a["g3"].shape[-1]) * (a["g3"] > 0)
    de3, g["W4"], g["b4"] = conv_bwd(a["e3"], P["W4"][0], dg3)
    de3 = de3 * (a["e3"] > 0)
    dp3, g["W3"], g["b3"] = conv_bwd(a["p3"], P["W3"][0], de3)
    de2 = (de2 + pool_bwd(dp3, a["e2"].shape[-1])) * (a["e2"] > 0)
    dp2, g["W2"], g["b2"] = conv_bwd(a["p2"], P["W2"][0], de2)
    de1 = (de1 + pool_bwd(dp2, a["e1"].shape[-1])) * (a["e1"] > 0)
    dp1, g["W1"], g["b1"] = conv_bwd(a["p1"], P["W1"][0], de1)
    de0 = (de0 + pool_bwd(dp1, a["e0"].shape[-1])) * (a["e0"] > 0)
    _, g["W0"], g["b0"] = conv_bwd(a["x"], P["W0"][0], de0)
    flat = []
    for name, ci, co, k in LAYERS:
        flat.append(g[name].reshape(-1))
        flat.append(g["b" + name[1:]].reshape(-1))
    return L, np.concatenate(flat)
