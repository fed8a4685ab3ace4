"""CPU checks of the learned preconditioner's numpy checker (oracle/lp_net):
its gradients against finite differences, layer by layer, and the shapes
of the pooling/upsampling on odd lattices."""
import numpy as np

from oracle import lp_net as L


def test_parameter_count():
    assert L.num_params() == 47489


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159265, 0.0],
                 np.float32)
    r = L.bf16(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: even mantissa is 1
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125
    assert abs(r[3] + 3.140625) < 1e-12 and r[4] == 0.0


def test_pool_and_up_shapes_on_odd_lattice():
    x = np.arange(2 * 3 * 7 ** 3, dtype=np.float64).reshape(2, 3, 7, 7, 7)
    p = L.pool(x)
    assert p.shape == (2, 3, 4, 4, 4)
    # corner cell of the coarse lattice holds only one fine child
    assert p[0, 0, 3, 3, 3] == x[0, 0, 6, 6, 6] / 8
    u = L.up(p, 7)
    assert u.shape == x.shape and u[1, 2, 5, 4, 6] == p[1, 2, 2, 2, 3]


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    n = 7
    th = L.init(1).astype(np.float64)
    x = rng.normal(size=(2, 3, n, n, n))
    t = rng.normal(size=(2, 1, n, n, n))
    _, g = L.backward(th, x, t, quant=False)
    o, worst = 0, 0.0
    for name, ci, co, k in L.LAYERS:
        nw = co * ci * k ** 3
        picks = list(rng.choice(nw, 3, replace=False) + o) + [o + nw]
        for i in picks:
            h = 1e-5
            tp, tm = th.copy(), th.copy()
            tp[i] += h
            tm[i] -= h
            fd = (L.loss(L.forward(tp, x, quant=False), t)[0] -
                  L.loss(L.forward(tm, x, quant=False), t)[0]) / (2 * h)
            worst = max(worst, abs(fd - g[i]) / max(1e-9, abs(fd) + abs(g[i])))
        o += nw + co
    assert worst < 1e-5
