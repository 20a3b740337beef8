"""The FNO oracle's backward pass against central finite differences of its
own forward pass (float64, no bf16 rounding), and the product's parameter
layout against the oracle's."""
import numpy as np

from oracle import fno as O


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(1)
    S, m, C, cin, cout, layers = 16, 4, 6, 3, 2, 2
    p = O.init_params(cin, cout, seed=3, C=C, m=m, layers=layers)
    for k in p:
        p[k] = p[k] + 0.1 * rng.standard_normal(p[k].shape)
    a = rng.standard_normal((2, cin, S, S))
    t = rng.standard_normal((2, cout, S, S))
    w = [1.0, 0.5]

    def loss(q):
        return O.loss_and_grad(q, a, t, w, layers=layers, m=m, bf16_mode=False)[0]

    _, _, g = O.loss_and_grad(p, a, t, w, layers=layers, m=m, bf16_mode=False)
    for name in p:
        flat = p[name].ravel()
        for i in rng.choice(flat.size, min(4, flat.size), replace=False):
            e = 1e-6
            q = {k: v.copy() for k, v in p.items()}
            q[name].ravel()[i] += e
            lp = loss(q)
            q[name].ravel()[i] -= 2 * e
            lm = loss(q)
            fd = (lp - lm) / (2 * e)
            an = g[name].ravel()[i]
            assert abs(fd - an) <= 1e-4 * (abs(fd) + abs(an)) + 1e-9, (name, i, fd, an)


def test_bf16_rounding_is_round_to_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -2.5, 3.0e38], dtype=np.float32)
    got = O.bf16(x)
    assert got[0] == 1.0 and got[1] == 1.0 and got[2] == 1.0 + 2 ** -6 and got[3] == 1.0
    assert got[4] == -2.5


def test_product_layout_matches_oracle():
    from turbulence_tracing_gb300 import fno

    for cin, cout, layers in ((2, 3, 4), (1, 1, 1), (8, 4, 8)):
        lay_p, n_p = fno.param_layout(cin, cout, layers)
        lay_o, n_o = O.param_layout(cin + 2, cout, layers=layers)
        assert n_p == n_o
        assert [(a, b, tuple(c)) for a, b, c in lay_p] == [(a, b, tuple(c)) for a, b, c in lay_o]
