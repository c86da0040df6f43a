"""The warm-start network's CPU oracle: its backward pass is the exact
gradient of its forward pass (central differences, float64 without the BF16
rounding), and the grid transfers are transposes of each other."""
import numpy as np

from oracle import nn_oracle as N


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    p = N.init_params(3)
    x = rng.uniform(-1, 1, (9, 9, 9, 2))
    t = rng.normal(size=(9, 9, 9, 4))
    _, g = N.loss_grad(p, x, t, exact=True)
    o = 0
    for _, ci, co, _ in N.LAYERS:
        n = 27 * ci * co + co
        for j in rng.choice(n, 2, replace=False):
            i, e = o + j, 1e-6
            pp, pm = p.copy(), p.copy()
            pp[i] += e
            pm[i] -= e
            fd = (N.loss_grad(pp, x, t, exact=True)[0] - N.loss_grad(pm, x, t, exact=True)[0]) / (2 * e)
            assert abs(fd - g[i]) <= 1e-5 * max(abs(fd), 1e-3), (i, fd, g[i])
        o += n


def test_transfers_are_transposes():
    rng = np.random.default_rng(2)
    c = rng.normal(size=(5, 9, 5, 3))
    f = rng.normal(size=(9, 17, 9, 3))
    assert np.isclose(np.sum(N.prolong(c) * f), np.sum(c * N.prolong_t(f)))
    assert np.isclose(np.sum(N.restrict(f) * c), np.sum(f * N.restrict_t(c)))
    # the normalised restriction keeps constants
    assert np.allclose(N.restrict(np.ones((9, 17, 9, 1))), 1.0)
