"""CPU checks of the CNN oracle: finite-difference gradient of <gy, y>."""
import numpy as np

from oracle import cnn_oracle as C


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    N = (3, 4, 2)
    nc = int(np.prod(N))
    ci, ch, co = 5, 4, 3
    n_params = ch * ci + ch + ch * ch * 27 + ch + co * ch * 27 + co + co * ci
    p = rng.normal(0, 0.3, n_params)
    x = rng.normal(0, 1, (ci, nc))
    gy = rng.normal(0, 1, (co, nc))
    g = C.backward(p, x, gy, N, ci, ch, co)
    for idx in rng.choice(n_params, 25, replace=False):
        e = np.zeros(n_params)
        e[idx] = 1e-6
        fp = np.sum(gy * C.forward(p + e, x, N, ci, ch, co)[0])
        fm = np.sum(gy * C.forward(p - e, x, N, ci, ch, co)[0])
        assert abs((fp - fm) / 2e-6 - g[idx]) <= 1e-6 * max(1.0, abs(g[idx]))
