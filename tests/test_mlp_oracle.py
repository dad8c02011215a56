"""The numpy cost-model oracle (oracle/mlp_ref.py) is itself checked: its
analytic gradient against central finite differences in float64."""
import numpy as np

from oracle import mlp_ref


def test_mlp_ref_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    n_p = mlp_ref.H * mlp_ref.D + mlp_ref.H + mlp_ref.H * mlp_ref.H + mlp_ref.H + mlp_ref.H + 1
    p = rng.standard_normal(n_p) * 0.1
    X = rng.standard_normal((37, mlp_ref.D))
    y = rng.standard_normal(37)
    _, g = mlp_ref.loss_grad(p, X, y)
    idx = rng.choice(n_p, size=40, replace=False)
    h = 1e-6
    for i in idx:
        e = np.zeros(n_p)
        e[i] = h
        fd = (mlp_ref.loss_grad(p + e, X, y)[0] - mlp_ref.loss_grad(p - e, X, y)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(g[i]), (i, fd, g[i])
