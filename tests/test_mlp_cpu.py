"""The CPU model of the learned-skin network: analytic gradient against
central finite differences (FP64, no rounding)."""
import numpy as np

from oracle import mlp_ref


def test_mlp_reference_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = rng.normal(scale=0.3, size=mlp_ref.NP)
    X = rng.normal(size=(12, mlp_ref.NIN))
    T = rng.normal(size=(12, mlp_ref.NOUT))
    loss, g = mlp_ref.loss_and_grad(p, X, T, half=False)
    idx = rng.choice(mlp_ref.NP, 60, replace=False)
    eps = 1e-6
    for k in idx:
        q = p.copy()
        q[k] += eps
        lp, _ = mlp_ref.loss_and_grad(q, X, T, half=False)
        q[k] -= 2 * eps
        lm, _ = mlp_ref.loss_and_grad(q, X, T, half=False)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-6 + 1e-5 * abs(fd), (k, fd, g[k])
