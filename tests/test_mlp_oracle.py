"""The CPU oracle of the learned sensor's network is itself checked: with the
BF16 rounding switched off its analytic gradient equals central finite
differences of its loss (float64)."""
import numpy as np


def test_oracle_gradient_finite_differences():
    import mlp
    rng = np.random.default_rng(0)
    n = 64
    X = rng.normal(0.5, 0.4, (n, 40))
    y = (rng.uniform(size=n) < 0.4).astype(np.float64)
    w = rng.uniform(0.5, 2.0, n)
    P = mlp.init_params(1).astype(np.float64)
    P[mlp.OFF_B1:mlp.OFF_W2] = 0.05
    mlp.ROUND = False
    try:
        _, g = mlp.loss_and_grad(P, X, y, w)
        idx = np.concatenate([rng.choice(mlp.NPARAMS - 1, 60, replace=False), [mlp.NPARAMS - 1]])
        h = 1e-6
        for i in idx:
            Pp, Pm = P.copy(), P.copy()
            Pp[i] += h
            Pm[i] -= h
            fd = (mlp.loss_and_grad(Pp, X, y, w)[0] - mlp.loss_and_grad(Pm, X, y, w)[0]) / (2 * h)
            assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])
    finally:
        mlp.ROUND = True


def test_bf16_rounding_matches_torch():
    import mlp
    import torch
    x = np.random.default_rng(3).normal(0, 10, 10000).astype(np.float32)
    ref = torch.from_numpy(x).to(torch.bfloat16).to(torch.float32).numpy()
    assert np.array_equal(mlp.bf16(x), ref)
