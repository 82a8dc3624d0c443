"""The oracle's network gradient against central differences (float64, CPU)."""

import numpy as np

from oracle import oracle_py as orc


def test_mlp_gradient_finite_differences():
    rng = np.random.default_rng(0)
    n_params = sum(int(np.prod(s)) for _, s in orc.MLP_SHAPES)
    assert n_params == 1445
    p = rng.standard_normal(n_params) * 0.3
    X = rng.standard_normal((40, 6))
    y = rng.integers(0, 5, 40)
    loss, g, hits = orc.mlp_loss_grad(p, X, y)
    assert 0 <= hits <= 40
    idx = rng.choice(n_params, 60, replace=False)
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (orc.mlp_loss_grad(pp, X, y)[0] - orc.mlp_loss_grad(pm, X, y)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd))


def test_branch_features_invariants():
    rng = np.random.default_rng(1)
    n = 64
    E = rng.standard_normal((n, 6)) * 1e-3
    c_bar = np.full(n, 10.0)
    sin_phi = np.full(n, 0.5)
    shear = np.full(n, 8000.0)
    lame = np.full(n, 12000.0)
    X = orc.branch_features(E, c_bar, sin_phi, shear, lame)
    assert X.shape == (n, 6)
    assert np.all(np.abs(X[:, 3]) <= 1.0)
    # a pure volumetric strain has no deviator: first feature 0, Lode parameter 0
    Ev = np.zeros((1, 6))
    Ev[0, :3] = 1e-3
    Xv = orc.branch_features(Ev, c_bar[:1], sin_phi[:1], shear[:1], lame[:1])
    assert Xv[0, 0] == 0.0 and Xv[0, 3] == 0.0 and Xv[0, 1] > 0
