"""CPU checks of the surrogate network's oracle (oracle/mlp_oracle.c), the
reference the GPU training kernels are compared with: its gradient agrees with
central finite differences, and the loss vanishes when the targets are the
network's own outputs."""
import numpy as np

from oracle import oracle as O

NP = 50306


def _params(seed):
    rng = np.random.default_rng(seed)
    dims = [3, 128, 128, 128, 128, 2]
    out = []
    for a, b in zip(dims[:-1], dims[1:]):
        out.append(rng.uniform(-1, 1, a * b) * np.sqrt(6.0 / (a + b)))
        out.append(rng.normal(0, 0.1, b))
    return np.concatenate(out)


def test_parameter_count():
    assert O.lib().oracle_mlp_n_params() == NP


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = _params(1)
    x = rng.uniform(-1, 1, (16, 3))
    t = rng.normal(0, 1, (16, 2))
    _, g, _ = O.mlp_loss_grad(p, x, t)
    # 48 parameters spread over every weight and bias block
    idx = np.unique(np.concatenate([rng.integers(0, NP, 40), [0, 383, 384, 511, NP - 1, NP - 2, NP - 3, NP - 258]]))
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (O.mlp_loss_grad(pp, x, t)[0] - O.mlp_loss_grad(pm, x, t)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, fd, g[i])


def test_zero_loss_at_own_outputs():
    rng = np.random.default_rng(5)
    p = _params(2)
    x = rng.uniform(-1, 1, (32, 3))
    _, _, y = O.mlp_loss_grad(p, x, np.zeros((32, 2)))
    loss, g, _ = O.mlp_loss_grad(p, x, y)
    assert loss == 0.0
    assert np.all(g == 0.0)
