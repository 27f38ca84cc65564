"""CPU restatement of the learned indicator (oracle/mlp.py): its gradient against finite
differences of its own loss, and its BF16 rounding."""
import numpy as np

from oracle import mlp


def random_params(rng, scale=1.0):
    P = np.zeros(mlp.NPARAM)
    P[mlp.OFF_W1:mlp.OFF_B1] = rng.uniform(-1, 1, mlp.NH * mlp.NIN) / np.sqrt(mlp.NIN) * scale
    P[mlp.OFF_W2:mlp.OFF_B2] = rng.uniform(-1, 1, mlp.NH * mlp.NH) / 8.0 * scale
    P[mlp.OFF_W3:mlp.OFF_B3] = rng.uniform(-1, 1, mlp.NH) / 8.0 * scale
    P[mlp.OFF_B1:mlp.OFF_W2] = rng.normal(0, 0.1, mlp.NH)
    P[mlp.OFF_B2:mlp.OFF_W3] = rng.normal(0, 0.1, mlp.NH)
    P[mlp.OFF_B3] = 0.1
    return P


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -3.14159, 1e-3, 0.0])
    r = mlp.to_bf16(x)
    assert r[0] == 1.0 and r[5] == 0.0
    assert r[1] == 1.0                     # tie: rounds to even
    assert r[2] == 1.0 + 2 ** -7           # above the tie
    assert abs(r[3] + 3.140625) < 1e-12
    assert abs(r[4] - 1e-3) / 1e-3 < 2 ** -8


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(5)
    P = random_params(rng)
    X = rng.normal(size=(24, mlp.NIN))
    y = (rng.uniform(size=24) < 0.4).astype(float)
    loss, g = mlp.loss_and_grad(P, X, y, bf16=False)
    idx = np.concatenate([rng.choice(np.arange(mlp.OFF_W1, mlp.OFF_B1), 20),
                          rng.choice(np.arange(mlp.OFF_B1, mlp.OFF_W2), 5),
                          rng.choice(np.arange(mlp.OFF_W2, mlp.OFF_B2), 20),
                          rng.choice(np.arange(mlp.OFF_B2, mlp.NPARAM), 10), [mlp.OFF_B3]])
    h = 1e-6
    for i in idx:
        Pp, Pm = P.copy(), P.copy()
        Pp[i] += h
        Pm[i] -= h
        fd = (mlp.loss_and_grad(Pp, X, y, False)[0] - mlp.loss_and_grad(Pm, X, y, False)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])) + 1e-8, (i, fd, g[i])


def test_adamw_step_moves_against_gradient():
    rng = np.random.default_rng(1)
    P = random_params(rng)
    G = rng.normal(size=mlp.NPARAM)
    P1, M, V = mlp.adamw_step(P, G, np.zeros_like(P), np.zeros_like(P), 1, 1e-3, 0.0)
    assert np.all(np.sign(P - P1)[G != 0] == np.sign(G[G != 0]))
    big = np.abs(G) > 1e-3
    assert np.allclose(np.abs(P - P1)[big], 1e-3, rtol=1e-4)   # first step: lr * sign(g)
