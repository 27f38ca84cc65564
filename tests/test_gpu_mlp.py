"""Learned refinement indicator on the GPU (csrc/ffv_mlp.cu) against its CPU restatement
(oracle/mlp.py): forward probabilities, the gradient of the loss (the restatement rounds to
BF16 where the tensor-core kernels do; the rest is FP32 accumulation, hence the 5e-3
tolerance relative to the largest gradient entry of each parameter block), one AdamW step
and the feature gather."""
import numpy as np
import pytest
import torch

from conftest import load_golden, m5_params
from helpers import mesh_from_golden

from forestfv_public_gb300 import Solver
from forestfv_public_gb300.indicator import KIN, Indicator
from oracle import mlp

pytestmark = pytest.mark.gpu
BLOCKS = [(mlp.OFF_W1, mlp.OFF_B1), (mlp.OFF_B1, mlp.OFF_W2), (mlp.OFF_W2, mlp.OFF_B2),
          (mlp.OFF_B2, mlp.OFF_W3), (mlp.OFF_W3, mlp.OFF_B3), (mlp.OFF_B3, mlp.NPARAM)]


def random_params(rng):
    P = np.zeros(mlp.NPARAM)
    P[mlp.OFF_W1:mlp.OFF_B1] = rng.uniform(-1, 1, mlp.NH * mlp.NIN) / np.sqrt(mlp.NIN) * 2
    P[mlp.OFF_W2:mlp.OFF_B2] = rng.uniform(-1, 1, mlp.NH * mlp.NH) / 8.0 * 2
    P[mlp.OFF_W3:mlp.OFF_B3] = rng.uniform(-1, 1, mlp.NH) / 8.0 * 3
    P[mlp.OFF_B1:mlp.OFF_W2] = rng.normal(0, 0.2, mlp.NH)
    P[mlp.OFF_B2:mlp.OFF_W3] = rng.normal(0, 0.2, mlp.NH)
    P[mlp.OFF_B3] = -0.3
    return P.astype(np.float32)


def data(rng, n):
    Xf = mlp.to_bf16(rng.normal(size=(n, mlp.NIN)))
    Xp = np.zeros((n, KIN), np.float32)
    Xp[:, :mlp.NIN] = Xf
    X = torch.from_numpy(Xp).to(torch.bfloat16).cuda()
    y = (rng.uniform(size=n) < 0.3).astype(np.float32)
    return Xf, X, y, torch.from_numpy(y).cuda()


def test_forward_matches_oracle(built_lib):
    rng = np.random.default_rng(2)
    ind = Indicator(seed=3)
    P = random_params(rng)
    ind.set_params(P)
    Xf, X, _, _ = data(rng, 1000)  # not a multiple of 16
    p = ind.forward(X).cpu().numpy()
    ref, _ = mlp.forward(P.astype(np.float64), Xf)
    # an FP32-vs-FP64 difference can move a hidden value across a BF16 rounding boundary
    assert np.abs(p - ref).max() < 2e-3 and np.abs(p - ref).mean() < 1e-4
    ind.close()


def test_forward_many_tiles_matches_oracle(built_lib):
    """More 128-row tiles than the inference kernel has CTAs (each CTA loops over several),
    the last tile partial."""
    rng = np.random.default_rng(4)
    ind = Indicator(seed=3)
    P = random_params(rng)
    ind.set_params(P)
    Xf, X, _, _ = data(rng, 200_003)
    p = ind.forward(X).cpu().numpy()
    ref, _ = mlp.forward(P.astype(np.float64), Xf)
    assert np.abs(p - ref).max() < 2e-3 and np.abs(p - ref).mean() < 1e-4
    ind.close()


@pytest.mark.parametrize("n", [1, 5, 127, 128, 129])
def test_forward_partial_tile_matches_oracle(n, built_lib):
    """Fewer rows than one 128-row tile, exactly one, and one more: the rows past n are zero
    in the tile and never written."""
    rng = np.random.default_rng(100 + n)
    ind = Indicator(seed=3)
    P = random_params(rng)
    ind.set_params(P)
    Xf, X, _, _ = data(rng, n)
    p = ind.forward(X).cpu().numpy()
    ref, _ = mlp.forward(P.astype(np.float64), Xf)
    assert p.shape == (n,) and np.abs(p - ref).max() < 2e-3
    ind.close()


def test_predict_equals_forward_of_features(built_lib):
    """ffv_mlp_predict (stencil gather fused with the network) gives the bits of
    ffv_mlp_forward on the rows of ffv_mlp_features."""
    g = load_golden("m5_wall_amr")
    m = mesh_from_golden(g)
    q = m5_params(g)
    s = Solver(model=5, gamma=q["gamma"], pinf=q["pinf"], mu=q["mu"], amin=q["amin"],
               avf_lim=q["avf_lim"], prelax=q["prelax"])
    s.set_mesh(m)
    s.upload_state(np.ascontiguousarray(g["S_final"].T))
    ind = Indicator(seed=5)
    ind.set_params(random_params(np.random.default_rng(11)))
    F = ind.fields(s).cpu().numpy().astype(np.float64)
    ind.set_norm(F.mean(axis=1), F.std(axis=1) + 1e-3)
    p = ind.predict(s)
    pf = ind.forward(ind.features(s)).cpu().numpy()
    assert np.array_equal(p, pf)
    ind.close()
    s.close()


@pytest.mark.parametrize("B", [16, 1000, 8192])
def test_gradient_matches_oracle(B, built_lib):
    rng = np.random.default_rng(B)
    ind = Indicator(seed=3)
    P = random_params(rng)
    ind.set_params(P)
    Xf, X, y, yd = data(rng, B)
    g, loss = ind.grad(X, yd)
    lref, gref = mlp.loss_and_grad(P.astype(np.float64), Xf, y)
    assert abs(loss - lref) <= 1e-4 * max(1.0, lref)
    for a, b in BLOCKS:
        scale = np.abs(gref[a:b]).max()
        err = np.abs(g[a:b] - gref[a:b]).max() / scale
        assert err < 5e-3, (a, b, err)
    ind.close()


def sample_rows(seed, step, B, N):
    """The kernels' hashed batch draw (splitmix64 finaliser), restated."""
    M = (1 << 64) - 1
    i = np.arange(B, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = (np.uint64(seed) + np.uint64(0x9E3779B97F4A7C15) *
             (np.uint64((step * 1315423911) & M) + i + np.uint64(1)))
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z ^= z >> np.uint64(31)
    return (z % np.uint64(N)).astype(np.int64)


def test_adamw_steps_match_oracle(built_lib):
    rng = np.random.default_rng(9)
    ind = Indicator(seed=3)
    P = random_params(rng)
    ind.set_params(P)
    N, B = 3000, 512
    Xf, X, y, yd = data(rng, N)
    ind.train(X, yd, steps=2, batch=B, lr=1e-3, wd=1e-2, seed=77)
    Pr = P.astype(np.float64)
    M = np.zeros_like(Pr)
    V = np.zeros_like(Pr)
    gmin = np.full(mlp.NPARAM, np.inf)
    for t in range(2):
        rows = sample_rows(77, t, B, N)
        _, G = mlp.loss_and_grad(Pr, Xf[rows], y[rows])
        for a, b in BLOCKS:
            gmin[a:b] = np.minimum(gmin[a:b], np.abs(G[a:b]) / np.abs(G[a:b]).max())
        Pr, M, V = mlp.adamw_step(Pr, G, M, V, t + 1, 1e-3, 1e-2)
    Pg = ind.params()
    # the first steps move every parameter by about lr whatever its gradient's size, so a
    # parameter whose gradient is at rounding level can move either way: compare the
    # moves where the gradient is at least 1 % of its block's largest in both steps
    move_g, move_r = Pg - P, Pr - P
    sig = gmin > 1e-2
    assert sig.mean() > 0.5
    assert np.abs(move_g - move_r)[sig].max() < 2e-5
    assert (np.abs(move_g - move_r) < 2e-5).mean() > 0.99
    ind.close()


def test_training_reduces_loss(built_lib):
    rng = np.random.default_rng(4)
    n = 20000
    Xf = mlp.to_bf16(rng.normal(size=(n, mlp.NIN)))
    y = ((Xf[:, 3] + 0.5 * Xf[:, 70] - Xf[:, 100]) > 0.3).astype(np.float32)
    Xp = np.zeros((n, KIN), np.float32)
    Xp[:, :mlp.NIN] = Xf
    X = torch.from_numpy(Xp).to(torch.bfloat16).cuda()
    yd = torch.from_numpy(y).cuda()
    ind = Indicator(seed=5)
    losses = ind.train(X, yd, steps=300, batch=2048, lr=3e-3, wd=1e-4, seed=11)
    assert losses[-20:].mean() < 0.3 * losses[:5].mean()
    p = ind.forward(X).cpu().numpy()
    assert ((p > 0.5) == (y > 0.5)).mean() > 0.95
    ind.close()


def test_features_match_oracle(built_lib):
    g = load_golden("m5_wall_amr")
    m = mesh_from_golden(g)
    q = m5_params(g)
    s = Solver(model=5, gamma=q["gamma"], pinf=q["pinf"], mu=q["mu"], amin=q["amin"],
               avf_lim=q["avf_lim"], prelax=q["prelax"])
    s.set_mesh(m)
    s.upload_state(np.ascontiguousarray(g["S_final"].T))
    ind = Indicator()
    F = ind.fields(s).cpu().numpy().astype(np.float64)
    mean, std = F.mean(axis=1), F.std(axis=1) + 1e-3
    ind.set_norm(mean, std)
    X = ind.features(s).float().cpu().numpy()
    ref = mlp.to_bf16(mlp.stencil_features(m.export(), F.astype(np.float32).astype(np.float64),
                                           mean.astype(np.float32), std.astype(np.float32)))
    assert np.array_equal(X[:, mlp.NIN:], np.zeros((m.n, KIN - mlp.NIN)))
    assert np.abs(X[:, :mlp.NIN] - ref).max() <= 1e-2 * max(1.0, np.abs(ref).max())
    ind.close()
    s.close()


def test_fields_match_host_eos(built_lib):
    """The indicator's per-cell fields (FP32 with double-float pressure recovery) against the
    host float64 restatement of the reference's equation of state."""
    from forestfv_public_gb300.fields import primitives
    g = load_golden("m5_wall_amr")
    m = mesh_from_golden(g)
    q = m5_params(g)
    s = Solver(model=5, gamma=q["gamma"], pinf=q["pinf"], mu=q["mu"], amin=q["amin"],
               avf_lim=q["avf_lim"], prelax=q["prelax"])
    s.set_mesh(m)
    S = np.ascontiguousarray(g["S_final"].T)
    s.upload_state(S)
    ind = Indicator()
    F = ind.fields(s).cpu().numpy().astype(np.float64)
    ref = primitives(S, q["gamma"], q["pinf"], q["mu"], q["amin"])
    N = len(q["gamma"])
    u = np.linalg.norm(S[N:N + 3], axis=0) / ref["rho"]
    assert np.abs(F[0] - np.log(ref["rho"])).max() <= 1e-6
    hi = ref["p"] > 100.0  # below, log max(p, 1 Pa) of near-floor pressures is ill-conditioned
    assert np.abs(F[1][hi] - np.log(ref["p"][hi])).max() <= 1e-4
    assert np.abs(F[2] - ref["alpha"][0]).max() <= 1e-6
    assert np.abs(F[3] - u).max() <= 1e-5 * max(1.0, u.max())
    # the FP32 elastic deviator: for strains ~1e-6, dev(G^2) - |G|^(1/3) dev(G) is a
    # difference of O(1) numbers, resolved to ~1 % in FP32 -- ample for a network input
    assert np.abs(F[4] - ref["vm"]).max() <= 1e-2 * max(1.0, ref["vm"].max())
    assert np.all(F[4][ref["vm"] == 0.0] == 0.0)
    ind.close()
    s.close()


@pytest.mark.parametrize("threshold", [0.2, 0.5])
def test_marks_equal_predicted_probabilities(threshold, built_lib):
    """ffv_mlp_mark (on the device, nothing copied back) gives the marks of
    ffv_mlp_predict's probabilities against the threshold, accumulation OR-ing into earlier
    marks."""
    g = load_golden("m5_wall_amr")
    m = mesh_from_golden(g)
    q = m5_params(g)
    s = Solver(model=5, gamma=q["gamma"], pinf=q["pinf"], mu=q["mu"], amin=q["amin"],
               avf_lim=q["avf_lim"], prelax=q["prelax"])
    s.set_mesh(m)
    s.upload_state(np.ascontiguousarray(g["S_final"].T))
    ind = Indicator(seed=5)
    ind.set_params(random_params(np.random.default_rng(9)))
    F = ind.fields(s).cpu().numpy().astype(np.float64)
    ind.set_norm(F.mean(axis=1), F.std(axis=1) + 1e-3)
    p = ind.predict(s)
    assert 0 < (p > threshold).sum() < m.n  # both outcomes occur
    marks = torch.zeros(m.n, dtype=torch.uint8, device="cuda")
    ind.mark(s, threshold, marks, accumulate=False)
    s.sync()
    assert np.array_equal(marks.cpu().numpy(), (p > threshold).astype(np.uint8))
    prior = torch.from_numpy((np.arange(m.n) % 7 == 0).astype(np.uint8)).cuda()
    ind.mark(s, threshold, prior, accumulate=True)
    s.sync()
    assert np.array_equal(prior.cpu().numpy(),
                          ((p > threshold) | (np.arange(m.n) % 7 == 0)).astype(np.uint8))
    ind.close()
    s.close()
