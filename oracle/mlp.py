"""CPU restatement of the learned refinement indicator (test infrastructure: the oracle for
the CUDA kernels in forestfv_public_gb300/csrc/ffv_mlp.cu, never the thing measured).

The indicator has no counterpart in the reference; this restates its equations in float64
numpy: a 135-64-64-1 perceptron, GELU (erf form) hidden layers, sigmoid output, mean binary
cross-entropy, AdamW.  `bf16=True` rounds to BF16 (round to nearest even) at the points the
tensor-core kernels do -- the inputs, W1, W2, the first hidden layer and the two
pre-activation gradients that enter tensor-core products -- so that the GPU results can be
compared within FP32 accumulation error; `bf16=False` is the exact float64 network, used to
check the gradient by finite differences.
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf

NIN, NH = 135, 64
OFF_W1, OFF_B1 = 0, NH * NIN
OFF_W2 = OFF_B1 + NH
OFF_B2 = OFF_W2 + NH * NH
OFF_W3 = OFF_B2 + NH
OFF_B3 = OFF_W3 + NH
NPARAM = OFF_B3 + 1


def to_bf16(x) -> np.ndarray:
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    f = np.asarray(x, dtype=np.float32)
    b = f.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(P):
    P = np.asarray(P, dtype=np.float64)
    return (P[OFF_W1:OFF_B1].reshape(NH, NIN), P[OFF_B1:OFF_W2], P[OFF_W2:OFF_B2].reshape(NH, NH),
            P[OFF_B2:OFF_W3], P[OFF_W3:OFF_B3], P[OFF_B3])


def gelu(x):
    return 0.5 * x * (1.0 + erf(x / np.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + erf(x / np.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / np.sqrt(2.0 * np.pi)


def forward(P, X, bf16: bool = True):
    """X [B, 135] -> (probabilities, cache)."""
    W1, b1, W2, b2, w3, b3 = unpack(P)
    r = to_bf16 if bf16 else (lambda a: np.asarray(a, np.float64))
    Xr, W1r, W2r = r(X), r(W1), r(W2)
    a1 = Xr @ W1r.T + b1
    h1 = r(gelu(a1))
    a2 = h1 @ W2r.T + b2
    h2 = gelu(a2)
    z = h2 @ w3 + b3
    p = 1.0 / (1.0 + np.exp(-z))
    return p, dict(X=Xr, W2=W2r, a1=a1, h1=h1, a2=a2, h2=h2, z=z)


def loss_and_grad(P, X, y, bf16: bool = True):
    """Mean binary cross-entropy and its gradient (NPARAM vector)."""
    W1, b1, W2, b2, w3, b3 = unpack(P)
    r = to_bf16 if bf16 else (lambda a: np.asarray(a, np.float64))
    p, c = forward(P, X, bf16)
    B = len(y)
    eps = 1e-12
    loss = -np.mean(y * np.log(np.maximum(p, eps)) + (1 - y) * np.log(np.maximum(1 - p, eps)))
    dz = (p - y) / B
    g = np.zeros(NPARAM)
    g[OFF_W3:OFF_B3] = c["h2"].T @ dz
    g[OFF_B3] = dz.sum()
    da2 = dz[:, None] * w3[None, :] * gelu_grad(c["a2"])
    g[OFF_B2:OFF_W3] = da2.sum(0)
    da2r = r(da2)
    g[OFF_W2:OFF_B2] = (da2r.T @ c["h1"]).reshape(-1)
    dh1 = da2r @ c["W2"]
    da1 = dh1 * gelu_grad(c["a1"])
    g[OFF_B1:OFF_W2] = da1.sum(0)
    g[OFF_W1:OFF_B1] = (r(da1).T @ c["X"]).reshape(-1)
    return loss, g


def weight_mask() -> np.ndarray:
    """Parameters under decoupled weight decay: W1, W2, w3 (not the biases)."""
    m = np.zeros(NPARAM, bool)
    m[OFF_W1:OFF_B1] = True
    m[OFF_W2:OFF_B2] = True
    m[OFF_W3:OFF_B3] = True
    return m


def adamw_step(P, G, M, V, t, lr, wd, b1=0.9, b2=0.999, eps=1e-8):
    """One AdamW step (t counts from 1); returns new (P, M, V)."""
    M = b1 * M + (1 - b1) * G
    V = b2 * V + (1 - b2) * G * G
    P = np.where(weight_mask(), P - lr * wd * P, P)
    P = P - lr * (M / (1 - b1 ** t)) / (np.sqrt(V / (1 - b2 ** t)) + eps)
    return P, M, V


# ----------------------------------------------------------------------------- features
def face_step(ex: dict, c: int, f: int) -> int:
    """The cell across face f of cell c in the reference-form geometry of ffv_mesh_export:
    a boundary face keeps c, four finer neighbours give the first."""
    if ex["bc"][c, f] != 0:
        return c
    return int(ex["nb"][c, f, 0])


# reference-form face index of the steps -x, +x, -y, +y, -z, +z
STEP_FACE = {(0, -1): 0, (0, 1): 2, (1, -1): 3, (1, 1): 1, (2, -1): 4, (2, 1): 5}


def stencil_features(ex: dict, F: np.ndarray, mean, stdev) -> np.ndarray:
    """Feature rows [n, 135] (float64, before BF16 rounding) of fields F [5, n]."""
    n = F.shape[1]
    out = np.zeros((n, NIN))
    for c in range(n):
        for o in range(27):
            d = (o % 3 - 1, (o // 3) % 3 - 1, o // 9 - 1)
            e = c
            for ax in range(3):
                if d[ax]:
                    e = face_step(ex, e, STEP_FACE[(ax, d[ax])])
            out[c, o * 5:o * 5 + 5] = (F[:, e] - np.asarray(mean)) / np.asarray(stdev)
    return out
