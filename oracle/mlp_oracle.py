"""FP64 numpy restatement of the learned return map's network (forward, loss and
backward) for the gradient checks of the GPU kernels.

TEST INFRASTRUCTURE ONLY (the checker): used by tests/ only.  With bf16=True the
weights and every GEMM input are rounded to bfloat16 (round to nearest even) at the
same points as the tensor-core kernels (aep_mlp.cu), so the two differ only by FP32
accumulation order: the hidden activations and the output gradients are rounded,
and the FP32 input features enter the first layer as the sum of two bfloat16
values, hi = bf16(x) and lo = bf16(x - hi), both against the feature's weight (the
kernels' A operand carries hi and lo in separate columns).  With bf16=False it is
the exact FP64 function, which the tests pin against central finite differences.

Packed parameters (9928 floats): W1^T [64][16], W2^T [64][64], W3^T [64][64],
W4^T [8][64], b1 [64], b2 [64], b3 [64], b4 [8].  Records: [ln s0, ln s1, ln s2,
q, material, d0, d1, d2] (material 0 snow, 1 sand); cloth records (material 2)
carry [r13, r23, r33 - 1, cap ratio, 2, change of (r13, r23, r33)].  Features and
targets are scaled per record (sand and cloth by 1/|first three|, snow by 50;
column 3 is q x 100 for sand, the cap ratio for cloth), as the kernels do
(aep_mlp.cuh mlp_features).
"""
from __future__ import annotations

import numpy as np

LN_SCALE = 50.0
Q_SCALE = 100.0
LAYOUT = [("w1t", (64, 16)), ("w2t", (64, 64)), ("w3t", (64, 64)), ("w4t", (8, 64)),
          ("b1", (64,)), ("b2", (64,)), ("b3", (64,)), ("b4", (8,))]


def unpack(p):
    out, off = {}, 0
    for name, shape in LAYOUT:
        k = int(np.prod(shape))
        out[name] = np.asarray(p[off:off + k], np.float64).reshape(shape)
        off += k
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], np.float64).ravel() for name, _ in LAYOUT])


def bf16(x):
    """Round float32 values to bfloat16 (nearest, ties to even); returns float64."""
    a = np.ascontiguousarray(np.asarray(x, np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def scales(rec):
    """Per-record scaling of features and outputs: sand and cloth 1/|first three|
    (the cone projection is positively homogeneous), snow 50."""
    rec = np.asarray(rec, np.float64)
    ln = rec[:, 0:3].astype(np.float32)
    r = np.sqrt((ln * ln).sum(1, dtype=np.float32)).astype(np.float32)
    scaled = rec[:, 4].astype(int) != 0
    sc = np.full(len(rec), np.float32(LN_SCALE), np.float32)
    sc[scaled] = np.float32(1.0) / np.maximum(r[scaled], np.float32(1e-30))
    return sc


def features(rec, rnd=True):
    """The FP32 feature rows [n, 16] (7 used); with rnd, each feature as the sum of
    its bfloat16 hi and lo parts, as the first layer's tensor-core operand sees it."""
    rec = np.asarray(rec, np.float64)
    n = len(rec)
    X = np.zeros((n, 16), np.float32)
    sc = scales(rec)
    X[:, 0:3] = rec[:, 0:3].astype(np.float32) * sc[:, None]
    mat = rec[:, 4].astype(int)
    q = rec[:, 3].astype(np.float32)
    X[:, 3] = np.where(mat == 1, q * np.float32(Q_SCALE), np.where(mat == 2, q, np.float32(0.0)))
    X[:, 4] = (mat == 0)
    X[:, 5] = (mat == 1)
    X[:, 6] = (mat == 2)
    if not rnd:
        return X.astype(np.float64)
    hi = bf16(X)
    lo = bf16((X.astype(np.float64) - hi).astype(np.float32))
    return hi + lo


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, rec, bf=True):
    P = unpack(p)
    r = bf16 if bf else (lambda a: np.asarray(a, np.float64))
    W = [r(P["w1t"]), r(P["w2t"]), r(P["w3t"]), r(P["w4t"])]
    b = [P["b1"], P["b2"], P["b3"], P["b4"]]
    X = features(rec, bf)
    Z, H = [], [X]
    for l in range(3):
        z = H[-1] @ W[l].T + b[l]
        Z.append(z)
        H.append(r(silu(z)))
    Y = H[-1] @ W[3].T + b[3]
    return dict(W=W, X=X, Z=Z, H=H, Y=Y)


def loss_and_grad(p, rec, bf=True):
    rec = np.asarray(rec, np.float64)
    n = len(rec)
    f = forward(p, rec, bf)
    r = bf16 if bf else (lambda a: np.asarray(a, np.float64))
    T = rec[:, 5:8] * scales(rec)[:, None].astype(np.float64)
    diff = f["Y"][:, :3] - T
    loss = float((diff ** 2).sum() / (3.0 * n))
    dY = np.zeros((n, 8))
    dY[:, :3] = 2.0 * diff / (3.0 * n)
    dY = r(dY)
    W, Z, H = f["W"], f["Z"], f["H"]
    g = {"w4t": dY.T @ H[3], "b4": dY.sum(0)}
    dZ = r((dY @ W[3]) * dsilu(Z[2]))
    for l in (2, 1, 0):
        g[f"w{l + 1}t"] = dZ.T @ H[l]
        g[f"b{l + 1}"] = dZ.sum(0)
        if l > 0:
            dZ = r((dZ @ W[l]) * dsilu(Z[l - 1]))
    return loss, pack(g)


def predict(p, rec, bf=True):
    """Predicted corrections d (ln units), [n, 3]."""
    return forward(p, rec, bf)["Y"][:, :3] / scales(rec)[:, None].astype(np.float64)


def adam_step(p, g, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update in FP64 (the optimiser of aep_mlp_train, step t >= 1):
    m <- b1 m + (1 - b1) g, v <- b2 v + (1 - b2) g^2,
    p <- p - lr (m / (1 - b1^t)) / (sqrt(v / (1 - b2^t)) + eps).  Returns (p, m, v)."""
    g = np.asarray(g, np.float64)
    m = b1 * np.asarray(m, np.float64) + (1.0 - b1) * g
    v = b2 * np.asarray(v, np.float64) + (1.0 - b2) * g * g
    c1, c2 = 1.0 - b1 ** t, 1.0 - b2 ** t
    p = np.asarray(p, np.float64) - lr * (m / c1) / (np.sqrt(v / c2) + eps)
    return p, m, v
