"""Per-particle stress of the reference's two constitutive laws, evaluated in FP64
on the host from a particle state, and the relative error measure used to compare
the GPU state with the FP64 oracle's.

TEST INFRASTRUCTURE ONLY (the checker): used by tests/ and bench.py's error leg.

    snow  (HybridSolver.cpp:314-325): P = 2 mu (F - R) + lambda (J - 1) J F^-T,
          mu, lambda scaled by exp(xi (1 - J_P))
    sand  (HybridSolver.cpp:326-339): P = U (2 mu S^-1 ln S + lambda tr(ln S) S^-1) V^T
    both: vol P F^T (the stress the force pass scatters, HS:352)
"""
from __future__ import annotations

import numpy as np


def stress(F, plastic, mat, prm, vol=1.0):
    """vol P(F) F^T per particle; F: (N, 3, 3), plastic: J_P (snow) / q (sand),
    mat: material tags, prm: aep_params."""
    F = np.asarray(F, np.float64)
    out = np.zeros_like(F)
    mat = np.asarray(mat)
    snow = mat == 0
    sand = mat == 1
    if snow.any() or sand.any():
        U, S, Vt = np.linalg.svd(F)
    if snow.any():
        E, nu, xi = prm.snow.E, prm.snow.nu, prm.snow.xi
        lam0, mu0 = E * nu / (1 + nu) / (1 - 2 * nu), E / 2 / (1 + nu)
        hard = np.exp(xi * (1 - np.asarray(plastic, np.float64)[snow]))
        Fs = F[snow]
        R = U[snow] @ Vt[snow]
        J = np.linalg.det(Fs)
        cof = np.linalg.inv(Fs).transpose(0, 2, 1) * J[:, None, None]
        P = 2 * (mu0 * hard)[:, None, None] * (Fs - R) + ((lam0 * hard) * (J - 1))[:, None, None] * cof
        out[snow] = P @ Fs.transpose(0, 2, 1)
    if sand.any():
        E, nu = prm.sand.E, prm.sand.nu
        lam, mu = E * nu / (1 + nu) / (1 - 2 * nu), E / 2 / (1 + nu)
        ln = np.log(S[sand])
        d = (2 * mu * ln + lam * ln.sum(1, keepdims=True)) / S[sand]
        P = U[sand] @ (d[:, :, None] * Vt[sand])
        out[sand] = P @ F[sand].transpose(0, 2, 1)
    return out * np.asarray(vol, np.float64).reshape(-1, 1, 1)


def rel_stats(a, b, floor_frac: float = 1e-2):
    """Per-particle |P_a - P_b|_F / max(|P_b|_F, floor_frac * rms |P_b|) with median,
    p99 and max, and the error relative to the rms stress (p99_rms, max_rms)."""
    na = np.linalg.norm((np.asarray(a) - np.asarray(b)).reshape(len(a), -1), axis=1)
    nb = np.linalg.norm(np.asarray(b).reshape(len(b), -1), axis=1)
    rms = float(np.sqrt(np.mean(nb ** 2))) if len(nb) else 0.0
    if not len(nb) or rms == 0.0:
        return {"median": 0.0, "p99": 0.0, "max": 0.0, "p99_rms": 0.0, "max_rms": 0.0, "particles": int(len(nb)),
                "floor": 0.0}
    floor = floor_frac * rms
    r = na / np.maximum(nb, floor)
    return {"median": float(np.median(r)), "p99": float(np.percentile(r, 99)), "max": float(r.max()),
            "p99_rms": float(np.percentile(na, 99) / rms), "max_rms": float(na.max() / rms),
            "particles": int(len(r)), "floor": float(floor)}
