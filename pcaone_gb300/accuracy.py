"""Accuracy measures reported next to the timings.

The benchmark spec's bars are the largest principal angle between subspaces
(sin, <= 1e-6) and the relative eigenvalue error (<= 1e-8) of the PCs against
an FP64 result.  Only the leading PCs separated from the next one by a
relative eigen-gap above 5% are compared: near-degenerate noise PCs are not
determined by a few power iterations (the reference's own FP64 methods
disagree on them).
"""
from __future__ import annotations

import numpy as np


def well_separated(S: np.ndarray, gap: float = 0.05) -> int:
    """Number of leading components whose squared singular value lies above
    the next one by a relative gap larger than ``gap`` (the last such index)."""
    e = np.asarray(S, dtype=np.float64) ** 2
    n = 0
    for i in range(len(e) - 1):
        if (e[i] - e[i + 1]) / e[i] > gap:
            n = i + 1
    return n


def sin_largest_angle(A: np.ndarray, B: np.ndarray) -> float:
    """sin of the largest principal angle between span(A) and span(B), as
    ||(I - Qa Qa^T) Qb||_2 (no arccos of cosines close to 1)."""
    Qa = np.linalg.qr(A)[0]
    Qb = np.linalg.qr(B)[0]
    return float(np.linalg.norm(Qb - Qa @ (Qa.T @ Qb), 2))


def eig_relerr(S: np.ndarray, Sref: np.ndarray) -> np.ndarray:
    """Relative error of the eigenvalues S^2 against Sref^2."""
    return np.abs(S ** 2 - Sref ** 2) / np.abs(Sref ** 2)


def compare_pcs(U, S, V, Uref, Sref, Vref, n: int | None = None) -> dict:
    """Errors of (U, S, V) against a reference on its well-separated PCs."""
    if n is None:
        n = max(1, well_separated(Sref))
    out = {"pcs_compared": int(n),
           "sin_angle_u": sin_largest_angle(U[:, :n], Uref[:, :n]),
           "eig_relerr": float(np.max(eig_relerr(S[:n], Sref[:n])))}
    if V is not None and Vref is not None:
        out["sin_angle_v"] = sin_largest_angle(V[:, :n], Vref[:, :n])
    return out
