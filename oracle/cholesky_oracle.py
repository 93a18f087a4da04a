"""CPU restatement of the reference's modified Cholesky decomposition
(integrals.py:3-46).  TEST INFRASTRUCTURE ONLY: the checker for the
engine's afq_modified_cholesky.  Pinned against the reference function's
own outputs (tests/golden/cholesky.npz, made by
tests/golden/make_chol_golden.py).

Steps kept alike to the reference (the result must be the reference's):
pivot on the largest diagonal, v_0 = M[nu] / sqrt(d[nu]); while the
residual pivot exceeds max_error and fewer than size - 1 vectors were
made: update the diagonal approximation, pivot on the largest |residual|,
project the pivot row; the last vector made is not returned.
"""
from __future__ import annotations

import numpy as np


def modified_cholesky(mat: np.ndarray, max_error: float = 1e-6) -> np.ndarray:
    mat = np.asarray(mat, dtype=np.float64)
    size = mat.shape[0]
    norb = int(((-1 + (1 + 8 * size) ** 0.5) / 2))
    diag = np.diagonal(mat).copy()
    vecs = [None] * size
    nu = int(np.argmax(diag))
    dmax = diag[nu]
    vecs[0] = mat[nu] / np.sqrt(dmax)
    approx = np.zeros(size)
    k = 0
    while abs(dmax) > max_error and k + 1 < size:
        approx = approx + vecs[k] * vecs[k]
        res = diag - approx
        nu = int(np.argmax(np.abs(res)))
        dmax = abs(res[nu])
        proj = np.zeros(size)
        for i in range(k + 1):  # ascending, as the engine sums
            proj = proj + vecs[i][nu] * vecs[i]
        vecs[k + 1] = (mat[nu] - proj) / np.sqrt(dmax + 1e-10)
        k += 1
    out = np.zeros((k, norb, norb))
    iu = [(m, q) for m in range(norb) for q in range(m + 1)]
    for c in range(k):
        for t, (m, q) in enumerate(iu):
            out[c, m, q] = out[c, q, m] = vecs[c][t]
    return out


def packed_eri(chol: np.ndarray) -> np.ndarray:
    """4-fold packed ERI matrix M[(ij), (kl)] = sum_g L_g[i, j] L_g[k, l]
    (i >= j, k >= l, row-major triangle order) of symmetric vectors L_g."""
    n = chol.shape[1]
    idx = [(m, q) for m in range(n) for q in range(m + 1)]
    rows = np.array([[chol[g, m, q] for (m, q) in idx] for g in range(chol.shape[0])])
    return rows.T @ rows
