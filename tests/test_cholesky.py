"""Modified Cholesky decomposition (integrals.py:3-46): the oracle against
the reference's own outputs (golden), the engine's afq_modified_cholesky
against both, and the reconstruction property at larger sizes.

Tolerance: 1e-10 relative to the largest vector entry (the projections sum
in a different order than the reference's BLAS dot; the pivot sequence is
the same)."""
import os

import numpy as np
import pytest

from oracle import cholesky_oracle as CO

GOLD = os.path.join(os.path.dirname(__file__), "golden", "cholesky.npz")


def _cases():
    z = np.load(GOLD)
    k = 0
    while f"mat{k}" in z:
        yield z[f"mat{k}"], float(z[f"err{k}"]), z[f"chol{k}"]
        k += 1


def test_oracle_matches_reference_golden():
    for M, err, ref in _cases():
        got = CO.modified_cholesky(M, err)
        assert got.shape == ref.shape
        np.testing.assert_allclose(got, ref, rtol=0, atol=1e-10 * np.abs(ref).max())


@pytest.mark.gpu
def test_engine_matches_golden_and_oracle(cuda):
    from ad_afqmc_prototype_gb300.integrals import modified_cholesky
    for M, err, ref in _cases():
        got = modified_cholesky(M, max_error=err)
        assert got.shape == ref.shape, (got.shape, ref.shape)
        np.testing.assert_allclose(got, ref, rtol=0, atol=1e-10 * np.abs(ref).max())


@pytest.mark.gpu
@pytest.mark.parametrize("n,g,err", [(16, 60, 1e-8), (24, 400, 1e-5)])
def test_engine_reconstructs_larger_matrices(cuda, n, g, err):
    from ad_afqmc_prototype_gb300.integrals import modified_cholesky_device
    rng = np.random.default_rng(n)
    b = rng.normal(size=(g, n, n))
    L = 0.5 * (b + np.swapaxes(b, 1, 2)) * np.exp(-np.arange(g) / 20.0)[:, None, None]
    M = CO.packed_eri(L)
    got = modified_cholesky_device(M, max_error=err).cpu().numpy()
    ora = CO.modified_cholesky(M, err)
    assert got.shape == ora.shape
    np.testing.assert_allclose(got, ora, rtol=0, atol=1e-9 * np.abs(ora).max())
    # the residual diagonal of M - sum_c v_c v_c^T is below the stopping threshold
    iu = [(m, q) for m in range(n) for q in range(m + 1)]
    V = np.array([[got[c, m, q] for (m, q) in iu] for c in range(got.shape[0])])
    resid = np.diagonal(M - V.T @ V)
    assert np.abs(resid).max() < 50 * err, np.abs(resid).max()
