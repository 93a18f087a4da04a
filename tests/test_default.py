"""default.Rhf (default.py:15-47 of the reference) without pyscf: the MO-basis
two-electron integrals are passed in, packed the way pyscf packs them."""
import numpy as np
import pytest

from ad_afqmc_prototype_gb300.default import Rhf, restore_4fold
from oracle.cholesky_oracle import packed_eri


def _synthetic_mf(n=8, nocc=3, g=10, seed=5):
    """A mean-field-like object: MO integrals from symmetric Cholesky vectors,
    an orthogonal AO->MO transform, h1 with the occupied orbitals lowest."""
    rng = np.random.default_rng(seed)
    b = rng.normal(size=(g, n, n))
    L = 0.5 * (b + np.swapaxes(b, 1, 2)) * (0.3 * np.exp(-np.arange(g) / 3.0))[:, None, None]
    a = rng.normal(size=(n, n))
    h1_mo = np.diag(np.linspace(-2.0, 0.5, n)) + 0.05 * (a + a.T)
    U = np.linalg.qr(rng.normal(size=(n, n)))[0]

    class Mol:
        nao = n
        nelec = (nocc, nocc)
        nelectron = 2 * nocc

    class MF:
        mol = Mol()
        mo_coeff = U

        def get_hcore(self):
            return U @ h1_mo @ U.T

        def energy_nuc(self):
            return 1.25

    eri_full = np.einsum("gij,gkl->ijkl", L, L)
    return MF(), eri_full, L, h1_mo


def test_restore_4fold_forms_agree():
    _, eri_full, L, _ = _synthetic_mf()
    n = eri_full.shape[0]
    e4 = restore_4fold(eri_full, n)
    np.testing.assert_allclose(e4, packed_eri(L), rtol=0, atol=1e-14)
    np.testing.assert_array_equal(restore_4fold(e4, n), e4)
    r, c = np.tril_indices(e4.shape[0])
    np.testing.assert_array_equal(restore_4fold(e4[r, c], n), e4)
    with pytest.raises(ValueError):
        restore_4fold(np.zeros((3, 3)), n)


def test_rhf_without_pyscf_needs_eri():
    try:
        import pyscf  # noqa: F401
        pytest.skip("pyscf is installed")
    except ImportError:
        pass
    mf, _, _, _ = _synthetic_mf()
    with pytest.raises(ImportError, match="eri="):
        Rhf(mf)


@pytest.mark.gpu
def test_rhf_from_integrals_runs_the_driver(cuda):
    mf, eri_full, L, h1_mo = _synthetic_mf()
    r = Rhf(mf, eri=eri_full)
    n = eri_full.shape[0]
    chol = r.ham_data.chol.cpu().numpy()
    # the Cholesky vectors reproduce the integrals to the decomposition's threshold
    np.testing.assert_allclose(np.einsum("gij,gkl->ijkl", chol, chol), eri_full, atol=1e-5)
    np.testing.assert_allclose(r.ham_data.h1.cpu().numpy(), h1_mo, atol=1e-13)
    assert r.ham_data.h0 == 1.25
    assert tuple(r.trial_data.mo_coeff.shape) == (n, 3)
    assert r.params.n_eql_blocks == 20 and r.params.n_blocks == 200
    from dataclasses import replace
    # 200 sampling blocks as in the reference's default: its progress lines run the blocking
    # analysis every n_blocks / 10 blocks, which needs 20 blocks at least
    r.params = replace(r.params, n_eql_blocks=2, n_blocks=200, n_walkers=32, n_prop_steps=10, seed=3)
    mu, se, e, w = r.kernel()
    assert np.isfinite(float(mu)) and np.all(np.isfinite(e.numpy()))
    # the trial's own energy (walkers start at the trial) is the first equilibration entry
    from oracle import afqmc_oracle as O
    c = np.eye(n, 3)
    ctx = O.build_meas_ctx(h1_mo, chol, c)
    e_trial = float(np.real(O.energy_r(c[None].astype(complex), 1.25, ctx, c))[0])
    assert abs(float(e[0]) - e_trial) < 1e-10
