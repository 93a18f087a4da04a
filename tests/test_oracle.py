"""CPU checks that pin the oracle: the reference's own known-answer tests
restated, first-principles (Fock-space) checks of its RHF kernels, and
properties of QR, the Taylor series and the comb."""
import numpy as np
import pytest
import scipy.linalg

from oracle import afqmc_oracle as O
from tests import fock
from tests import philox_ref


def _rand_orthonormal(rng, n, k, complex_=True):
    a = rng.normal(size=(n, k)) + (1j * rng.normal(size=(n, k)) if complex_ else 0)
    return np.linalg.qr(a)[0][:, :k]


def _small_ham(rng, n, g):
    a = rng.normal(size=(n, n))
    h1 = 0.5 * (a + a.T)
    b = rng.normal(size=(g, n, n))
    chol = 0.5 * (b + np.swapaxes(b, 1, 2))
    return float(rng.normal()), h1, chol


# ---- the reference's known-answer tests -------------------------------------

def test_weight_update_known_answer():
    """tests/test_prop_afqmc_step.py:46-94: h1 = chol = 0, h0 = 1, dt = 0.2,
    overlap == 1 and force bias == 0 -> weights = exp(-dt), shift = 0.1."""
    norb, nocc, nw, nf = 4, 2, 8, 3
    prob = O.make_problem(1.0, np.zeros((norb, norb)), np.zeros((nf, norb, norb)),
                          np.eye(norb, nocc), 0.2)
    # the reference test builds the prop ctx from a zero rdm1
    prob.prop_ctx = O.build_prop_ctx(1.0, np.zeros((norb, norb)), np.zeros((nf, norb, norb)),
                                     np.zeros((norb, norb)), 0.2)
    params = O.Params(dt=0.2, n_chunks=2, n_exp_terms=4, pop_control_damping=0.1)
    st = O.State(walkers=np.ones((nw, norb, nocc), complex), weights=np.ones(nw),
                 overlaps=np.ones(nw, complex), pop_control_ene_shift=0.0, e_estimate=0.0)
    fields = np.random.default_rng(0).normal(size=(nw, nf))
    out = O.afqmc_step(prob, params, st, fields,
                       force_bias_fn=lambda w: np.zeros((w.shape[0], nf), complex),
                       overlap_fn=lambda w: np.ones(w.shape[0], complex))
    np.testing.assert_allclose(out.weights, np.exp(-0.2) * np.ones(nw), rtol=1e-14)
    assert abs(out.pop_control_ene_shift - 0.1) < 1e-14
    assert out.e_estimate == 0.0


def test_energy_is_h0_for_zero_hamiltonian():
    """tests/test_trial_rhf.py:88-110."""
    rng = np.random.default_rng(3)
    norb, nocc, nchol = 5, 2, 4
    c = _rand_orthonormal(rng, norb, nocc)
    ctx = O.build_meas_ctx(np.zeros((norb, norb)), np.zeros((nchol, norb, norb)), c)
    w = (c @ (np.eye(nocc) * (1.1 + 0.2j)))[None]
    e = O.energy_r(w, 1.234, ctx, c)
    np.testing.assert_allclose(e, 1.234, atol=1e-14)


def test_meas_ctx_shapes():
    """tests/test_trial_rhf.py:35-46."""
    rng = np.random.default_rng(0)
    norb, nocc, nchol = 6, 2, 5
    h0, h1, chol = _small_ham(rng, norb, nchol)
    ctx = O.build_meas_ctx(h1, chol, _rand_orthonormal(rng, norb, nocc))
    assert ctx.rot_h1.shape == (nocc, norb)
    assert ctx.rot_chol.shape == (nchol, nocc, norb)
    assert ctx.rot_chol_flat.shape == (nchol, nocc * norb)


def test_prop_ctx_shapes():
    """tests/test_prop_chol_afqmc_ops.py:21-36."""
    rng = np.random.default_rng(0)
    h0, h1, chol = _small_ham(rng, 5, 7)
    ctx = O.build_prop_ctx(0.0, h1, chol, np.zeros((5, 5)), 0.2)
    assert ctx.mf_shifts.shape == (7,)
    assert ctx.exp_h1_half.shape == (5, 5)


# ---- first principles: mixed estimators in Fock space ------------------------

@pytest.mark.parametrize("complex_trial", [False, True])
def test_kernels_match_fock_space(complex_trial):
    rng = np.random.default_rng(11)
    n, o, g = 4, 2, 3
    h0, h1, chol = _small_ham(rng, n, g)
    chol *= 0.3
    cr, E = fock.excitation_ops(n)
    H = fock.hamiltonian(h0, h1, chol, E)
    c = _rand_orthonormal(rng, n, o, complex_trial)
    ctx = O.build_meas_ctx(h1, chol, c)
    psi_t = fock.determinant(c, cr, n)
    for k in range(3):
        w = rng.normal(size=(n, o)) + 1j * rng.normal(size=(n, o))
        psi_w = fock.determinant(w, cr, n)
        ov = np.vdot(psi_t, psi_w)
        np.testing.assert_allclose(O.overlap_r(w[None], c)[0], ov, rtol=1e-12)
        e_ref = np.vdot(psi_t, H @ psi_w) / ov
        np.testing.assert_allclose(O.energy_r(w[None], h0, ctx, c)[0], e_ref, rtol=1e-11, atol=1e-11)
        fb_ref = [np.vdot(psi_t, np.einsum("ij,ijab->ab", L, E) @ psi_w) / ov for L in chol]
        np.testing.assert_allclose(O.force_bias_r(w[None], ctx, c)[0], fb_ref, rtol=1e-11, atol=1e-12)


def test_force_bias_equals_full_green_trace():
    """fb_g = tr(L_g G) summed over spins, G = W (C^H W)^-1 C^H."""
    rng = np.random.default_rng(1)
    n, o, g = 7, 3, 5
    _, h1, chol = _small_ham(rng, n, g)
    c = _rand_orthonormal(rng, n, o)
    w = rng.normal(size=(2, n, o)) + 1j * rng.normal(size=(2, n, o))
    ctx = O.build_meas_ctx(h1, chol, c)
    fb = O.force_bias_r(w, ctx, c)
    for k in range(2):
        G = w[k] @ np.linalg.inv(c.conj().T @ w[k]) @ c.conj().T
        ref = 2.0 * np.einsum("gij,ji->g", chol, G)
        np.testing.assert_allclose(fb[k], ref, rtol=1e-12)


# ---- propagator pieces ------------------------------------------------------

def test_taylor_converges_to_expm():
    rng = np.random.default_rng(2)
    n, o = 6, 3
    v = 0.3 * (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)))
    w = rng.normal(size=(n, o)) + 1j * rng.normal(size=(n, o))
    a = 1j * np.sqrt(0.01)
    out = O.taylor_expm_action(a, v[None], w[None], 25)[0]
    np.testing.assert_allclose(out, scipy.linalg.expm(a * v) @ w, rtol=1e-13, atol=1e-14)


def test_mf_shift_sign_and_h1_eff():
    rng = np.random.default_rng(4)
    n, g = 5, 4
    h0, h1, chol = _small_ham(rng, n, g)
    c = _rand_orthonormal(rng, n, 2, complex_=False)
    rdm1 = O.get_rdm1(c)
    ctx = O.build_prop_ctx(h0, h1, chol, rdm1, 0.01)
    t = np.einsum("gij,ji->g", chol, 2 * c @ c.T)
    np.testing.assert_allclose(ctx.mf_shifts, 1j * t, rtol=1e-13)
    h1_eff = h1 - 0.5 * np.einsum("gik,gkj->ij", chol, chol) + np.einsum("g,gij->ij", t, chol)
    np.testing.assert_allclose(ctx.exp_h1_half, scipy.linalg.expm(-0.005 * h1_eff), rtol=1e-13)
    np.testing.assert_allclose(ctx.h0_prop, -h0 + 0.5 * np.sum(t * t), rtol=1e-13)


@pytest.mark.parametrize("n,o", [(12, 6), (20, 20), (9, 1)])
def test_qr_phase_convention(n, o):
    rng = np.random.default_rng(5)
    w = rng.normal(size=(3, n, o)) + 1j * rng.normal(size=(3, n, o))
    q, det_r = O.qr_phase(w)
    for k in range(3):
        np.testing.assert_allclose(q[k].conj().T @ q[k], np.eye(o), atol=1e-13)
        r = q[k].conj().T @ w[k]
        np.testing.assert_allclose(np.tril(r, -1), 0, atol=1e-12)
        d = np.diag(r)
        assert np.all(np.abs(d.imag) < 1e-12) and np.all(d.real > 0)
        np.testing.assert_allclose(det_r[k], np.prod(d), rtol=1e-12)


# ---- comb -------------------------------------------------------------------

def test_assoc_scan_dyadic_equals_sequential():
    rng = np.random.default_rng(6)
    for W in (1, 2, 3, 31, 32, 33, 100, 1000, 4096, 5000):
        w = rng.integers(0, 1 << 20, size=W) / 1024.0  # dyadic: every partial sum is exact
        np.testing.assert_array_equal(O.assoc_scan(w), np.cumsum(w))


def test_assoc_scan_tree_order():
    """The association order of jax.lax.associative_scan for n = 5:
    s1 = x0+x1, s3 = (x0+x1)+(x2+x3), s2 = s1+x2, s4 = s3+x4."""
    x = np.array([1.0, 1e-16, 1e-16, 1.0, 3e-16])
    s = O.assoc_scan(x)
    assert s[1] == x[0] + x[1]
    assert s[3] == (x[0] + x[1]) + (x[2] + x[3])
    assert s[2] == (x[0] + x[1]) + x[2]
    assert s[4] == s[3] + x[4]


def test_assoc_scan_close_to_cumsum():
    rng = np.random.default_rng(7)
    for W in (33, 257, 4096, 10000):
        w = rng.random(W) * rng.choice([0.0, 1.0, 1e-3, 50.0], size=W)
        np.testing.assert_allclose(O.assoc_scan(w), np.cumsum(w), rtol=1e-12)


def test_searchsorted_probe_sequence_matches_numpy_on_sorted():
    rng = np.random.default_rng(8)
    for W in (1, 2, 7, 64, 1000):
        cw = np.cumsum(rng.random(W) * (rng.random(W) > 0.3))
        z = np.concatenate([cw, rng.random(50) * cw[-1], [0.0, -1.0, cw[-1] * 2]])
        np.testing.assert_array_equal(O.searchsorted_left(cw, z), np.searchsorted(cw, z, side="left"))


def test_sr_indices_edge_cases():
    W = 64
    # all weight on one walker -> every index is that walker
    w = np.zeros(W)
    w[17] = 3.0
    idx, _ = O.sr_indices(w, 0.5, W, cumsum=O.assoc_scan)
    assert np.all(idx == 17)
    # uniform weights, zeta in [0, 1) -> identity permutation
    idx, _ = O.sr_indices(np.ones(W), 0.999, W, cumsum=O.assoc_scan)
    np.testing.assert_array_equal(idx, np.arange(W))
    # all-zero weights -> index 0 everywhere (searchsorted of 0 in zeros)
    idx, _ = O.sr_indices(np.zeros(W), 0.3, W, cumsum=O.assoc_scan)
    assert np.all(idx == 0)
    # negative weights use |w|
    idx1, _ = O.sr_indices(-np.arange(1.0, W + 1), 0.25, W)
    idx2, _ = O.sr_indices(np.arange(1.0, W + 1), 0.25, W)
    np.testing.assert_array_equal(idx1, idx2)


# ---- RNG --------------------------------------------------------------------

def test_philox_known_answers():
    """Philox4x32-10 known-answer vectors published with Random123."""
    cases = [
        ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
        ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
        ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
         (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
    ]
    for ctr, key, want in cases:
        got = philox_ref.philox4x32_10(np.array([ctr], dtype=np.uint32), np.array(key, dtype=np.uint32))[0]
        assert tuple(int(x) for x in got) == want


def test_philox_normals_moments():
    x = philox_ref.normal(200000, 5, 3)
    assert abs(x.mean()) < 0.01 and abs(x.std() - 1.0) < 0.01
    u = philox_ref.uniform(100001, 5, 4)
    assert u.min() >= 0.0 and u.max() < 1.0 and abs(u.mean() - 0.5) < 0.01
