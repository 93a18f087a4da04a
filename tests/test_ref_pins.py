"""The oracle against outputs of the reference's own hot-path code.

The fixtures tests/golden/ref_*.npz were produced by running the reference
package's functions unmodified on NumPy (tests/golden/make_ref_golden.py:
meas/rhf.py, prop/utils.py, prop/chol_afqmc_ops.py, walkers.py,
prop/afqmc.py, prop/blocks.py).  Every restated function of the oracle is
compared with the reference's result on the same inputs and draws.
"""
import os

import numpy as np
import pytest

from oracle import afqmc_oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    return dict(np.load(os.path.join(GOLDEN, name)))


@pytest.fixture(scope="module")
def kern():
    return _load("ref_kernels.npz")


@pytest.mark.parametrize("tag", ["real", "cplx"])
def test_contexts_match_reference(kern, tag):
    """build_meas_ctx (meas/rhf.py:141-150), _build_prop_ctx (prop/chol_afqmc_ops.py:77-103)."""
    c = kern[f"{tag}_mo"]
    ctx = O.build_meas_ctx(kern["h1"], kern["chol"], c)
    np.testing.assert_allclose(ctx.rot_h1, kern[f"{tag}_rot_h1"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(ctx.rot_chol, kern[f"{tag}_rot_chol"], rtol=0, atol=1e-14)
    p = O.build_prop_ctx(float(kern["h0"]), kern["h1"], kern["chol"], O.get_rdm1(c), float(kern["dt"]))
    np.testing.assert_allclose(p.exp_h1_half, kern[f"{tag}_exp_h1_half"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(p.mf_shifts, kern[f"{tag}_mf"], rtol=0, atol=1e-14)
    assert abs(p.h0_prop - complex(kern[f"{tag}_h0_prop"])) < 1e-13


@pytest.mark.parametrize("tag", ["real", "cplx"])
def test_meas_kernels_match_reference(kern, tag):
    """overlap_r, _half_green_from_overlap_matrix, force_bias_kernel_r and
    energy_kernel_r (meas/rhf.py:15-50) on random walkers."""
    c, w = kern[f"{tag}_mo"], kern["walkers"]
    ctx = O.build_meas_ctx(kern["h1"], kern["chol"], c)
    np.testing.assert_allclose(O.overlap_r(w, c), kern[f"{tag}_overlap"], rtol=1e-12)
    np.testing.assert_allclose(O.half_green(w, c), kern[f"{tag}_green"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(O.force_bias_r(w, ctx, c), kern[f"{tag}_fb"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(O.energy_r(w, float(kern["h0"]), ctx, c), kern[f"{tag}_energy"], rtol=1e-12)


def test_taylor_and_trotter_match_reference(kern):
    """taylor_expm_action (prop/utils.py:20-31) and apply_trotter
    (prop/chol_afqmc_ops.py:173-183) with a = i sqrt(dt), six terms."""
    w, dt = kern["walkers"], float(kern["dt"])
    out = O.taylor_expm_action(1j * np.sqrt(dt), kern["taylor_V"], w, 6)
    np.testing.assert_allclose(out, kern["taylor_out"], rtol=0, atol=1e-13)
    c = kern["real_mo"]
    p = O.build_prop_ctx(float(kern["h0"]), kern["h1"], kern["chol"], O.get_rdm1(c), dt)
    chol_flat = kern["chol"].reshape(kern["chol"].shape[0], -1)
    tw = O.apply_trotter_r(w, kern["trotter_fields"], p, chol_flat, 6)
    np.testing.assert_allclose(tw, kern["trotter_out"], rtol=0, atol=1e-13)


def test_qr_matches_reference(kern):
    """_qr with the phase convention and orthogonalize's det(R)^2 (walkers.py:169-203)."""
    q, det_r = O.qr_phase(kern["walkers"])
    np.testing.assert_allclose(q, kern["qr_q"], rtol=0, atol=1e-13)
    np.testing.assert_allclose(det_r, kern["qr_det_r"], rtol=1e-12)
    q2, norm = O.orthogonalize(kern["walkers"])
    np.testing.assert_allclose(q2, kern["orth_q"], rtol=0, atol=1e-13)
    np.testing.assert_allclose(norm, kern["orth_norm"], rtol=1e-12)


@pytest.mark.parametrize("k", range(5))
def test_comb_matches_reference_on_dyadic_weights(kern, k):
    """_sr_indices and the new weights of stochastic_reconfiguration
    (walkers.py:233-265).  Dyadic weights have exact prefix sums, so the
    reference's indices are the same in every association order and the
    oracle's (associative_scan order) must equal them bit for bit."""
    wts, z = kern[f"sr{k}_weights"], float(kern[f"sr{k}_zeta"])
    idx, cw = O.sr_indices(wts, z, wts.shape[0])
    np.testing.assert_array_equal(idx, kern[f"sr{k}_idx"])
    np.testing.assert_array_equal(np.full(wts.shape[0], cw[-1] / wts.shape[0]), kern[f"sr{k}_weights_new"])


def _check_blocks(ref, H, W, n_steps, atol_e, atol_w):
    prob = O.make_problem(H["h0"], H["h1"], H["chol"], ref["mo_coeff"], 0.005)
    P = O.Params(dt=0.005, n_prop_steps=n_steps, qr_every=0)
    w0 = ref["init_walkers"]
    if w0.shape[0] != W:  # stored as one row: every walker starts at the trial
        w0 = np.ascontiguousarray(np.broadcast_to(w0[0], (W, *w0.shape[1:])))
    st = O.init_prop_state(prob, W, w0)
    assert abs(st.e_estimate - float(ref["e_estimate"])) < 1e-11
    np.testing.assert_allclose(st.overlaps, ref["init_overlaps"], rtol=1e-12)
    s1 = O.afqmc_step(prob, P, st, ref["fields"][0, 0])
    nk = ref["step1_walkers"].shape[0]
    np.testing.assert_allclose(s1.walkers[:nk], ref["step1_walkers"], rtol=0, atol=atol_w)
    np.testing.assert_allclose(s1.weights, ref["step1_weights"], rtol=1e-11)
    np.testing.assert_allclose(s1.overlaps, ref["step1_overlaps"], rtol=1e-10)
    assert abs(s1.pop_control_ene_shift - float(ref["step1_pop_shift"])) < 1e-10
    for b in range(ref["fields"].shape[0]):
        st, obs, idx = O.afqmc_block(prob, P, st, ref["fields"][b], float(ref["zetas"][b]))
        np.testing.assert_array_equal(idx, ref["sr_idx"][b])
        assert abs(obs["energy"] - ref["block_energy"][b]) < atol_e, (b, obs["energy"], ref["block_energy"][b])
        assert abs(obs["weight"] - ref["block_weight"][b]) < 1e-10 * max(1.0, abs(ref["block_weight"][b]))
        assert abs(st.pop_control_ene_shift - ref["block_pop_shift"][b]) < atol_e
    nk = ref["final_walkers"].shape[0]
    np.testing.assert_allclose(st.walkers[:nk], ref["final_walkers"], rtol=0, atol=atol_w)
    np.testing.assert_allclose(st.weights, ref["final_weights"], rtol=1e-11)
    np.testing.assert_allclose(st.overlaps, ref["final_overlaps"], rtol=1e-9)


def test_block_c1_matches_reference():
    """init_prop_state, afqmc_step and two afqmc_blocks (prop/afqmc.py:17-147,
    prop/blocks.py:22-95) on the 12-orbital workload, 32 walkers, 10 steps a
    block, the reference's own draws: energies to 1e-11 Ha, comb indices equal."""
    from ad_afqmc_prototype_gb300 import synth
    ref = _load("ref_block_c1.npz")
    H = synth.make_workload(synth.WORKLOADS["c1_n12_o6_g48_w256"])
    _check_blocks(ref, H, W=32, n_steps=10, atol_e=1e-11, atol_w=1e-12)


def test_block_c4_shape_matches_reference():
    """One block of 4 steps on the 200-orbital, 1000-vector Hamiltonian of the
    benchmark workload (4 walkers): energy to 1e-10 Ha."""
    from ad_afqmc_prototype_gb300 import synth
    ref = _load("ref_block_c4.npz")
    H = synth.make_workload(synth.WORKLOADS["c4_n200_o30_g1000_w4096"])
    chk = np.array([H["chol"].sum(), np.abs(H["chol"]).sum(), H["h1"].sum()])
    np.testing.assert_allclose(chk, ref["chol_checksum"], rtol=1e-12)
    _check_blocks(ref, H, W=4, n_steps=4, atol_e=1e-10, atol_w=1e-12)
