"""GPU parity of the fused step and block, and the reference's own step tests
ported to the drop-in API.  Tolerances: binary64 on both sides; walkers
1e-10 absolute, energies 1e-10 Ha (1e-9 after two blocks), comb indices
bit-exact."""
import os

import numpy as np
import pytest
import torch

from oracle import afqmc_oracle as O

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def cpu(t):
    return t.detach().cpu().numpy()


@pytest.fixture(scope="module")
def api(cuda):
    from ad_afqmc_prototype_gb300 import engine, synth
    from ad_afqmc_prototype_gb300.core.system import system
    from ad_afqmc_prototype_gb300.ham.chol import ham_chol
    from ad_afqmc_prototype_gb300.meas.rhf import make_rhf_meas_ops
    from ad_afqmc_prototype_gb300.prop.afqmc import afqmc_step, init_prop_state
    from ad_afqmc_prototype_gb300.prop.blocks import afqmc_block
    from ad_afqmc_prototype_gb300.prop.chol_afqmc_ops import make_chol_afqmc_ops
    from ad_afqmc_prototype_gb300.prop.types import afqmc_params, prop_state, PRNGKey
    from ad_afqmc_prototype_gb300.trial.rhf import get_rdm1, make_rhf_trial_ops, rhf_trial
    return dict(engine=engine, synth=synth, system=system, ham_chol=ham_chol, make_rhf_meas_ops=make_rhf_meas_ops,
                afqmc_step=afqmc_step, init_prop_state=init_prop_state, afqmc_block=afqmc_block,
                make_chol_afqmc_ops=make_chol_afqmc_ops, afqmc_params=afqmc_params, prop_state=prop_state,
                PRNGKey=PRNGKey, get_rdm1=get_rdm1, make_rhf_trial_ops=make_rhf_trial_ops, rhf_trial=rhf_trial)


def _setup(api, H, W, **pkw):
    n, o = H["mo_coeff"].shape
    sys_ = api["system"](norb=n, nelec=(o, o), walker_kind="restricted")
    ham = api["ham_chol"](h0=H["h0"], h1=H["h1"], chol=H["chol"])
    trial = api["rhf_trial"](H["mo_coeff"])
    t_ops, m_ops = api["make_rhf_trial_ops"](sys_), api["make_rhf_meas_ops"](sys_)
    p_ops = api["make_chol_afqmc_ops"](ham, "restricted")
    params = api["afqmc_params"](**pkw)
    pctx = p_ops.build_prop_ctx(api["get_rdm1"](trial), params.dt)
    mctx = m_ops.build_meas_ctx(ham, trial)
    w0 = api["synth"].trial_walkers(H["mo_coeff"], W)
    state = api["init_prop_state"](sys=sys_, n_walkers=W, seed=params.seed, ham_data=ham, trial_ops_=t_ops,
                                   trial_data=trial, meas_ops=m_ops, initial_walkers=w0)
    kw = dict(params=params, ham_data=ham, trial_data=trial, meas_ops=m_ops, prop_ops=p_ops, prop_ctx=pctx,
              meas_ctx=mctx)
    return sys_, state, kw


def test_block_matches_golden(api):
    g = np.load(os.path.join(ROOT, "tests", "golden", "c1_block.npz"))
    H = api["synth"].make_workload(api["synth"].WORKLOADS["c1_n12_o6_g48_w256"])
    W = g["fields"].shape[2]
    sys_, state, kw = _setup(api, H, W, dt=0.005, n_prop_steps=10, qr_every=5)
    assert abs(float(state.e_estimate) - float(g["e_estimate"])) < 1e-10
    np.testing.assert_allclose(cpu(state.overlaps), g["init_overlaps"], rtol=1e-12)
    s1 = api["afqmc_step"](state, fields=g["fields"][0, 0], **kw)
    np.testing.assert_allclose(cpu(s1.walkers), g["step1_walkers"], atol=1e-12)
    np.testing.assert_allclose(cpu(s1.weights), g["step1_weights"], rtol=1e-11)
    np.testing.assert_allclose(cpu(s1.overlaps), g["step1_overlaps"], rtol=1e-11)
    assert abs(float(s1.pop_control_ene_shift) - float(g["step1_pop_shift"])) < 1e-10
    for b in range(g["fields"].shape[0]):
        state, obs = api["afqmc_block"](state, sys=sys_, fields=g["fields"][b], zeta=float(g["zetas"][b]), **kw)
        assert abs(float(obs.scalars["energy"]) - g["block_energy"][b]) < 1e-9
        assert abs(float(obs.scalars["weight"]) - g["block_weight"][b]) < 1e-9 * abs(g["block_weight"][b])
    np.testing.assert_allclose(cpu(state.walkers), g["final_walkers"], atol=1e-10)
    np.testing.assert_allclose(cpu(state.weights), g["final_weights"], rtol=1e-10)
    assert abs(float(state.pop_control_ene_shift) - float(g["final_pop_shift"])) < 1e-9


def test_block_comb_indices_bit_exact(api):
    g = np.load(os.path.join(ROOT, "tests", "golden", "c1_block.npz"))
    H = api["synth"].make_workload(api["synth"].WORKLOADS["c1_n12_o6_g48_w256"])
    W = g["fields"].shape[2]
    sys_, state, kw = _setup(api, H, W, dt=0.005, n_prop_steps=10, qr_every=5)
    from ad_afqmc_prototype_gb300.prop.afqmc import device_state, engine_problem
    prob = engine_problem(n_walkers=W, need_energy=True, **kw)
    st = device_state(state, inplace=False)
    for b in range(g["fields"].shape[0]):
        _, _, idx = api["engine"].block(prob, kw["params"], st, 0, 0, fields=g["fields"][b],
                                        zeta=float(g["zetas"][b]), return_idx=True)
        np.testing.assert_array_equal(cpu(idx), g["sr_idx"][b])


@pytest.mark.parametrize("wl,W,steps", [("c3_n60_o10_g300_w1024", 64, 3), ("c2_n120_o20_g600_w2048", 16, 2)])
def test_steps_match_oracle_larger(api, wl, W, steps):
    H = api["synth"].make_workload(api["synth"].WORKLOADS[wl])
    sys_, state, kw = _setup(api, H, W, dt=0.005)
    prob = O.make_problem(H["h0"], H["h1"], H["chol"], H["mo_coeff"], 0.005)
    P = O.Params(dt=0.005)
    ost = O.init_prop_state(prob, W, api["synth"].trial_walkers(H["mo_coeff"], W))
    assert abs(float(state.e_estimate) - ost.e_estimate) < 1e-10
    rng = np.random.default_rng(4)
    for s in range(steps):
        f = rng.standard_normal((W, H["chol"].shape[0]))
        state = api["afqmc_step"](state, fields=f, **kw)
        ost = O.afqmc_step(prob, P, ost, f)
    np.testing.assert_allclose(cpu(state.walkers), ost.walkers, atol=1e-10)
    np.testing.assert_allclose(cpu(state.weights), ost.weights, rtol=1e-10)
    assert abs(float(state.pop_control_ene_shift) - ost.pop_control_ene_shift) < 1e-9


def test_drawn_fields_are_the_philox_stream(api):
    """Without injected fields the step draws N(0,1) fields from (seed, counter)."""
    H = api["synth"].make_workload(api["synth"].WORKLOADS["c1_n12_o6_g48_w256"])
    W = 32
    sys_, state, kw = _setup(api, H, W, dt=0.005, seed=11)
    out = api["afqmc_step"](state, **kw)
    f = api["engine"].fill_normal((W, 48), 11, 0)
    ref = api["afqmc_step"](state, fields=f, **kw)
    np.testing.assert_array_equal(cpu(out.walkers), cpu(ref.walkers))
    assert list(out.rng_key) == [11, 1]
    # the input state is left untouched
    np.testing.assert_array_equal(cpu(state.walkers), api["synth"].trial_walkers(H["mo_coeff"], W))


# ---- the reference's tests/test_prop_afqmc_step.py, ported ------------------

def _dummy_ops():
    from ad_afqmc_prototype_gb300.core.ops import meas_ops, trial_ops

    def overlap(_w, _t):
        return torch.ones((), dtype=torch.complex128, device="cuda")

    def fb(walker, ham, _ctx, _t):
        return torch.zeros((ham.chol.shape[0],), dtype=walker.dtype, device=walker.device)

    return (trial_ops(overlap=overlap, get_rdm1=lambda td: td["rdm1"]),
            meas_ops(overlap=overlap, build_meas_ctx=lambda h, t: None, kernels={"force_bias": fb}))


def test_weight_update_matches_h0_prop_and_pop_control_update(api):
    """tests/test_prop_afqmc_step.py:46-94."""
    norb, nocc, nw, nf = 4, 2, 8, 3
    ham = api["ham_chol"](basis="restricted", h0=1.0, h1=np.zeros((norb, norb)), chol=np.zeros((nf, norb, norb)))
    params = api["afqmc_params"](dt=0.2, n_chunks=2, n_exp_terms=4, pop_control_damping=0.1)
    t_ops, m_ops = _dummy_ops()
    trial_data = {"rdm1": torch.zeros((norb, norb), dtype=torch.float64)}
    st = api["prop_state"](walkers=torch.ones((nw, norb, nocc), dtype=torch.complex64, device="cuda"),
                           weights=torch.ones(nw, dtype=torch.float64, device="cuda"),
                           overlaps=torch.ones(nw, dtype=torch.complex64, device="cuda"),
                           rng_key=api["PRNGKey"](0),
                           pop_control_ene_shift=torch.tensor(0.0, dtype=torch.float64, device="cuda"),
                           e_estimate=torch.tensor(0.0, dtype=torch.float64, device="cuda"))
    p_ops = api["make_chol_afqmc_ops"](ham, "restricted")
    pctx = p_ops.build_prop_ctx(trial_data["rdm1"], params.dt)
    out = api["afqmc_step"](st, params=params, ham_data=ham, trial_data=trial_data, meas_ops=m_ops, prop_ops=p_ops,
                            prop_ctx=pctx, meas_ctx=None)
    np.testing.assert_allclose(cpu(out.weights), np.exp(-0.2) * np.ones(nw), rtol=1e-14)
    assert abs(float(out.pop_control_ene_shift) - 0.1) < 1e-14
    assert float(out.e_estimate) == 0.0


def test_step_matches_manual_walker_propagation_and_is_chunk_invariant(api):
    """tests/test_prop_afqmc_step.py:97-173."""
    norb, nocc, nw, nf = 5, 2, 6, 4
    rng = np.random.default_rng(42)
    a = rng.normal(size=(norb, norb))
    ham = api["ham_chol"](basis="restricted", h0=0.0, h1=0.05 * (a + a.T), chol=0.02 * rng.normal(size=(nf, norb, norb)))
    p1 = api["afqmc_params"](dt=0.1, n_chunks=1, n_exp_terms=6)
    p2 = api["afqmc_params"](dt=0.1, n_chunks=3, n_exp_terms=6)
    t_ops, m_ops = _dummy_ops()
    trial_data = {"rdm1": torch.zeros((norb, norb), dtype=torch.float64)}
    w = (rng.normal(size=(nw, norb, nocc)) + 1j * rng.normal(size=(nw, norb, nocc)))
    st = api["prop_state"](walkers=torch.as_tensor(w).cuda(), weights=torch.ones(nw, dtype=torch.float64).cuda(),
                           overlaps=torch.ones(nw, dtype=torch.complex128).cuda(), rng_key=api["PRNGKey"](0),
                           pop_control_ene_shift=torch.tensor(0.0, dtype=torch.float64).cuda(),
                           e_estimate=torch.tensor(0.0, dtype=torch.float64).cuda())
    p_ops = api["make_chol_afqmc_ops"](ham, "restricted")
    pctx = p_ops.build_prop_ctx(trial_data["rdm1"], p1.dt)
    kw = dict(ham_data=ham, trial_data=trial_data, meas_ops=m_ops, prop_ops=p_ops, prop_ctx=pctx, meas_ctx=None)
    out1 = api["afqmc_step"](st, params=p1, **kw)
    fields = api["engine"].fill_normal((nw, nf), 0, 0)
    expected = torch.stack([p_ops.apply_trotter(st.walkers[i], fields[i].to(torch.complex128), pctx, 6)
                            for i in range(nw)])
    np.testing.assert_allclose(cpu(out1.walkers), cpu(expected), rtol=1e-13, atol=1e-14)
    np.testing.assert_allclose(cpu(out1.overlaps), np.ones(nw))
    assert list(out1.rng_key) == [0, 1]
    out2 = api["afqmc_step"](st, params=p2, **kw)
    np.testing.assert_allclose(cpu(out2.walkers), cpu(out1.walkers), rtol=1e-14, atol=1e-15)
    np.testing.assert_allclose(cpu(out2.weights), cpu(out1.weights), rtol=1e-14)
    # the fused engine step is chunk invariant too
    H = api["synth"].make_hamiltonian(10, 3, 20, seed=2)
    sys_, s0, kwa = _setup(api, H, 12, dt=0.01, n_chunks=1)
    _, _, kwb = _setup(api, H, 12, dt=0.01, n_chunks=4)
    f = np.random.default_rng(1).standard_normal((12, 20))
    ra = api["afqmc_step"](s0, fields=f, **kwa)
    rb = api["afqmc_step"](s0, fields=f, **kwb)
    np.testing.assert_array_equal(cpu(ra.walkers), cpu(rb.walkers))


def test_generic_block_path_equals_fused(api):
    """A block composed from the per-walker ops gives the fused block's result."""
    from ad_afqmc_prototype_gb300.core.ops import meas_ops
    H = api["synth"].make_workload(api["synth"].WORKLOADS["c1_n12_o6_g48_w256"])
    W = 16
    sys_, state, kw = _setup(api, H, W, dt=0.005, n_prop_steps=4, qr_every=2)
    fields = np.random.default_rng(0).standard_normal((4, W, 48))
    a, oa = api["afqmc_block"](state, sys=sys_, fields=fields, zeta=0.6, **kw)
    m = kw["meas_ops"]
    wrapped = meas_ops(overlap=lambda w, t: m.overlap(w, t), build_meas_ctx=m.build_meas_ctx,
                       kernels={k: (lambda f: (lambda *x: f(*x)))(f) for k, f in m.kernels.items()})
    for k, f in m.kernels.items():
        wrapped.kernels[k].batched = f.batched
    wrapped.overlap.batched = m.overlap.batched
    kw2 = dict(kw, meas_ops=wrapped)
    b, ob = api["afqmc_block"](state, sys=sys_, fields=fields, zeta=0.6, **kw2)
    np.testing.assert_allclose(cpu(b.walkers), cpu(a.walkers), atol=1e-13)
    assert abs(float(ob.scalars["energy"]) - float(oa.scalars["energy"])) < 1e-12


def test_api_errors(api):
    sys_x = api["system"](norb=4, nelec=(2, 2), walker_kind="generalized")
    object.__setattr__(sys_x, "walker_kind", "bogus")
    with pytest.raises(ValueError):
        api["make_rhf_meas_ops"](sys_x)
    with pytest.raises(ValueError):
        api["make_rhf_trial_ops"](api["system"](norb=4, nelec=(2, 1), walker_kind="restricted"))
    with pytest.raises(ValueError):
        api["ham_chol"](h0=0.0, h1=np.zeros((3, 4)), chol=np.zeros((2, 3, 4)))
    from ad_afqmc_prototype_gb300.core.ops import meas_ops
    with pytest.raises(KeyError, match="available"):
        meas_ops(overlap=None).require_kernel("energy")
    from ad_afqmc_prototype_gb300 import walkers as wk
    with pytest.raises(ValueError, match="divisible"):
        wk.apply_chunked(torch.zeros((6, 2, 1), dtype=torch.complex128, device="cuda"), lambda w: w.sum(), 4)


def test_full_size_properties(api):
    """4096 walkers of the 200-orbital workload after one step: QR gives
    orthonormal columns and the comb conserves the total |weight|."""
    H = api["synth"].make_workload(api["synth"].WORKLOADS["c4_n200_o30_g1000_w4096"])
    W = 4096
    sys_, state, kw = _setup(api, H, W, dt=0.005)
    state = api["afqmc_step"](state, inplace=True, **kw)
    q, _ = api["engine"].orthogonalize(state.walkers)
    qq = torch.einsum("wia,wib->wab", q.conj(), q)
    err = (qq - torch.eye(30, dtype=qq.dtype, device=qq.device)).abs().max().item()
    assert err < 1e-12
    wt = state.weights
    out, wout, idx = api["engine"].stochastic_reconfiguration(q, wt, 0.5)
    assert abs(wout.sum().item() - wt.abs().sum().item()) < 1e-9 * wt.abs().sum().item()
    assert int(idx.min()) >= 0 and int(idx.max()) < W
    assert bool(torch.all(wt[idx] > 0))  # the comb never picks a zero-weight walker
