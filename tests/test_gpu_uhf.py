"""Unrestricted walkers with the RHF trial (walker_kind "unrestricted"):
the engine's afq_*_u kernels and block against the oracle restatement
(oracle/uhf_oracle.py), and the physics check that a pair of identical
spins reproduces the restricted run step for step.

Tolerances: kernels 1e-11 relative; block energies 1e-10 relative after
three blocks (binary64 rounding of the same arithmetic in another order);
comb indices exact."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _ham(n=12, o=4, G=30, seed=3):
    from ad_afqmc_prototype_gb300 import synth
    return synth.make_hamiltonian(n, o, G, seed=seed)


def _objects(H, W, kind, **pkw):
    from ad_afqmc_prototype_gb300.core.system import system
    from ad_afqmc_prototype_gb300.ham.chol import ham_chol
    from ad_afqmc_prototype_gb300.meas.rhf import make_rhf_meas_ops
    from ad_afqmc_prototype_gb300.prop.chol_afqmc_ops import make_chol_afqmc_ops
    from ad_afqmc_prototype_gb300.prop.types import afqmc_params
    from ad_afqmc_prototype_gb300.trial.rhf import make_rhf_trial_ops, rhf_trial
    n, o = H["h1"].shape[0], H["mo_coeff"].shape[1]
    sys_ = system(norb=n, nelec=(o, o), walker_kind=kind)
    ham = ham_chol(h0=H["h0"], h1=H["h1"], chol=H["chol"])
    trial = rhf_trial(H["mo_coeff"])
    params = afqmc_params(dt=0.01, n_walkers=W, seed=5, **pkw)
    t_ops, m_ops = make_rhf_trial_ops(sys_), make_rhf_meas_ops(sys_)
    p_ops = make_chol_afqmc_ops(ham, kind)
    kw = dict(sys=sys_, params=params, ham_data=ham, trial_data=trial, meas_ops=m_ops, prop_ops=p_ops,
              prop_ctx=p_ops.build_prop_ctx(t_ops.get_rdm1(trial), params.dt),
              meas_ctx=m_ops.build_meas_ctx(ham, trial))
    return sys_, t_ops, kw


def _pairs(H, W, seed=0):
    rng = np.random.default_rng(seed)
    mo = H["mo_coeff"]
    n, o = mo.shape
    wu = mo[None] + 0.3 * (rng.normal(size=(W, n, o)) + 1j * rng.normal(size=(W, n, o)))
    wd = mo[None] + 0.3 * (rng.normal(size=(W, n, o)) + 1j * rng.normal(size=(W, n, o)))
    return wu, wd


def test_kernels_match_oracle(cuda):
    from ad_afqmc_prototype_gb300 import engine
    from oracle import afqmc_oracle as O
    from oracle import uhf_oracle as U
    H = _ham()
    W = 8
    wu, wd = _pairs(H, W)
    prob = O.make_problem(H["h0"], H["h1"], H["chol"], H["mo_coeff"], 0.01)
    sys_, t_ops, kw = _objects(H, W, "unrestricted")
    mc, trial = kw["meas_ctx"], kw["trial_data"]
    pair = (torch.as_tensor(wu, device="cuda"), torch.as_tensor(wd, device="cuda"))
    ov = engine.overlap_u(pair, trial.mo_coeff, True).cpu().numpy()
    np.testing.assert_allclose(ov, U.overlap_u(wu, wd, H["mo_coeff"]), rtol=1e-11)
    fb = engine.force_bias_u(pair, trial.mo_coeff, mc.rot_chol, True).cpu().numpy()
    ref_fb = U.force_bias_u(wu, wd, prob.meas_ctx, H["mo_coeff"])
    np.testing.assert_allclose(fb, ref_fb, rtol=1e-11, atol=1e-11 * np.abs(ref_fb).max())
    e = engine.energy_u(pair, H["h0"], trial.mo_coeff, mc.rot_h1, mc.rot_chol, True).cpu().numpy()
    np.testing.assert_allclose(e, U.energy_u(wu, wd, H["h0"], prob.meas_ctx, H["mo_coeff"]), rtol=1e-11)
    rng = np.random.default_rng(1)
    xs = rng.normal(size=(W, H["chol"].shape[0])) + 0.1j * rng.normal(size=(W, H["chol"].shape[0]))
    out = engine.apply_trotter_u(pair, torch.as_tensor(xs, device="cuda"), kw["ham_data"].chol,
                                 kw["prop_ctx"].exp_h1_half, float(kw["prop_ctx"].sqrt_dt), 6).cpu().numpy()
    ru, rd = U.apply_trotter_u(wu, wd, xs, prob.prop_ctx, prob.chol_flat, 6)
    np.testing.assert_allclose(out[0], ru, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(out[1], rd, rtol=1e-12, atol=1e-12)


def test_blocks_match_oracle(cuda):
    from ad_afqmc_prototype_gb300.prop.afqmc import init_prop_state
    from ad_afqmc_prototype_gb300.prop.blocks import afqmc_block
    from oracle import afqmc_oracle as O
    from oracle import uhf_oracle as U
    H = _ham()
    W, S = 32, 4
    sys_, t_ops, kw = _objects(H, W, "unrestricted", n_prop_steps=S, qr_every=2)
    wu, wd = _pairs(H, W, seed=2)
    st = init_prop_state(sys=sys_, n_walkers=W, seed=5, ham_data=kw["ham_data"], trial_ops_=t_ops,
                         trial_data=kw["trial_data"], meas_ops=kw["meas_ops"],
                         initial_walkers=(torch.as_tensor(wu), torch.as_tensor(wd)))
    prob = O.make_problem(H["h0"], H["h1"], H["chol"], H["mo_coeff"], 0.01)
    ost = U.StateU(wu=wu, wd=wd, weights=np.ones(W), overlaps=st.overlaps.cpu().numpy(),
                   pop_control_ene_shift=float(st.pop_control_ene_shift), e_estimate=float(st.e_estimate))
    np.testing.assert_allclose(ost.overlaps, U.overlap_u(wu, wd, H["mo_coeff"]), rtol=1e-11)
    op = O.Params(dt=0.01, n_prop_steps=S, qr_every=2)
    rng = np.random.default_rng(7)
    for b in range(3):
        f = rng.normal(size=(S, W, H["chol"].shape[0]))
        z = float(rng.uniform())
        st, obs = afqmc_block(st, fields=f, zeta=z, **kw)
        ost, oobs, idx = U.block_u(prob, op, ost, f, z)
        assert abs(float(obs.scalars["energy"]) - oobs["energy"]) <= 1e-10 * abs(oobs["energy"])
        assert abs(float(obs.scalars["weight"]) - oobs["weight"]) <= 1e-10 * abs(oobs["weight"])
    np.testing.assert_allclose(st.walkers[0].cpu().numpy(), ost.wu, rtol=0, atol=1e-9)
    np.testing.assert_allclose(st.walkers[1].cpu().numpy(), ost.wd, rtol=0, atol=1e-9)


def test_identical_spins_reproduce_restricted_run(cuda):
    """(W, W) pairs follow the restricted walkers W: the same overlaps
    (det^2), force bias (2 L~ G), energies and weights, block by block."""
    from ad_afqmc_prototype_gb300.prop.afqmc import init_prop_state
    from ad_afqmc_prototype_gb300.prop.blocks import afqmc_block
    H = _ham(n=16, o=5, G=40, seed=4)
    W = 64
    sys_r, t_r, kw_r = _objects(H, W, "restricted", n_prop_steps=6, qr_every=3)
    sys_u, t_u, kw_u = _objects(H, W, "unrestricted", n_prop_steps=6, qr_every=3)
    sr = init_prop_state(sys=sys_r, n_walkers=W, seed=5, ham_data=kw_r["ham_data"], trial_ops_=t_r,
                         trial_data=kw_r["trial_data"], meas_ops=kw_r["meas_ops"])
    su = init_prop_state(sys=sys_u, n_walkers=W, seed=5, ham_data=kw_u["ham_data"], trial_ops_=t_u,
                         trial_data=kw_u["trial_data"], meas_ops=kw_u["meas_ops"])
    assert abs(float(sr.e_estimate) - float(su.e_estimate)) < 1e-12 * abs(float(sr.e_estimate))
    for b in range(3):
        sr, orr = afqmc_block(sr, **kw_r)
        su, ou = afqmc_block(su, **kw_u)
        er, eu = float(orr.scalars["energy"]), float(ou.scalars["energy"])
        assert abs(er - eu) < 1e-10 * abs(er), (b, er, eu)
    torch.testing.assert_close(su.walkers[0], sr.walkers, rtol=0, atol=1e-10)
    torch.testing.assert_close(su.walkers[1], sr.walkers, rtol=0, atol=1e-10)


def test_driver_runs_unrestricted(cuda, capsys):
    from ad_afqmc_prototype_gb300.driver import run_afqmc_energy
    from ad_afqmc_prototype_gb300.prop.blocks import afqmc_block
    H = _ham(n=12, o=4, G=30, seed=6)
    sys_, t_ops, kw = _objects(H, 32, "unrestricted", n_prop_steps=5, qr_every=0, n_eql_blocks=2, n_blocks=100)
    mu, err, e_all, w_all = run_afqmc_energy(sys=sys_, params=kw["params"], ham_data=kw["ham_data"],
                                            trial_data=kw["trial_data"], meas_ops=kw["meas_ops"],
                                            trial_ops=t_ops, block_fn=afqmc_block)
    assert np.isfinite(mu) and err >= 0 and e_all.shape[0] >= 90


# ---- generalized walkers (W, 2n, 2o) ------------------------------------------

def _gwalkers(H, W, seed=0):
    rng = np.random.default_rng(seed)
    mo = H["mo_coeff"]
    n, o = mo.shape
    base = np.zeros((2 * n, 2 * o), complex)
    base[:n, :o] = mo
    base[n:, o:] = mo
    return base[None] + 0.3 * (rng.normal(size=(W, 2 * n, 2 * o)) + 1j * rng.normal(size=(W, 2 * n, 2 * o)))


def test_generalized_kernels_match_oracle(cuda):
    from ad_afqmc_prototype_gb300 import engine
    from oracle import afqmc_oracle as O
    from oracle import uhf_oracle as U
    H = _ham()
    W = 8
    w = _gwalkers(H, W)
    prob = O.make_problem(H["h0"], H["h1"], H["chol"], H["mo_coeff"], 0.01)
    sys_, t_ops, kw = _objects(H, W, "generalized")
    mc, trial = kw["meas_ctx"], kw["trial_data"]
    wt = torch.as_tensor(w, device="cuda")
    np.testing.assert_allclose(engine.overlap_g(wt, trial.mo_coeff, True).cpu().numpy(),
                               U.overlap_g(w, H["mo_coeff"]), rtol=1e-11)
    fb = engine.force_bias_g(wt, trial.mo_coeff, mc.rot_chol, True).cpu().numpy()
    ref = U.force_bias_g(w, prob.meas_ctx, H["mo_coeff"])
    np.testing.assert_allclose(fb, ref, rtol=1e-11, atol=1e-11 * np.abs(ref).max())
    rng = np.random.default_rng(1)
    xs = rng.normal(size=(W, H["chol"].shape[0])) + 0.1j * rng.normal(size=(W, H["chol"].shape[0]))
    out = kw["prop_ops"].apply_trotter.batched(wt, torch.as_tensor(xs, device="cuda"), kw["prop_ctx"], 6)
    np.testing.assert_allclose(out.cpu().numpy(), U.apply_trotter_g(w, xs, prob.prop_ctx, prob.chol_flat, 6),
                               rtol=1e-12, atol=1e-12)


def test_generalized_step_matches_oracle_and_restricted(cuda):
    """A generalized step against the oracle; block-diagonal walkers
    [[W, 0], [0, W]] follow the restricted walkers W (same weights)."""
    from ad_afqmc_prototype_gb300.prop.afqmc import afqmc_step, init_prop_state
    from oracle import afqmc_oracle as O
    from oracle import uhf_oracle as U
    H = _ham(n=10, o=3, G=24, seed=8)
    W = 16
    n, o = H["mo_coeff"].shape
    sys_r, t_r, kw_r = _objects(H, W, "restricted")
    sys_g, t_g, kw_g = _objects(H, W, "generalized")
    sr = init_prop_state(sys=sys_r, n_walkers=W, seed=5, ham_data=kw_r["ham_data"], trial_ops_=t_r,
                         trial_data=kw_r["trial_data"], meas_ops=kw_r["meas_ops"])
    wr = sr.walkers.cpu().numpy()
    wg = np.zeros((W, 2 * n, 2 * o), complex)
    wg[:, :n, :o] = wr
    wg[:, n:, o:] = wr
    sg = init_prop_state(sys=sys_g, n_walkers=W, seed=5, ham_data=kw_g["ham_data"], trial_ops_=t_g,
                         trial_data=kw_g["trial_data"], meas_ops=kw_g["meas_ops"], initial_walkers=wg,
                         initial_e_estimate=sr.e_estimate)
    np.testing.assert_allclose(sg.overlaps.cpu().numpy(), sr.overlaps.cpu().numpy(), rtol=1e-11)
    step_kw = {k: v for k, v in kw_g.items() if k != "sys"}
    step_kw_r = {k: v for k, v in kw_r.items() if k != "sys"}
    prob = O.make_problem(H["h0"], H["h1"], H["chol"], H["mo_coeff"], 0.01)
    op = O.Params(dt=0.01)
    ost = O.State(walkers=wg, weights=np.ones(W), overlaps=sg.overlaps.cpu().numpy(),
                  pop_control_ene_shift=float(sg.pop_control_ene_shift), e_estimate=float(sg.e_estimate))
    rng = np.random.default_rng(3)
    for k in range(3):
        f = rng.normal(size=(W, H["chol"].shape[0]))
        sg = afqmc_step(sg, fields=f, **step_kw)
        sr = afqmc_step(sr, fields=f, **step_kw_r)
        ost = U.step_g(prob, op, ost, f)
        np.testing.assert_allclose(sg.walkers.cpu().numpy(), ost.walkers, rtol=0, atol=1e-11)
        np.testing.assert_allclose(sg.weights.cpu().numpy(), ost.weights, rtol=1e-11, atol=1e-14)
        np.testing.assert_allclose(sg.weights.cpu().numpy(), sr.weights.cpu().numpy(), rtol=1e-11, atol=1e-14)
        np.testing.assert_allclose(sg.walkers[:, :n, :o].cpu().numpy(), sr.walkers.cpu().numpy(), rtol=0, atol=1e-11)


def test_generalized_block_has_no_energy_kernel(cuda):
    """As in the reference, generalized meas ops have no energy kernel: the
    block's measurement raises KeyError naming the available kernels."""
    from ad_afqmc_prototype_gb300.prop.afqmc import init_prop_state
    from ad_afqmc_prototype_gb300.prop.blocks import afqmc_block
    H = _ham(n=8, o=2, G=12, seed=9)
    sys_g, t_g, kw_g = _objects(H, 8, "generalized", n_prop_steps=2)
    st = init_prop_state(sys=sys_g, n_walkers=8, seed=5, ham_data=kw_g["ham_data"], trial_ops_=t_g,
                         trial_data=kw_g["trial_data"], meas_ops=kw_g["meas_ops"], initial_e_estimate=0.0)
    assert tuple(st.walkers.shape) == (8, 16, 4)
    with pytest.raises(KeyError, match="available"):
        afqmc_block(st, **kw_g)
