"""The energy driver: the graph-replayed block loop gives the same blocks as
calling afqmc_block block by block (same random stream, same kernels, so the
same bits), and run_afqmc_energy returns the same result through either."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _objects(W, **pkw):
    from ad_afqmc_prototype_gb300 import synth
    from ad_afqmc_prototype_gb300.core.system import system
    from ad_afqmc_prototype_gb300.ham.chol import ham_chol
    from ad_afqmc_prototype_gb300.meas.rhf import make_rhf_meas_ops
    from ad_afqmc_prototype_gb300.prop.types import afqmc_params
    from ad_afqmc_prototype_gb300.trial.rhf import make_rhf_trial_ops, rhf_trial
    wl = synth.WORKLOADS["c1_n12_o6_g48_w256"]
    H = synth.make_workload(wl)
    sys_ = system(norb=wl.nbasis, nelec=(wl.nocc, wl.nocc), walker_kind="restricted")
    ham = ham_chol(h0=H["h0"], h1=H["h1"], chol=H["chol"])
    trial = rhf_trial(H["mo_coeff"])
    params = afqmc_params(dt=0.005, n_walkers=W, seed=3, n_prop_steps=10, qr_every=5, **pkw)
    return sys_, ham, trial, make_rhf_trial_ops(sys_), make_rhf_meas_ops(sys_), params


def test_graph_loop_equals_block_by_block(cuda):
    from ad_afqmc_prototype_gb300.driver import make_run_blocks
    from ad_afqmc_prototype_gb300.prop.afqmc import init_prop_state
    from ad_afqmc_prototype_gb300.prop.blocks import afqmc_block
    from ad_afqmc_prototype_gb300.prop.chol_afqmc_ops import make_chol_afqmc_ops
    sys_, ham, trial, t_ops, m_ops, params = _objects(64)
    p_ops = make_chol_afqmc_ops(ham, "restricted")
    kw = dict(sys=sys_, params=params, ham_data=ham, trial_data=trial, meas_ops=m_ops, prop_ops=p_ops,
              prop_ctx=p_ops.build_prop_ctx(t_ops.get_rdm1(trial), params.dt),
              meas_ctx=m_ops.build_meas_ctx(ham, trial))
    st0 = init_prop_state(sys=sys_, n_walkers=64, seed=params.seed, ham_data=ham, trial_ops_=t_ops,
                          trial_data=trial, meas_ops=m_ops)
    a = st0
    ea = []
    for _ in range(6):
        a, obs = afqmc_block(a, **kw)
        ea.append(float(obs.scalars["energy"]))
    run = make_run_blocks(lambda s: afqmc_block(s, **kw), kw)
    b, eb, wb = run(st0, n_blocks=6)
    np.testing.assert_array_equal(np.array(ea), eb.numpy())
    assert torch.equal(torch.as_tensor(a.walkers), torch.as_tensor(b.walkers))
    assert int(a.rng_key[1]) == int(b.rng_key[1])


def test_run_afqmc_energy_engine_and_generic_paths_agree(cuda, capsys):
    from ad_afqmc_prototype_gb300.driver import run_afqmc_energy
    from ad_afqmc_prototype_gb300.prop.blocks import afqmc_block
    sys_, ham, trial, t_ops, m_ops, params = _objects(64, n_eql_blocks=5, n_blocks=100)
    args = dict(sys=sys_, params=params, ham_data=ham, trial_data=trial, meas_ops=m_ops, trial_ops=t_ops)
    mu, err, e_all, w_all = run_afqmc_energy(block_fn=afqmc_block, **args)

    def generic(state, **kw):  # not afqmc_block itself: the block-by-block path
        return afqmc_block(state, **kw)
    mu2, err2, e2, w2 = run_afqmc_energy(block_fn=generic, **args)
    assert mu == mu2 and err == err2
    assert torch.equal(e_all, e2) and torch.equal(w_all, w2)
    assert e_all.shape[0] <= 1 + 5 + 100 and np.isfinite(mu) and err >= 0
    out = capsys.readouterr().out
    assert "Final blocking analysis" in out and "Equilibration" in out
