"""The differentiated energy: the engine's adjoint kernels (afq_grad_*)
against the oracle's adjoint (oracle/adjoint_oracle.py) on the same fields,
and dE/dlam for h1 + lam D against common-random-number central
differences with the comb held at the unperturbed run's indices (the
function the adjoint differentiates; the free-comb difference is also
computed and agrees when no index moves).

Tolerances: block energies against the oracle 1e-10 relative (binary64
rounding of the same arithmetic over a few blocks); dL/dh1 against the
oracle 1e-7 relative in norm; dE/dlam against central differences 1e-5
relative at lam = +-1e-5 (truncation ~eps^2, rounding ~1e-12 / eps) and 1 %
at the 60-orbital workload's lam = +-1e-4."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _case(n, o, G, W, seed=11, steps=4, qr_every=2, dt=0.01, **H_kw):
    from ad_afqmc_prototype_gb300 import synth
    from ad_afqmc_prototype_gb300.core.system import system
    from ad_afqmc_prototype_gb300.ham.chol import ham_chol
    from ad_afqmc_prototype_gb300.meas.rhf import make_rhf_meas_ops
    from ad_afqmc_prototype_gb300.prop.afqmc import init_prop_state
    from ad_afqmc_prototype_gb300.prop.types import afqmc_params
    from ad_afqmc_prototype_gb300.trial.rhf import make_rhf_trial_ops, rhf_trial
    H = synth.make_hamiltonian(n, o, G, seed=seed, **H_kw)
    sys_ = system(norb=n, nelec=(o, o), walker_kind="restricted")
    ham = ham_chol(h0=H["h0"], h1=H["h1"], chol=H["chol"])
    trial = rhf_trial(H["mo_coeff"])
    params = afqmc_params(dt=dt, n_walkers=W, seed=seed, n_prop_steps=steps, qr_every=qr_every)
    t_ops, m_ops = make_rhf_trial_ops(sys_), make_rhf_meas_ops(sys_)
    st0 = init_prop_state(sys=sys_, n_walkers=W, seed=seed, ham_data=ham, trial_ops_=t_ops, trial_data=trial,
                          meas_ops=m_ops)
    D = torch.as_tensor(H["D"], device="cuda")
    return dict(H=H, sys=sys_, ham=ham, trial=trial, params=params, t_ops=t_ops, m_ops=m_ops, st0=st0, D=D)


def _energies(c, h1, n_blocks, seed, ck_steps, sr_fixed=None, runs=None):
    from ad_afqmc_prototype_gb300.grad import block_energies
    return block_energies(h1, ham_data=c["ham"], trial_data=c["trial"], params=c["params"], state=c["st0"],
                          n_blocks=n_blocks, seed=seed, counter=0, checkpoint_every=ck_steps, sr_fixed=sr_fixed,
                          run_out=runs)


def _grad(c, n_blocks, seed, ck_steps, loss="mixed"):
    from ad_afqmc_prototype_gb300.grad import mixed_energy
    h1 = c["ham"].h1.clone().requires_grad_(True)
    runs = []
    e, w = _energies(c, h1, n_blocks, seed, ck_steps, runs=runs)
    L = mixed_energy(e, w) if loss == "mixed" else torch.log(w).sum() + e[-1]
    L.backward()
    return h1.grad.detach(), e.detach(), w.detach(), runs[0]


def _fd(c, n_blocks, seed, eps, sr_fixed, loss="mixed"):
    from ad_afqmc_prototype_gb300.grad import mixed_energy
    vals, idxs = [], []
    with torch.no_grad():
        for s in (1.0, -1.0):
            runs = []
            e, w = _energies(c, c["ham"].h1 + s * eps * c["D"], n_blocks, seed, 10**9, sr_fixed=sr_fixed,
                             runs=runs)
            L = mixed_energy(e, w) if loss == "mixed" else torch.log(w).sum() + e[-1]
            vals.append(float(L))
            idxs.append(runs[0].sr_idx)
    return (vals[0] - vals[1]) / (2 * eps), idxs


def test_forward_equals_block_by_block(cuda):
    """The taped forward is afqmc_block: same fields, same kernels, same bits."""
    from ad_afqmc_prototype_gb300 import engine
    from ad_afqmc_prototype_gb300.prop.afqmc import device_state, engine_problem
    from ad_afqmc_prototype_gb300.prop.chol_afqmc_ops import make_chol_afqmc_ops
    c = _case(12, 4, 30, 64)
    p_ops = make_chol_afqmc_ops(c["ham"], "restricted")
    prob = engine_problem(params=c["params"], ham_data=c["ham"], trial_data=c["trial"], meas_ops=c["m_ops"],
                          prop_ops=p_ops, prop_ctx=p_ops.build_prop_ctx(c["t_ops"].get_rdm1(c["trial"]), 0.01),
                          meas_ctx=c["m_ops"].build_meas_ctx(c["ham"], c["trial"]), n_walkers=64, need_energy=True)
    st = device_state(c["st0"], inplace=False)
    S = c["params"].n_prop_steps
    ref = [engine.block(prob, c["params"], st, 5, b * (S + 1), return_idx=True) for b in range(4)]
    runs = []
    with torch.no_grad():
        e, w = _energies(c, c["ham"].h1, 4, 5, 8, runs=runs)
    for b, (eb, wb, ib) in enumerate(ref):
        assert float(eb) == float(e[b]) and float(wb) == float(w[b])
        assert torch.equal(ib.int(), runs[0].sr_idx[b])
    assert torch.equal(st.walkers, runs[0].final_state.walkers)


def test_adjoint_matches_oracle(cuda):
    """Same fields and comb uniforms through the oracle: block energies,
    comb indices and dL/dh1."""
    from ad_afqmc_prototype_gb300 import engine
    from oracle import adjoint_oracle as A
    from oracle import afqmc_oracle as O
    n, o, G, W, B, S = 10, 4, 20, 32, 3, 4
    c = _case(n, o, G, W, steps=S, qr_every=2)
    seed = 9
    g, e, w, run = _grad(c, B, seed, 2 * S)
    H = c["H"]
    st0 = c["st0"]
    ost = O.State(walkers=torch.as_tensor(st0.walkers).cpu().numpy(), weights=st0.weights.cpu().numpy(),
                  overlaps=st0.overlaps.cpu().numpy(), pop_control_ene_shift=float(st0.pop_control_ene_shift),
                  e_estimate=float(st0.e_estimate))
    fields, zetas = [], []
    for b in range(B):
        cb = b * (S + 1)
        fields.append(np.stack([engine.fill_normal((W, G), seed, cb + s).cpu().numpy() for s in range(S)]))
        zetas.append(float(engine.fill_uniform((1,), seed, cb + S).cpu()[0]))
    op = O.Params(dt=0.01, n_prop_steps=S, qr_every=2)
    prob = O.make_problem(H["h0"], H["h1"], H["chol"], H["mo_coeff"], 0.01)
    es, ws, tapes = A.run_forward(prob, op, ost, fields, zetas)
    np.testing.assert_allclose(e.cpu().numpy(), es, rtol=1e-10, atol=0)
    np.testing.assert_allclose(w.cpu().numpy(), ws, rtol=1e-10, atol=0)
    for b in range(B):
        assert np.array_equal(run.sr_idx[b].cpu().numpy(), tapes[b].idx)
    eb, wb = A.mixed_energy_bar(es, ws)
    h1bar, _ = A.run_backward(prob, op, tapes, eb, wb, W)
    got = g.cpu().numpy()
    assert np.linalg.norm(got - h1bar) <= 1e-7 * np.linalg.norm(h1bar), (np.linalg.norm(got - h1bar),
                                                                            np.linalg.norm(h1bar))


@pytest.mark.parametrize("loss", ["mixed", "weights_and_last"])
def test_derivative_matches_fixed_comb_fd(cuda, loss):
    c = _case(16, 5, 40, 128, steps=6, qr_every=3)
    B, seed = 5, 21
    g, e, w, run = _grad(c, B, seed, 12, loss=loss)  # checkpoints every 2 blocks: segments 2, 2, 1
    adj = float((g * c["D"]).sum())
    fd, idxs = _fd(c, B, seed, 1e-5, run.sr_idx, loss=loss)
    assert abs(adj - fd) <= 1e-5 * abs(fd) + 1e-10, (adj, fd)
    free, fidx = _fd(c, B, seed, 1e-5, None, loss=loss)
    if all(torch.equal(i, run.sr_idx) for i in fidx):
        assert abs(adj - free) <= 1e-5 * abs(free) + 1e-10, (adj, free)
    from ad_afqmc_prototype_gb300 import engine
    assert engine.workspace_status() == 0


def test_derivative_past_32_occupied_orbitals(cuda):
    """nocc 36 (the per-walker adjoint algebra past one warp's width): the
    adjoint against fixed-comb central differences."""
    c = _case(48, 36, 60, 32, steps=4, qr_every=2, dt=0.005)
    B, seed = 2, 5
    g, e, w, run = _grad(c, B, seed, 8)
    adj = float((g * c["D"]).sum())
    fd, _ = _fd(c, B, seed, 1e-5, run.sr_idx)
    assert abs(adj - fd) <= 1e-5 * abs(fd) + 1e-10, (adj, fd)


def test_checkpoint_interval_does_not_change_the_gradient(cuda):
    c = _case(12, 4, 24, 64, steps=4, qr_every=2)
    gs = [_grad(c, 5, 3, ck)[0] for ck in (4, 8, 20, 400)]
    for g in gs[1:]:
        assert torch.equal(g, gs[0])


def test_c3_workload_derivative(cuda):
    """nbasis 60, nocc 10, nchol 300, 1024 walkers, 200 steps (20 blocks of
    10, QR every 5), checkpoints every 20 steps: dE/dlam against central
    differences at lam = +-1e-4 with common random fields."""
    from ad_afqmc_prototype_gb300 import synth
    wl = synth.WORKLOADS["c3_n60_o10_g300_w1024"]
    c = _case(wl.nbasis, wl.nocc, wl.nchol, wl.n_walkers, seed=wl.seed, steps=10, qr_every=5, dt=0.005)
    B, seed = wl.n_steps // 10, 17
    g, e, w, run = _grad(c, B, seed, 20)
    adj = float((g * c["D"]).sum())
    fd, _ = _fd(c, B, seed, 1e-4, run.sr_idx)
    free, fidx = _fd(c, B, seed, 1e-4, None)
    flips = sum(int((i != run.sr_idx).sum()) for i in fidx)
    print(f"C3: dE/dlam adjoint {adj:.10f}  fixed-comb FD {fd:.10f}  free-comb FD {free:.10f} "
          f"(comb indices moved: {flips})")
    assert abs(adj - fd) <= 1e-2 * abs(fd), (adj, fd)
