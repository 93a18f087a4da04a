"""The mixed-precision forms against the binary64 form, through the same API,
from identical states and fields, for both split widths ("mixed": six bf16
sections, products to ~2^-24; "mixed_fast": three sections, ~2^-17).
Tolerances: one step moves walkers by <= 1e-4 relative; block energies
agree to 1e-4 Ha (0.1 mHa, the accuracy target of the mixed form) and the
energy kernel alone (a block of zero steps) to 1e-4 Ha as well."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _setup(wl_name, W, precision, asym=0.0, **pkw):
    from ad_afqmc_prototype_gb300 import synth
    from ad_afqmc_prototype_gb300.core.system import system
    from ad_afqmc_prototype_gb300.ham.chol import ham_chol
    from ad_afqmc_prototype_gb300.meas.rhf import make_rhf_meas_ops
    from ad_afqmc_prototype_gb300.prop.afqmc import engine_problem, init_prop_state
    from ad_afqmc_prototype_gb300.prop.chol_afqmc_ops import make_chol_afqmc_ops
    from ad_afqmc_prototype_gb300.prop.types import afqmc_params
    from ad_afqmc_prototype_gb300.trial.rhf import get_rdm1, make_rhf_trial_ops, rhf_trial
    wl = synth.WORKLOADS[wl_name] if isinstance(wl_name, str) else wl_name
    H = synth.make_workload(wl)
    if asym:  # an antisymmetric part: V = sum_g x_g L_g is then not symmetric
        r = np.random.default_rng(wl.seed + 1).normal(size=H["chol"].shape)
        H["chol"] = H["chol"] + asym * np.abs(H["chol"]).mean() * (r - np.swapaxes(r, 1, 2))
    n, o = wl.nbasis, wl.nocc
    sys_ = system(norb=n, nelec=(o, o), walker_kind="restricted")
    ham = ham_chol(h0=H["h0"], h1=H["h1"], chol=H["chol"])
    trial = rhf_trial(H["mo_coeff"])
    t_ops, m_ops = make_rhf_trial_ops(sys_), make_rhf_meas_ops(sys_)
    p_ops = make_chol_afqmc_ops(ham, "restricted")
    params = afqmc_params(dt=0.005, precision=precision, **pkw)
    pctx = p_ops.build_prop_ctx(get_rdm1(trial), params.dt)
    mctx = m_ops.build_meas_ctx(ham, trial)
    st = init_prop_state(sys=sys_, n_walkers=W, seed=1, ham_data=ham, trial_ops_=t_ops, trial_data=trial,
                         meas_ops=m_ops, initial_walkers=synth.trial_walkers(H["mo_coeff"], W))
    kw = dict(params=params, ham_data=ham, trial_data=trial, meas_ops=m_ops, prop_ops=p_ops, prop_ctx=pctx,
              meas_ctx=mctx)
    return engine_problem(n_walkers=W, need_energy=True, **kw), params, st


def _dstate(st):
    from ad_afqmc_prototype_gb300.prop.afqmc import device_state
    return device_state(st, inplace=False)


PRECISIONS = ["mixed", "mixed_fast"]


@pytest.mark.parametrize("prec", PRECISIONS)
@pytest.mark.parametrize("wl,W", [("c3_n60_o10_g300_w1024", 64), ("c1_n12_o6_g48_w256", 100),
                                  ("c4_n200_o30_g1000_w4096", 40)])
def test_mixed_step_close_to_fp64(cuda, wl, W, prec):
    """c4 (norb 200 = 8 k, nocc 30 <= 32) takes the tensor-core Taylor kernel
    in the three-section form; c1 and c3 the fp32 SIMT one."""
    from ad_afqmc_prototype_gb300 import engine
    pa, pra, st = _setup(wl, W, "fp64")
    pb, prb, _ = _setup(wl, W, prec)
    a, b = _dstate(st), _dstate(st)
    G = pa.nchol
    for k in range(3):
        f = engine.fill_normal((W, G), 3, k)
        engine.step(pa, pra, a, 0, 0, fields=f)
        engine.step(pb, prb, b, 0, 0, fields=f)
    assert engine.workspace_status() == 0
    rel = float(((a.walkers - b.walkers).abs().max() / a.walkers.abs().max()).item())
    assert rel < 1e-4, rel
    relw = float(((a.weights - b.weights).abs() / a.weights.abs().clamp_min(1e-300)).max().item())
    assert relw < 1e-4, relw
    relo = float(((a.overlaps - b.overlaps).abs() / a.overlaps.abs()).max().item())
    assert relo < 1e-3, relo


@pytest.mark.parametrize("n,o,G,asym", [(40, 7, 96, 0.0), (120, 20, 240, 0.5), (200, 32, 400, 0.0),
                                        (256, 32, 300, 0.0), (248, 1, 200, 0.5)])
def test_tensor_core_taylor_shapes(cuda, n, o, G, asym):
    """The three-section step at the tensor-core Taylor kernel's edge shapes
    (norb a multiple of 8 up to 256, not of 16; nocc up to 32 and 1; three and
    four ring stages, the walker staged through the ring; Cholesky
    vectors with an antisymmetric part, so that a transposed V would show)
    against the binary64 step from the same state and fields: walkers within
    1e-5 of their largest entry after three steps."""
    from ad_afqmc_prototype_gb300 import engine, synth
    W = 24
    wl = synth.Workload(name=f"t_n{n}_o{o}_g{G}", nbasis=n, nocc=o, nchol=G, n_walkers=W, n_steps=3, seed=11)
    pa, pra, st = _setup(wl, W, "fp64", asym=asym)
    pb, prb, _ = _setup(wl, W, "mixed_fast", asym=asym)
    a, b = _dstate(st), _dstate(st)
    for k in range(3):
        f = engine.fill_normal((W, G), 5, k)
        engine.step(pa, pra, a, 0, 0, fields=f)
        engine.step(pb, prb, b, 0, 0, fields=f)
    assert engine.workspace_status() == 0
    rel = float(((a.walkers - b.walkers).abs().max() / a.walkers.abs().max()).item())
    print(f"n={n} o={o}: max |dW| / max |W| = {rel:.3e}")
    assert rel < 1e-5, rel


@pytest.mark.parametrize("prec", PRECISIONS)
@pytest.mark.parametrize("wl,W", [("c3_n60_o10_g300_w1024", 128), ("c4_n200_o30_g1000_w4096", 256)])
def test_mixed_energy_kernel_close_to_fp64(cuda, wl, W, prec):
    """A block of zero steps is QR + energy + comb: isolates the energy GEMM."""
    from ad_afqmc_prototype_gb300 import engine
    pa, pra, st = _setup(wl, W, "fp64", n_prop_steps=3)
    pb, prb, _ = _setup(wl, W, prec, n_prop_steps=3)
    a = _dstate(st)
    engine.block(pa, pra, a, 5, 0)  # move the walkers off the trial
    z0a = pra.__class__(**{**pra.__dict__, "n_prop_steps": 0})
    z0b = prb.__class__(**{**prb.__dict__, "n_prop_steps": 0})
    x, y = engine.DeviceState(*[t.clone() for t in (a.walkers, a.weights, a.overlaps, a.pop_shift, a.e_estimate)]), \
        engine.DeviceState(*[t.clone() for t in (a.walkers, a.weights, a.overlaps, a.pop_shift, a.e_estimate)])
    ea, _ = engine.block(pa, z0a, x, 5, 100, zeta=0.5)
    eb, _ = engine.block(pb, z0b, y, 5, 100, zeta=0.5)
    assert engine.workspace_status() == 0
    assert abs(float(ea) - float(eb)) < 1e-4, (float(ea), float(eb))


@pytest.mark.parametrize("prec", PRECISIONS)
def test_mixed_block_energy_error_per_block(cuda, prec):
    """From identical block-start states and fields: |E_mixed - E_fp64| per
    10-step block (QR after step 5) within 0.1 mHa."""
    from ad_afqmc_prototype_gb300 import engine
    W = 512
    pa, pra, st = _setup("c4_n200_o30_g1000_w4096", W, "fp64", n_prop_steps=10, qr_every=5)
    pb, prb, _ = _setup("c4_n200_o30_g1000_w4096", W, prec, n_prop_steps=10, qr_every=5)
    ref = _dstate(st)
    errs = []
    for blk in range(3):
        f = engine.fill_normal((10, W, pa.nchol), 9, blk)
        b = engine.DeviceState(*[t.clone() for t in (ref.walkers, ref.weights, ref.overlaps, ref.pop_shift,
                                                      ref.e_estimate)])
        ea, wa = engine.block(pa, pra, ref, 0, 0, fields=f, zeta=0.25)
        eb, wb = engine.block(pb, prb, b, 0, 0, fields=f, zeta=0.25)
        errs.append(abs(float(ea) - float(eb)))
    assert engine.workspace_status() == 0
    print("per-block |dE| (Ha):", errs)
    assert max(errs) < 1e-4, errs


def test_mixed_overlap_matches_binary64(cuda):
    """The mixed forms form m = C^H W from exact integer digit products on the
    tensor cores (nocc <= 32; double-float arithmetic beyond), ~2^-44 of the
    entries' scale, and its LU in double-float: after a block of zero steps
    (QR, overlap, energy, comb) the overlaps agree with the binary64 form's
    to 1e-10 relative."""
    from ad_afqmc_prototype_gb300 import engine
    W = 64
    pa, pra, st = _setup("c4_n200_o30_g1000_w4096", W, "fp64", n_prop_steps=3)
    pb, prb, _ = _setup("c4_n200_o30_g1000_w4096", W, "mixed_fast", n_prop_steps=3)
    a = _dstate(st)
    engine.block(pa, pra, a, 5, 0)  # move the walkers off the trial
    z0a = pra.__class__(**{**pra.__dict__, "n_prop_steps": 0})
    z0b = prb.__class__(**{**prb.__dict__, "n_prop_steps": 0})
    x = engine.DeviceState(*[t.clone() for t in (a.walkers, a.weights, a.overlaps, a.pop_shift, a.e_estimate)])
    y = engine.DeviceState(*[t.clone() for t in (a.walkers, a.weights, a.overlaps, a.pop_shift, a.e_estimate)])
    engine.block(pa, z0a, x, 5, 100, zeta=0.5)
    engine.block(pb, z0b, y, 5, 100, zeta=0.5)
    assert engine.workspace_status() == 0
    rel = float(((x.overlaps - y.overlaps).abs() / x.overlaps.abs()).max().item())
    assert rel < 1e-10, rel


@pytest.mark.parametrize("n,o,G,W", [(45, 7, 60, 33), (12, 6, 48, 9), (100, 31, 200, 17), (37, 1, 40, 5),
                                     (200, 30, 300, 3)])
def test_tensor_core_overlap_shapes(cuda, n, o, G, W):
    """The tensor-core m at ragged shapes: norb not a multiple of the eight
    orbitals of a K step (a short last copy), nocc odd (a zero pad row pair in
    B), an odd walker count (a last tile of one walker), nocc 1 and 31.
    Overlaps after a block of zero steps against the binary64 form, 1e-10
    relative."""
    from ad_afqmc_prototype_gb300 import engine, synth
    wl = synth.Workload(name=f"oz_n{n}_o{o}_g{G}", nbasis=n, nocc=o, nchol=G, n_walkers=W, n_steps=3, seed=7)
    pa, pra, st = _setup(wl, W, "fp64", n_prop_steps=3)
    pb, prb, _ = _setup(wl, W, "mixed_fast", n_prop_steps=3)
    a = _dstate(st)
    engine.block(pa, pra, a, 5, 0)  # move the walkers off the trial
    z0a = pra.__class__(**{**pra.__dict__, "n_prop_steps": 0})
    z0b = prb.__class__(**{**prb.__dict__, "n_prop_steps": 0})
    x = engine.DeviceState(*[t.clone() for t in (a.walkers, a.weights, a.overlaps, a.pop_shift, a.e_estimate)])
    y = engine.DeviceState(*[t.clone() for t in (a.walkers, a.weights, a.overlaps, a.pop_shift, a.e_estimate)])
    engine.block(pa, z0a, x, 5, 100, zeta=0.5)
    engine.block(pb, z0b, y, 5, 100, zeta=0.5)
    assert engine.workspace_status() == 0
    rel = float(((x.overlaps - y.overlaps).abs() / x.overlaps.abs()).max().item())
    print(f"n={n} o={o} W={W}: max relative overlap difference {rel:.3e}")
    assert rel < 1e-10, rel


def test_large_walker_qr_matches_numpy(cuda):
    """400 x 50 walkers do not fit in shared memory: the Householder QR runs
    in place in global memory; Q equals numpy's phase-fixed Q."""
    from ad_afqmc_prototype_gb300 import engine
    from oracle import afqmc_oracle as O
    rng = np.random.default_rng(4)
    w = rng.normal(size=(3, 400, 50)) + 1j * rng.normal(size=(3, 400, 50))
    q, det = engine.orthogonalize(torch.as_tensor(w, device="cuda"))
    qo, deto = O.qr_phase(w)
    np.testing.assert_allclose(q.cpu().numpy(), qo, rtol=0, atol=1e-12)
    np.testing.assert_allclose(det.cpu().numpy().real, np.abs(deto), rtol=1e-11)


@pytest.mark.parametrize("prec", PRECISIONS)
def test_c5_block_matches_fp64(cuda, prec):
    """nbasis 400, nocc 50, nchol 2000: one 10-step block (QR after step 5)
    of the mixed form against the binary64 form on the same fields, within
    0.1 mHa; the QRs take the global-memory path at this size."""
    from ad_afqmc_prototype_gb300 import engine
    W = 64
    pa, pra, st = _setup("c5_n400_o50_g2000_w1024", W, "fp64", n_prop_steps=10, qr_every=5)
    pb, prb, _ = _setup("c5_n400_o50_g2000_w1024", W, prec, n_prop_steps=10, qr_every=5)
    ref = _dstate(st)
    b = engine.DeviceState(*[t.clone() for t in (ref.walkers, ref.weights, ref.overlaps, ref.pop_shift,
                                                  ref.e_estimate)])
    f = engine.fill_normal((10, W, pa.nchol), 9, 0)
    ea, wa = engine.block(pa, pra, ref, 0, 0, fields=f, zeta=0.25)
    eb, wb = engine.block(pb, prb, b, 0, 0, fields=f, zeta=0.25)
    assert engine.workspace_status() == 0
    print(f"C5 {prec}: E_fp64 {float(ea):.8f}  |dE| {abs(float(ea) - float(eb)):.2e}")
    assert abs(float(ea) - float(eb)) < 1e-4


def test_three_section_field_shift_against_binary64(cuda):
    """The three-section form's field shift (fp32 terms, fp32 lane sums, binary64
    warp sum) against the six-section kernel (binary64 throughout) on the same
    fp32 force bias, at the 200-orbital workload's 1000 Cholesky vectors with
    the binary64 force bias of its trial walkers: shift_term and fb_term (the
    two weight sums in the exponent of the walker weight) to 2e-6 relative of
    their magnitude (observed: about 2e-7)."""
    import ctypes
    from ad_afqmc_prototype_gb300 import _lib, engine
    from tests.test_gpu_step import cpu
    pb, params, st = _setup("c4_n200_o30_g1000_w4096", 256, "fp64")
    W, G = 256, pb.nchol
    rng = np.random.default_rng(11)
    w = st.walkers + 0.05 * torch.as_tensor(rng.normal(size=tuple(st.walkers.shape)), device="cuda")
    fb = engine.force_bias(w.contiguous(), pb.mo, pb.rot_chol, True)  # (W, G) c128
    half = torch.cat([fb.real, fb.imag], 0).mul(0.5).to(torch.float32).contiguous()  # (2W, G)
    x = torch.as_tensor(rng.standard_normal((W, G)), device="cuda")
    lib = _lib.load()
    out = {}
    for sec in (3, 6):
        nb = int(lib.afq_field_shift_lowp_bytes(W, G, sec))
        split = torch.empty((nb,), dtype=torch.uint8, device="cuda")
        sh = torch.empty((W,), dtype=torch.complex128, device="cuda")
        ft = torch.empty((W,), dtype=torch.complex128, device="cuda")
        _lib.call("afq_field_shift_lowp", W, G, sec, float(np.sqrt(params.dt)), engine.ptr(x), engine.ptr(half),
                  engine.ptr(pb.mf_shifts), engine.ptr(sh), engine.ptr(ft), engine.ptr(split), nb,
                  engine.stream_ptr())
        out[sec] = (cpu(sh), cpu(ft))
    for k in range(2):
        a, b = out[3][k], out[6][k]
        err = np.max(np.abs(a - b)) / np.max(np.abs(b))
        assert err < 2e-6, (k, err)
    # the binary64 kernel is the binary64 field shift of the fp32-rounded force bias
    fb32 = (half[:W].double() + 1j * half[W:].double()) * 2.0
    d = engine.make_dims(W, pb.norb, pb.nocc, G, True)
    xs = torch.empty((W, G), dtype=torch.complex128, device="cuda")
    sh = torch.empty((W,), dtype=torch.complex128, device="cuda")
    ft = torch.empty((W,), dtype=torch.complex128, device="cuda")
    _lib.call("afq_field_shift", ctypes.byref(d), float(np.sqrt(params.dt)), engine.ptr(x),
              engine.ptr(fb32.contiguous()), engine.ptr(pb.mf_shifts), engine.ptr(xs), engine.ptr(sh), engine.ptr(ft),
              engine.stream_ptr())
    np.testing.assert_allclose(out[6][0], cpu(sh), rtol=1e-12, atol=1e-12 * np.max(np.abs(cpu(sh))))
    np.testing.assert_allclose(out[6][1], cpu(ft), rtol=1e-12, atol=1e-12 * np.max(np.abs(cpu(ft))))
