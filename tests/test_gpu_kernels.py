"""GPU parity of the individual CUDA kernels against the CPU oracle, through
the C ABI.  Tolerances (binary64 on both sides): relative 1e-11 on kernel
outputs, 1e-10 Ha absolute on energies; comb indices bit-exact."""
import os

import numpy as np
import pytest
import torch

from oracle import afqmc_oracle as O
from tests import philox_ref

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = np.load(os.path.join(ROOT, "tests", "golden", "kernels.npz"))


def cpu(t):
    return t.detach().cpu().numpy()


def dev(x, dtype):
    from ad_afqmc_prototype_gb300 import engine
    return engine.as_device(x, dtype)


@pytest.fixture(scope="module")
def E(cuda):
    from ad_afqmc_prototype_gb300 import engine
    return engine


@pytest.mark.parametrize("tag", ["real", "cplx"])
def test_meas_kernels_match_golden(E, tag):
    g = GOLD
    c = g[f"{tag}_mo"]
    real = tag == "real"
    mo = dev(c, E.C128)
    h1, chol = dev(g["h1"], E.F64), dev(g["chol"], E.F64)
    rot_h1, rot_chol = E.build_meas_ctx(h1, chol, mo, real)
    np.testing.assert_allclose(cpu(rot_chol), g[f"{tag}_rot_chol"], rtol=1e-12, atol=1e-14)
    w = dev(g["walkers"], E.C128)
    np.testing.assert_allclose(cpu(E.overlap(w, mo, real)), g[f"{tag}_overlap"], rtol=1e-11)
    green, ov = E.half_green(w, mo, real, with_overlap=True)
    np.testing.assert_allclose(cpu(green), g[f"{tag}_green"], rtol=1e-11, atol=1e-13)
    np.testing.assert_allclose(cpu(ov), g[f"{tag}_overlap"], rtol=1e-11)
    np.testing.assert_allclose(cpu(E.force_bias(w, mo, rot_chol, real)), g[f"{tag}_fb"], rtol=1e-11, atol=1e-12)
    e = cpu(E.energy(w, float(g["h0"]), mo, rot_h1, rot_chol, real))
    np.testing.assert_allclose(e, g[f"{tag}_energy"], rtol=1e-11, atol=1e-10)


@pytest.mark.parametrize("tag", ["real", "cplx"])
def test_prop_ctx_matches_golden(E, tag):
    g = GOLD
    c = g[f"{tag}_mo"]
    rdm1 = O.get_rdm1(c)
    e, mf, h0p = E.build_prop_ctx(float(g["h0"]), dev(g["h1"], E.F64), dev(g["chol"], E.F64),
                                  dev(rdm1, E.C128), 0.01)
    np.testing.assert_allclose(cpu(e), g[f"{tag}_exp_h1_half"], rtol=1e-13, atol=1e-14)
    np.testing.assert_allclose(cpu(mf), g[f"{tag}_mf"], rtol=1e-12, atol=1e-13)
    np.testing.assert_allclose(cpu(h0p)[0], g[f"{tag}_h0_prop"], rtol=1e-12)


def test_expm_with_squaring(E):
    rng = np.random.default_rng(3)
    n, gch = 40, 3
    a = rng.normal(size=(n, n))
    h1 = 30.0 * (a + a.T)  # large norm: several squarings
    chol = np.zeros((gch, n, n))
    e, _, _ = E.build_prop_ctx(0.0, dev(h1, E.F64), dev(chol, E.F64), dev(np.zeros((n, n)), E.C128), 0.5)
    ref = O.build_prop_ctx(0.0, h1, chol, np.zeros((n, n)), 0.5).exp_h1_half
    np.testing.assert_allclose(cpu(e), ref, rtol=1e-9, atol=1e-12 * np.abs(ref).max())


@pytest.mark.parametrize("n,o,G,W", [(12, 6, 48, 33), (60, 10, 300, 16), (120, 20, 600, 8), (200, 30, 64, 4)])
def test_apply_trotter_matches_oracle(E, n, o, G, W):
    rng = np.random.default_rng(n + o)
    a = rng.normal(size=(n, n))
    h1 = 0.1 * (a + a.T)
    b = rng.normal(size=(G, n, n))
    chol = (3.6 / n) * 0.5 * (b + np.swapaxes(b, 1, 2))
    c = np.linalg.qr(rng.normal(size=(n, o)))[0]
    ctx = O.build_prop_ctx(0.0, h1, chol, O.get_rdm1(c), 0.005)
    w = rng.normal(size=(W, n, o)) + 1j * rng.normal(size=(W, n, o))
    x = rng.normal(size=(W, G)) + 0.1j * rng.normal(size=(W, G))
    ref = O.apply_trotter_r(w, x, ctx, chol.reshape(G, -1), 6)
    out = E.apply_trotter(dev(w, E.C128), dev(x, E.C128), dev(chol, E.F64), dev(ctx.exp_h1_half, E.F64),
                          float(np.sqrt(0.005)), 6)
    np.testing.assert_allclose(cpu(out), ref, rtol=1e-11, atol=1e-12)
    # chunked V workspace gives the same walkers
    out2 = E.apply_trotter(dev(w, E.C128), dev(x, E.C128), dev(chol, E.F64), dev(ctx.exp_h1_half, E.F64),
                           float(np.sqrt(0.005)), 6, n_chunks=3)
    np.testing.assert_allclose(cpu(out2), cpu(out), rtol=0, atol=0)


@pytest.mark.parametrize("n,o,W", [(12, 6, 5), (200, 30, 3), (64, 64, 2), (9, 1, 4)])
def test_qr_matches_oracle(E, n, o, W):
    rng = np.random.default_rng(o)
    w = rng.normal(size=(W, n, o)) + 1j * rng.normal(size=(W, n, o))
    q, det = E.orthogonalize(dev(w, E.C128))
    qr, dr = O.qr_phase(w)
    np.testing.assert_allclose(cpu(q), qr, rtol=0, atol=1e-12)
    np.testing.assert_allclose(cpu(det), dr, rtol=1e-11)


@pytest.mark.parametrize("n,o,W,cond", [(12, 6, 5, 0), (200, 30, 3, 0), (64, 64, 2, 0), (9, 1, 4, 0),
                                        (120, 20, 3, 1e4)])
def test_cholqr2_matches_oracle(E, n, o, W, cond):
    """The mixed forms' CholeskyQR2 gives the Householder form's unique Q and
    det(R); cond > 0 mixes the columns through singular values spanning
    `cond`, past what the fp32 first Gram matrix resolves (the binary64
    retry)."""
    from ad_afqmc_prototype_gb300 import _lib
    rng = np.random.default_rng(o + 7)
    w = rng.normal(size=(W, n, o)) + 1j * rng.normal(size=(W, n, o))
    if cond:
        u, _ = np.linalg.qr(rng.normal(size=(o, o)))
        v, _ = np.linalg.qr(rng.normal(size=(o, o)))
        w = w @ (u * np.logspace(0, -np.log10(cond), o)[None, :] @ v)
    for prec in (_lib.AFQ_PREC_MIXED, _lib.AFQ_PREC_MIXED_FAST):
        q, det = E.orthogonalize(dev(w, E.C128), precision=prec)
        qr, dr = O.qr_phase(w)
        np.testing.assert_allclose(cpu(q), qr, rtol=0, atol=1e-10)
        np.testing.assert_allclose(cpu(det), dr, rtol=1e-10)


@pytest.mark.parametrize("W", [1, 2, 3, 31, 32, 33, 256, 1000, 4096, 5000])
def test_comb_indices_bit_exact(E, W):
    rng = np.random.default_rng(W)
    w = rng.random(W) * rng.choice([0.0, 1.0, 1e-3, 7.0], size=W)
    if not np.any(w):
        w[0] = 1.0
    for zeta in (0.0, 0.3141, 0.999999):
        idx, cw = E.sr_indices(dev(w, E.F64), zeta)
        ridx, rcw = O.sr_indices(w, zeta, W)
        np.testing.assert_array_equal(cpu(cw), rcw)  # same bits
        np.testing.assert_array_equal(cpu(idx), ridx)


def test_comb_edge_cases(E):
    W = 100
    w = np.zeros(W)
    idx, _ = E.sr_indices(dev(w, E.F64), 0.5)
    assert np.all(cpu(idx) == 0)  # all-zero weights
    w[37] = 2.5
    idx, _ = E.sr_indices(dev(w, E.F64), 0.5)
    assert np.all(cpu(idx) == 37)  # a single surviving walker
    idx, _ = E.sr_indices(dev(-np.ones(W), E.F64), 0.25)
    np.testing.assert_array_equal(cpu(idx), np.arange(W))  # |w| and the identity comb
    d = (np.random.default_rng(0).integers(0, 1 << 16, W) / 64.0)  # dyadic: order independent
    idx, cw = E.sr_indices(dev(d, E.F64), 0.5)
    np.testing.assert_array_equal(cpu(cw), np.cumsum(d))
    z = d.sum() * (np.arange(W) + 0.5) / W
    np.testing.assert_array_equal(cpu(idx), np.minimum(np.searchsorted(np.cumsum(d), z, side="left"), W - 1))


def test_stochastic_reconfiguration_gathers(E):
    rng = np.random.default_rng(5)
    W, n, o = 300, 12, 6
    w = rng.normal(size=(W, n, o)) + 1j * rng.normal(size=(W, n, o))
    wt = rng.random(W) * (rng.random(W) > 0.2)
    out, wout, idx = E.stochastic_reconfiguration(dev(w, E.C128), dev(wt, E.F64), 0.42)
    rw, rwt, ridx = O.stochastic_reconfiguration(w, wt, 0.42)
    np.testing.assert_array_equal(cpu(idx), ridx)
    np.testing.assert_array_equal(cpu(out), rw)
    np.testing.assert_array_equal(cpu(wout), rwt)


def test_philox_matches_cpu_mirror(E):
    for count, seed, ctr in ((1, 0, 0), (7, 42, 3), (10001, 2**40 + 5, 2**33 + 1)):
        u = cpu(E.fill_uniform((count,), seed, ctr))
        np.testing.assert_array_equal(u, philox_ref.uniform(count, seed, ctr))
        x = cpu(E.fill_normal((count,), seed, ctr))
        # the device's fp32 log / sqrt / sincospi against float64 of the same inputs
        np.testing.assert_allclose(x, philox_ref.normal(count, seed, ctr), rtol=2e-6, atol=2e-6)


def test_field_shift_and_weight_update_match_oracle(E):
    from ad_afqmc_prototype_gb300.prop.types import afqmc_params
    rng = np.random.default_rng(8)
    W, G = 77, 29
    x = rng.normal(size=(W, G))
    fb = 0.3 * (rng.normal(size=(W, G)) + 1j * rng.normal(size=(W, G)))
    mf = 1j * rng.normal(size=G) + 0.01 * rng.normal(size=G)
    xs, st_, ft = E.field_shift(dev(x, E.F64), dev(fb, E.C128), dev(mf, E.C128), np.sqrt(0.01))
    fs = -np.sqrt(0.01) * (1j * fb - mf)
    np.testing.assert_allclose(cpu(xs), x - fs, rtol=1e-13, atol=1e-14)
    np.testing.assert_allclose(cpu(st_), np.sum((x - fs) * mf, axis=1), rtol=1e-12, atol=1e-13)
    np.testing.assert_allclose(cpu(ft), np.sum(x * fs - 0.5 * fs * fs, axis=1), rtol=1e-12, atol=1e-13)
    # weight update on the same terms, with overlaps that trip floor and cap
    ov_old = np.exp(rng.normal(size=W) + 1j * rng.normal(size=W))
    ov_new = ov_old * np.exp(0.5 * rng.normal(size=W) + 0.3j * rng.normal(size=W))
    ov_new[:3] = [0.0, 1e6 * ov_old[1], -ov_old[2]]
    weights = rng.random(W) * 3
    weights[5] = 99.0
    prob = O.Problem(h0=0.0, h1=None, chol=None, mo_coeff=None, meas_ctx=None,
                     prop_ctx=O.PropCtx(dt=0.01, sqrt_dt=np.sqrt(0.01), exp_h1_half=None, mf_shifts=mf,
                                        h0_prop=complex(-3.0 + 0.2j)))
    P = O.Params(dt=0.01)
    ost = O.State(walkers=None, weights=weights.copy(), overlaps=ov_old.copy(), pop_control_ene_shift=-2.5,
                  e_estimate=-2.0)
    _, rw, rpop = O.step_weights(prob, P, ost, x, fb, ov_new)
    lite = E.Problem(n_walkers=W, norb=1, nocc=1, nchol=G, trial_is_real=True, h0=0.0, chol=None, mo=None,
                     dt=0.01, sqrt_dt=float(np.sqrt(0.01)), exp_h1_half=None, mf_shifts=None,
                     h0_prop=complex(-3.0 + 0.2j), rot_h1=None, rot_chol=None)
    dst = E.DeviceState(walkers=dev(np.zeros((W, 1, 1)), E.C128), weights=dev(weights, E.F64),
                        overlaps=dev(ov_old, E.C128), pop_shift=dev(np.array([-2.5]), E.F64),
                        e_estimate=dev(np.array([-2.0]), E.F64))
    E.weight_update(lite, afqmc_params(dt=0.01), st_, ft, dev(ov_new, E.C128), dst)
    np.testing.assert_allclose(cpu(dst.weights), rw, rtol=1e-12, atol=1e-300)
    assert np.sum(cpu(dst.weights) == 0) == np.sum(rw == 0)
    assert abs(float(cpu(dst.pop_shift)[0]) - rpop) < 1e-10
    np.testing.assert_array_equal(cpu(dst.overlaps), ov_new)


@pytest.mark.parametrize("cplx", [False, True])
def test_trial_rdm1_matches_oracle(E, cplx):
    """get_rdm1 (trial/rhf.py:29-32) by the engine's kernel: [C C^H, C C^H]."""
    rng = np.random.default_rng(21)
    n, o = 37, 9
    c = rng.normal(size=(n, o)) + (1j * rng.normal(size=(n, o)) if cplx else 0)
    out = cpu(E.trial_rdm1(dev(c, E.C128)))
    np.testing.assert_allclose(out, O.get_rdm1(c), rtol=0, atol=1e-13)
