"""The CUDA engine against outputs of the reference's own code, and against
the oracle at the benchmark workloads' shapes.

Fixtures tests/golden/ref_*.npz come from running the reference's hot-path
modules unmodified on NumPy (tests/golden/make_ref_golden.py).  Tolerances:
binary64 kernels relative 1e-11 (energies 1e-10 Ha absolute), comb indices
bit-exact; binary64 blocks 1e-10 Ha per block energy; the mixed-precision
forms 1e-4 Ha per block (the benchmark's bound) against the binary64 oracle.
"""
import os

import numpy as np
import pytest

from oracle import afqmc_oracle as O
from tests.test_gpu_step import _setup, api, cpu  # noqa: F401  (fixture)

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _ref(name):
    return dict(np.load(os.path.join(ROOT, "tests", "golden", name)))


@pytest.fixture(scope="module")
def E(cuda):
    from ad_afqmc_prototype_gb300 import engine
    return engine


@pytest.mark.parametrize("tag", ["real", "cplx"])
def test_kernels_match_reference(E, tag):
    """meas/rhf.py:15-50,141-150 and prop/chol_afqmc_ops.py:77-103 outputs."""
    g = _ref("ref_kernels.npz")
    real = tag == "real"
    mo = E.as_device(g[f"{tag}_mo"], E.C128)
    h1, chol = E.as_device(g["h1"], E.F64), E.as_device(g["chol"], E.F64)
    rot_h1, rot_chol = E.build_meas_ctx(h1, chol, mo, real)
    np.testing.assert_allclose(cpu(rot_h1), g[f"{tag}_rot_h1"], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(cpu(rot_chol), g[f"{tag}_rot_chol"], rtol=1e-12, atol=1e-14)
    w = E.as_device(g["walkers"], E.C128)
    np.testing.assert_allclose(cpu(E.overlap(w, mo, real)), g[f"{tag}_overlap"], rtol=1e-11)
    green, _ = E.half_green(w, mo, real, with_overlap=True)
    np.testing.assert_allclose(cpu(green), g[f"{tag}_green"], rtol=1e-11, atol=1e-13)
    np.testing.assert_allclose(cpu(E.force_bias(w, mo, rot_chol, real)), g[f"{tag}_fb"], rtol=1e-11, atol=1e-12)
    e = cpu(E.energy(w, float(g["h0"]), mo, rot_h1, rot_chol, real))
    np.testing.assert_allclose(e, g[f"{tag}_energy"], rtol=1e-11, atol=1e-10)
    ex, mf, h0p = E.build_prop_ctx(float(g["h0"]), h1, chol, E.as_device(O.get_rdm1(g[f"{tag}_mo"]), E.C128),
                                   float(g["dt"]))
    np.testing.assert_allclose(cpu(ex), g[f"{tag}_exp_h1_half"], rtol=1e-13, atol=1e-14)
    np.testing.assert_allclose(cpu(mf), g[f"{tag}_mf"], rtol=1e-12, atol=1e-13)
    np.testing.assert_allclose(cpu(h0p)[0], g[f"{tag}_h0_prop"], rtol=1e-12)


def test_trotter_qr_comb_match_reference(E):
    """apply_trotter (prop/chol_afqmc_ops.py:173-183), _qr / orthogonalize
    (walkers.py:169-203) and _sr_indices on dyadic weights (walkers.py:233-240)."""
    g = _ref("ref_kernels.npz")
    dt = float(g["dt"])
    ctx = O.build_prop_ctx(float(g["h0"]), g["h1"], g["chol"], O.get_rdm1(g["real_mo"]), dt)
    out = E.apply_trotter(E.as_device(g["walkers"], E.C128), E.as_device(g["trotter_fields"], E.C128),
                          E.as_device(g["chol"], E.F64), E.as_device(ctx.exp_h1_half, E.F64), float(np.sqrt(dt)), 6)
    np.testing.assert_allclose(cpu(out), g["trotter_out"], rtol=1e-11, atol=1e-12)
    q, det = E.orthogonalize(E.as_device(g["walkers"], E.C128))
    np.testing.assert_allclose(cpu(q), g["qr_q"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(cpu(det) ** 2, g["orth_norm"], rtol=1e-11)
    for k in range(5):
        w, z = g[f"sr{k}_weights"], float(g[f"sr{k}_zeta"])
        idx, _ = E.sr_indices(E.as_device(w, E.F64), z)
        np.testing.assert_array_equal(cpu(idx), g[f"sr{k}_idx"])


def _blocks_vs_reference(api, ref, H, W, n_steps, tol_e):
    w0 = ref["init_walkers"]
    sys_, state, kw = _setup(api, {**H, "mo_coeff": ref["mo_coeff"]}, W, dt=0.005, n_prop_steps=n_steps,
                             qr_every=0)
    assert abs(float(state.e_estimate) - float(ref["e_estimate"])) < 1e-10
    if w0.shape[0] == W:
        np.testing.assert_array_equal(cpu(state.walkers), w0)
    s1 = api["afqmc_step"](state, fields=ref["fields"][0, 0], **kw)
    nk = ref["step1_walkers"].shape[0]
    np.testing.assert_allclose(cpu(s1.walkers)[:nk], ref["step1_walkers"], atol=1e-11)
    np.testing.assert_allclose(cpu(s1.weights), ref["step1_weights"], rtol=1e-10)
    from ad_afqmc_prototype_gb300.prop.afqmc import device_state, engine_problem
    prob = engine_problem(n_walkers=W, need_energy=True, **kw)
    st = device_state(state, inplace=False)
    for b in range(ref["fields"].shape[0]):
        e, wsum, idx = api["engine"].block(prob, kw["params"], st, 0, 0, fields=ref["fields"][b],
                                           zeta=float(ref["zetas"][b]), return_idx=True)
        np.testing.assert_array_equal(cpu(idx), ref["sr_idx"][b])
        assert abs(float(e) - ref["block_energy"][b]) < tol_e, (b, float(e), ref["block_energy"][b])
        assert abs(float(wsum) - ref["block_weight"][b]) < 1e-9 * abs(ref["block_weight"][b])
    nk = ref["final_walkers"].shape[0]
    np.testing.assert_allclose(cpu(st.walkers)[:nk], ref["final_walkers"], atol=1e-10)
    np.testing.assert_allclose(cpu(st.weights), ref["final_weights"], rtol=1e-10)


def test_block_c1_matches_reference(api):
    """Two of the reference's afqmc_blocks (prop/blocks.py:22-95) on the
    12-orbital workload, 32 walkers, the reference's own draws."""
    H = api["synth"].make_workload(api["synth"].WORKLOADS["c1_n12_o6_g48_w256"])
    _blocks_vs_reference(api, _ref("ref_block_c1.npz"), H, W=32, n_steps=10, tol_e=1e-10)


def test_block_c4_shape_matches_reference(api):
    """One of the reference's blocks (4 steps) on the benchmark's 200-orbital,
    1000-vector Hamiltonian, 4 walkers."""
    H = api["synth"].make_workload(api["synth"].WORKLOADS["c4_n200_o30_g1000_w4096"])
    _blocks_vs_reference(api, _ref("ref_block_c4.npz"), H, W=4, n_steps=4, tol_e=1e-10)


_ORACLE_RUNS = {}


def _oracle_block(api, wl, W, n_steps, qr_every, seed):
    """One oracle block from the trial walkers on seeded fields (cached: the
    400-orbital run takes tens of seconds on the host)."""
    key = (wl, W, n_steps, qr_every, seed)
    if key not in _ORACLE_RUNS:
        H = api["synth"].make_workload(api["synth"].WORKLOADS[wl])
        prob = O.make_problem(H["h0"], H["h1"], H["chol"], H["mo_coeff"], 0.005)
        P = O.Params(dt=0.005, n_prop_steps=n_steps, qr_every=qr_every)
        ost = O.init_prop_state(prob, W, api["synth"].trial_walkers(H["mo_coeff"], W))
        rng = np.random.default_rng(seed)
        fields = rng.standard_normal((n_steps, W, H["chol"].shape[0]))
        zeta = float(rng.random())
        ost, oobs, _ = O.afqmc_block(prob, P, ost, fields, zeta)
        _ORACLE_RUNS[key] = (H, fields, zeta, ost, oobs["energy"])
    return _ORACLE_RUNS[key]


def _engine_vs_oracle(api, wl, W, n_steps, qr_every, precision, seed):
    """One block of the engine and of the oracle from the same state and fields."""
    H, fields, zeta, ost, oe = _oracle_block(api, wl, W, n_steps, qr_every, seed)
    sys_, state, kw = _setup(api, H, W, dt=0.005, n_prop_steps=n_steps, qr_every=qr_every, precision=precision)
    out, obs = api["afqmc_block"](state, sys=sys_, fields=fields, zeta=zeta, **kw)
    return float(obs.scalars["energy"]), oe, out, ost


@pytest.mark.parametrize("wl,W,n_steps,qr_every", [("c4_n200_o30_g1000_w4096", 16, 10, 5),
                                                   ("c5_n400_o50_g2000_w1024", 8, 4, 2)])
def test_fp64_block_matches_oracle_at_benchmark_shapes(api, wl, W, n_steps, qr_every):
    """The binary64 block at the 200- and 400-orbital workloads' Hamiltonians
    (the shapes of the benchmark's main and large lines): 1e-10 Ha."""
    e, oe, out, ost = _engine_vs_oracle(api, wl, W, n_steps, qr_every, "fp64", 5)
    assert abs(e - oe) < 1e-10, (e, oe)
    np.testing.assert_allclose(cpu(out.walkers), ost.walkers, atol=1e-10)
    np.testing.assert_allclose(cpu(out.weights), ost.weights, rtol=1e-10)


@pytest.mark.parametrize("precision", ["mixed", "mixed_fast"])
@pytest.mark.parametrize("wl,W,n_steps,qr_every", [("c4_n200_o30_g1000_w4096", 16, 10, 5),
                                                   ("c5_n400_o50_g2000_w1024", 8, 4, 2)])
def test_mixed_block_within_bound_of_oracle(api, wl, W, n_steps, qr_every, precision):
    """The mixed-precision forms against the binary64 oracle on the same
    state and fields: block energy within 0.1 mHa."""
    e, oe, _, _ = _engine_vs_oracle(api, wl, W, n_steps, qr_every, precision, 5)
    assert abs(e - oe) < 1e-4, (precision, e, oe)
