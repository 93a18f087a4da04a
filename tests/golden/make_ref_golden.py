"""Golden vectors produced by the reference's own hot-path code.

    python tests/golden/make_ref_golden.py        (needs the reference checkout)

The reference (ad_afqmc_prototype) is a JAX program and JAX cannot be
installed here.  Its hot-path modules only use a small part of JAX (jnp
array functions, vmap, lax.scan, jax.random draws, scipy expm), so this
script runs them UNMODIFIED on NumPy: tests/golden/jax_standin/ is put first
on sys.path as the `jax` package, and the reference package is imported from
its checkout by path.  Random draws are injected through the stand-in's
queue (jax.random.normal / uniform return the arrays given to `feed`), so
the reference consumes exactly the fields and comb uniforms recorded here.

Functions executed (reference file:line):
  meas/rhf.py:15-50       _half_green_from_overlap_matrix, overlap_r,
                          force_bias_kernel_r, energy_kernel_r
  meas/rhf.py:141-150     build_meas_ctx
  prop/chol_afqmc_ops.py  _build_prop_ctx (:77-103), make_chol_afqmc_ops
                          (:215-262) -> apply_trotter (_apply_trotter_r :173-183)
  prop/utils.py:20-31     taylor_expm_action
  walkers.py:169-211      _qr, orthogonalize
  walkers.py:233-265      _sr_indices, stochastic_reconfiguration
  prop/afqmc.py:17-147    init_prop_state, afqmc_step
  prop/blocks.py:22-95    afqmc_block

What the stand-in cannot reproduce: jnp.cumsum runs as NumPy's sequential
sum, not XLA's association order, so comb indices are pinned with dyadic
weights (exact in every order) and the block fixtures record the indices
the reference's comb chose (recovered from its output walkers).

Outputs (tests/golden/): ref_kernels.npz, ref_block_c1.npz, ref_block_c4.npz.
"""
from __future__ import annotations

import importlib
import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("AFQ_REFERENCE", "/root/reference")
sys.dont_write_bytecode = True  # the reference checkout is read-only


def load_reference():
    """Imports the reference package from its checkout with the NumPy stand-in as `jax`."""
    sys.path.insert(0, os.path.join(HERE, "jax_standin"))
    import jax  # noqa: F401  (the stand-in)
    assert jax.__version__.endswith("numpy-standin"), "a real jax shadows the stand-in"
    pkg_dir = os.path.join(REF, "ad_afqmc_prototype")
    spec = importlib.util.spec_from_file_location("ad_afqmc_prototype", os.path.join(pkg_dir, "__init__.py"),
                                                  submodule_search_locations=[pkg_dir])
    pkg = importlib.util.module_from_spec(spec)
    sys.modules["ad_afqmc_prototype"] = pkg
    spec.loader.exec_module(pkg)
    mods = {}
    for name in ("core.system", "core.ops", "ham.chol", "trial.rhf", "meas.rhf", "prop.utils",
                 "prop.chol_afqmc_ops", "prop.types", "prop.afqmc", "prop.blocks", "walkers"):
        mods[name] = importlib.import_module("ad_afqmc_prototype." + name)
    return mods


def _sym(b):
    return 0.5 * (b + np.swapaxes(b, -1, -2))


def make_kernels(R):
    """Per-walker kernels on random walkers, real and complex trials."""
    import jax
    rng = np.random.default_rng(2718)
    n, o, g, W = 10, 4, 7, 6
    h1 = _sym(rng.normal(size=(n, n)))
    chol = 0.2 * _sym(rng.normal(size=(g, n, n)))
    h0 = 0.37
    dt = 0.01
    walkers = rng.normal(size=(W, n, o)) + 1j * rng.normal(size=(W, n, o))
    out = {"h1": h1, "chol": chol, "h0": np.array(h0), "dt": np.array(dt), "walkers": walkers}
    ham = R["ham.chol"].ham_chol(h0=np.array(h0), h1=h1, chol=chol)
    sys_ = R["core.system"].system(norb=n, nelec=(o, o), walker_kind="restricted")
    mrhf, trhf, ops = R["meas.rhf"], R["trial.rhf"], R["prop.chol_afqmc_ops"]
    for tag, cplx in (("real", False), ("cplx", True)):
        m = rng.normal(size=(n, o)) + (1j * rng.normal(size=(n, o)) if cplx else 0)
        c = np.linalg.qr(m)[0]
        trial = trhf.rhf_trial(mo_coeff=c)
        mctx = mrhf.build_meas_ctx(ham, trial)
        pctx = ops._build_prop_ctx(ham, trhf.get_rdm1(trial), dt)
        meas = mrhf.make_rhf_meas_ops(sys_)
        out[f"{tag}_mo"] = c
        out[f"{tag}_rot_h1"] = mctx.rot_h1
        out[f"{tag}_rot_chol"] = mctx.rot_chol
        out[f"{tag}_exp_h1_half"] = pctx.exp_h1_half
        out[f"{tag}_mf"] = pctx.mf_shifts
        out[f"{tag}_h0_prop"] = np.array(pctx.h0_prop)
        out[f"{tag}_overlap"] = jax.vmap(lambda w: meas.overlap(w, trial))(walkers)
        out[f"{tag}_green"] = jax.vmap(lambda w: mrhf._half_green_from_overlap_matrix(
            w, c.conj().T @ w))(walkers)
        fb = meas.require_kernel("force_bias")
        out[f"{tag}_fb"] = jax.vmap(lambda w: fb(w, ham, mctx, trial))(walkers)
        en = meas.require_kernel("energy")
        out[f"{tag}_energy"] = jax.vmap(lambda w: en(w, ham, mctx, trial))(walkers)
    # Taylor action of a random complex V on random walkers, six terms, a = i sqrt(dt)
    V = rng.normal(size=(W, n, n)) + 1j * rng.normal(size=(W, n, n))
    a = 1j * np.sqrt(dt)
    out["taylor_V"] = V
    out["taylor_out"] = np.stack([R["prop.utils"].taylor_expm_action(a, V[i], walkers[i], 6) for i in range(W)])
    # apply_trotter with the real trial's context on complex shifted fields
    p_ops = ops.make_chol_afqmc_ops(ham, "restricted")
    pctx = ops._build_prop_ctx(ham, trhf.get_rdm1(trhf.rhf_trial(mo_coeff=out["real_mo"])), dt)
    x = rng.normal(size=(W, g)) + 1j * rng.normal(size=(W, g))
    out["trotter_fields"] = x
    out["trotter_out"] = np.stack([p_ops.apply_trotter(walkers[i], x[i], pctx, 6) for i in range(W)])
    # phase-fixed QR and the restricted normalisation
    wk = R["walkers"]
    q, det_r = jax.vmap(wk._qr)(walkers)
    out["qr_q"], out["qr_det_r"] = q, det_r
    q2, norm = wk.orthogonalize(walkers, "restricted")
    out["orth_q"], out["orth_norm"] = q2, norm
    # comb indices on dyadic weights (exact prefix sums in every association order)
    for k, nw in enumerate((1, 7, 64, 257, 1000)):
        wts = rng.integers(0, 1 << 12, size=nw).astype(np.float64) / 1024.0
        wts[rng.random(nw) < 0.1] = 0.0
        if wts.sum() == 0:
            wts[0] = 1.0
        z = float(rng.integers(0, 1 << 20)) / (1 << 20)
        out[f"sr{k}_weights"], out[f"sr{k}_zeta"] = wts, np.array(z)
        out[f"sr{k}_idx"] = np.asarray(wk._sr_indices(wts, z, nw))
        ws, wn = wk.stochastic_reconfiguration(walkers[np.arange(nw) % W], wts, z, "restricted")
        out[f"sr{k}_weights_new"] = wn
    np.savez_compressed(os.path.join(HERE, "ref_kernels.npz"), **out)
    return out


def run_reference_blocks(R, H, W, n_steps, n_blocks, seed, w0=None):
    """The reference's init_prop_state and afqmc_block on injected draws."""
    import jax
    n, o = H["h1"].shape[0], H["mo_coeff"].shape[1]
    G = H["chol"].shape[0]
    sys_ = R["core.system"].system(norb=n, nelec=(o, o), walker_kind="restricted")
    ham = R["ham.chol"].ham_chol(h0=np.array(H["h0"]), h1=H["h1"], chol=H["chol"])
    trial = R["trial.rhf"].rhf_trial(mo_coeff=H["mo_coeff"])
    t_ops = R["trial.rhf"].make_rhf_trial_ops(sys_)
    m_ops = R["meas.rhf"].make_rhf_meas_ops(sys_)
    p_ops = R["prop.chol_afqmc_ops"].make_chol_afqmc_ops(ham, "restricted")
    params = R["prop.types"].afqmc_params(dt=0.005, n_prop_steps=n_steps, n_walkers=W, seed=seed)
    pctx = p_ops.build_prop_ctx(t_ops.get_rdm1(trial), params.dt)
    mctx = m_ops.build_meas_ctx(ham, trial)
    if w0 is None:
        w0 = np.ascontiguousarray(np.broadcast_to(H["mo_coeff"].astype(np.complex128), (W, n, o)))
    st = R["prop.afqmc"].init_prop_state(sys=sys_, n_walkers=W, seed=seed, ham_data=ham, trial_ops_=t_ops,
                                         trial_data=trial, meas_ops=m_ops, initial_walkers=w0)
    rng = np.random.default_rng(seed)
    fields = rng.standard_normal((n_blocks, n_steps, W, G))
    zetas = rng.random(n_blocks)
    out = {"mo_coeff": H["mo_coeff"], "init_walkers": w0, "fields": fields, "zetas": zetas,
           "e_estimate": np.array(st.e_estimate), "init_overlaps": np.asarray(st.overlaps)}
    # the first step alone
    jax.random.feed(normals=[fields[0, 0]])
    s1 = R["prop.afqmc"].afqmc_step(st, params=params, ham_data=ham, trial_data=trial, meas_ops=m_ops,
                                    prop_ops=p_ops, prop_ctx=pctx, meas_ctx=mctx)
    out.update(step1_walkers=s1.walkers, step1_weights=s1.weights, step1_overlaps=s1.overlaps,
               step1_pop_shift=np.array(s1.pop_control_ene_shift))
    energies, weights, shifts, idxs = [], [], [], []
    for b in range(n_blocks):
        jax.random.feed(normals=list(fields[b]), uniforms=[zetas[b]])
        prev = st
        st, obs = R["prop.blocks"].afqmc_block(st, sys=sys_, params=params, ham_data=ham, trial_data=trial,
                                               meas_ops=m_ops, prop_ops=p_ops, prop_ctx=pctx, meas_ctx=mctx)
        assert jax.random.remaining() == (0, 0)
        energies.append(float(obs.scalars["energy"]))
        weights.append(float(obs.scalars["weight"]))
        shifts.append(float(st.pop_control_ene_shift))
        idxs.append(recover_comb_indices(st.walkers, prev, R, params, ham, trial, m_ops, p_ops, pctx, mctx,
                                         fields[b], zetas[b], sys_))
    out.update(block_energy=np.array(energies), block_weight=np.array(weights), block_pop_shift=np.array(shifts),
               sr_idx=np.array(idxs), final_walkers=np.asarray(st.walkers), final_weights=np.asarray(st.weights),
               final_overlaps=np.asarray(st.overlaps))
    return out


def recover_comb_indices(walkers_after, prev, R, params, ham, trial, m_ops, p_ops, pctx, mctx, fields, zeta, sys_):
    """The comb indices the reference's block chose: replays the block's
    propagation with the reference's functions up to the comb, then matches
    each output walker to its source row exactly."""
    import jax
    jax.random.feed(normals=list(fields))
    st = prev
    for _ in range(params.n_prop_steps):
        st = R["prop.afqmc"].afqmc_step(st, params=params, ham_data=ham, trial_data=trial, meas_ops=m_ops,
                                        prop_ops=p_ops, prop_ctx=pctx, meas_ctx=mctx)
    q = R["walkers"].orthonormalize(st.walkers, "restricted")
    idx = np.asarray(R["walkers"]._sr_indices(st.weights, zeta, q.shape[0]))
    np.testing.assert_array_equal(q[idx], walkers_after)
    return idx


def make_block_c1(R):
    sys.path.insert(0, ROOT)
    from ad_afqmc_prototype_gb300 import synth
    H = synth.make_workload(synth.WORKLOADS["c1_n12_o6_g48_w256"])
    out = run_reference_blocks(R, H, W=32, n_steps=10, n_blocks=2, seed=4242)
    np.savez_compressed(os.path.join(HERE, "ref_block_c1.npz"), **out)
    return out


def make_block_c4(R):
    """The 200-orbital workload's Hamiltonian (seed 3, regenerated by the
    tests from ad_afqmc_prototype_gb300.synth; its checksum is recorded),
    4 walkers, one block of 4 steps.  Only walker 0 of the state after the
    first step and of the final state is stored, to keep the file small."""
    sys.path.insert(0, ROOT)
    from ad_afqmc_prototype_gb300 import synth
    wl = synth.WORKLOADS["c4_n200_o30_g1000_w4096"]
    H = synth.make_workload(wl)
    out = run_reference_blocks(R, H, W=4, n_steps=4, n_blocks=1, seed=77)
    out["chol_checksum"] = np.array([H["chol"].sum(), np.abs(H["chol"]).sum(), H["h1"].sum()])
    for k in ("step1_walkers", "final_walkers", "init_walkers"):
        out[k] = out[k][:1]
    np.savez_compressed(os.path.join(HERE, "ref_block_c4.npz"), **out)
    return out


if __name__ == "__main__":
    R = load_reference()
    k = make_kernels(R)
    c1 = make_block_c1(R)
    c4 = make_block_c4(R)
    print("ref_kernels:", len(k), "arrays")
    print("ref_block_c1: E =", c1["block_energy"], "W =", c1["block_weight"])
    print("ref_block_c4: E =", c4["block_energy"], "W =", c4["block_weight"])
