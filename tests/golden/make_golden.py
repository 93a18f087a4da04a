"""Generates the golden fixtures under tests/golden/ with the CPU oracle.

    python tests/golden/make_golden.py

c1_block.npz: the 12-orbital workload (seed 0), 64 walkers starting at the
trial, two blocks of 10 steps with a QR after step 5, injected N(0,1)
fields and comb uniforms; records per-step weights / overlaps / population
shift, block energies and weights, comb indices and the final state.
kernels.npz: overlaps, half Green's functions, force bias and local
energies of random walkers for a real and a complex trial (n=10, o=4, G=7).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import afqmc_oracle as O  # noqa: E402
from ad_afqmc_prototype_gb300 import synth  # noqa: E402


def make_block():
    H = synth.make_workload(synth.WORKLOADS["c1_n12_o6_g48_w256"])
    W, nsteps, nblocks = 64, 10, 2
    prob = O.make_problem(H["h0"], H["h1"], H["chol"], H["mo_coeff"], 0.005)
    P = O.Params(dt=0.005, n_prop_steps=nsteps, qr_every=5)
    w0 = synth.trial_walkers(H["mo_coeff"], W)
    st = O.init_prop_state(prob, W, w0)
    rng = np.random.default_rng(1234)
    fields = rng.standard_normal((nblocks, nsteps, W, H["chol"].shape[0]))
    zetas = rng.random(nblocks)
    out = {"fields": fields, "zetas": zetas, "e_estimate": st.e_estimate, "init_overlaps": st.overlaps}
    # the first step alone
    s1 = O.afqmc_step(prob, P, st, fields[0, 0])
    out.update(step1_walkers=s1.walkers, step1_weights=s1.weights, step1_overlaps=s1.overlaps,
               step1_pop_shift=s1.pop_control_ene_shift)
    energies, weights, idxs = [], [], []
    for b in range(nblocks):
        st, obs, idx = O.afqmc_block(prob, P, st, fields[b], zetas[b])
        energies.append(obs["energy"])
        weights.append(obs["weight"])
        idxs.append(idx)
    out.update(block_energy=np.array(energies), block_weight=np.array(weights), sr_idx=np.array(idxs),
               final_walkers=st.walkers, final_weights=st.weights, final_overlaps=st.overlaps,
               final_pop_shift=st.pop_control_ene_shift)
    np.savez_compressed(os.path.join(HERE, "c1_block.npz"), **out)


def make_kernels():
    rng = np.random.default_rng(99)
    n, o, g, W = 10, 4, 7, 8
    a = rng.normal(size=(n, n))
    h1 = 0.5 * (a + a.T)
    b = rng.normal(size=(g, n, n))
    chol = 0.2 * (b + np.swapaxes(b, 1, 2))
    h0 = 0.37
    out = {"h1": h1, "chol": chol, "h0": h0}
    walkers = rng.normal(size=(W, n, o)) + 1j * rng.normal(size=(W, n, o))
    out["walkers"] = walkers
    for tag, cplx in (("real", False), ("cplx", True)):
        m = rng.normal(size=(n, o)) + (1j * rng.normal(size=(n, o)) if cplx else 0)
        c = np.linalg.qr(m)[0]
        ctx = O.build_meas_ctx(h1, chol, c)
        pctx = O.build_prop_ctx(h0, h1, chol, O.get_rdm1(c), 0.01)
        out[f"{tag}_mo"] = c
        out[f"{tag}_overlap"] = O.overlap_r(walkers, c)
        out[f"{tag}_green"] = O.half_green(walkers, c)
        out[f"{tag}_fb"] = O.force_bias_r(walkers, ctx, c)
        out[f"{tag}_energy"] = O.energy_r(walkers, h0, ctx, c)
        out[f"{tag}_rot_chol"] = ctx.rot_chol
        out[f"{tag}_exp_h1_half"] = pctx.exp_h1_half
        out[f"{tag}_mf"] = pctx.mf_shifts
        out[f"{tag}_h0_prop"] = pctx.h0_prop
    np.savez_compressed(os.path.join(HERE, "kernels.npz"), **out)


if __name__ == "__main__":
    make_block()
    make_kernels()
    print("wrote", os.listdir(HERE))
