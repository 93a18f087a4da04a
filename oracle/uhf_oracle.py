"""CPU FP64 oracle for unrestricted and generalized walkers with the RHF
trial (walker_kind "unrestricted", "generalized").  TEST INFRASTRUCTURE
ONLY: the checker for the engine's afq_*_u and afq_*_g entry points.

Restates meas/rhf.py:53-100 (overlap_u, force_bias_kernel_u,
energy_kernel_u), prop/chol_afqmc_ops.py:118-183 (the unrestricted Trotter
step: the same V on both spins), walkers.py:183-265 (QR per spin, one set of
comb indices for both spins) and the step/block of prop/afqmc.py:74-147 and
prop/blocks.py:22-95 with a pair of walkers.  Fields and the comb uniform
are injected, as in afqmc_oracle.
"""
from __future__ import annotations

from dataclasses import dataclass, replace

import numpy as np

from . import afqmc_oracle as O


def _det(m):
    return np.linalg.det(m)


def overlap_u(wu, wd, mo):
    """det(C^H W_up) det(C^H W_dn).  meas/rhf.py:53-57."""
    return _det(O.overlap_matrix(wu, mo)) * _det(O.overlap_matrix(wd, mo))


def force_bias_u(wu, wd, meas_ctx: O.MeasCtx, mo):
    """L~_flat vec(G_up + G_dn).  meas/rhf.py:60-72."""
    g = O.half_green(wu, mo) + O.half_green(wd, mo)
    return g.reshape(g.shape[0], -1) @ meas_ctx.rot_chol_flat.T


def energy_u(wu, wd, h0, meas_ctx: O.MeasCtx, mo):
    """meas/rhf.py:75-100."""
    gu = O.half_green(wu, mo)
    gd = O.half_green(wd, mo)
    e1 = np.sum((gu + gd) * meas_ctx.rot_h1[None], axis=(1, 2))
    fu = np.einsum("gij,wkj->wgik", meas_ctx.rot_chol, gu, optimize=True)
    fd = np.einsum("gij,wkj->wgik", meas_ctx.rot_chol, gd, optimize=True)
    cu = np.einsum("wgii->wg", fu)
    cd = np.einsum("wgii->wg", fd)
    xu = np.einsum("wgij,wgji->w", fu, fu, optimize=True)
    xd = np.einsum("wgij,wgji->w", fd, fd, optimize=True)
    e2 = (np.sum(cu * cu, 1) + np.sum(cd * cd, 1) + 2.0 * np.sum(cu * cd, 1) - xu - xd) / 2.0
    return h0 + e1 + e2


def apply_trotter_u(wu, wd, shifted, ctx: O.PropCtx, chol_flat, n_terms):
    """prop/chol_afqmc_ops.py:118-183 (unrestricted): both spins with the same V."""
    return (O.apply_trotter_r(wu, shifted, ctx, chol_flat, n_terms),
            O.apply_trotter_r(wd, shifted, ctx, chol_flat, n_terms))


def init_walkers_u(mo, n_walkers):
    """walkers.py:69-75 with the RHF trial's rdm1 [C C^H, C C^H]."""
    dm = mo @ mo.conj().T
    w0 = O.natorbs(dm, mo.shape[1]) + 0.0j
    w = np.broadcast_to(w0, (n_walkers, *w0.shape)).copy()
    return w, w.copy()


@dataclass
class StateU:
    wu: np.ndarray
    wd: np.ndarray
    weights: np.ndarray
    overlaps: np.ndarray
    pop_control_ene_shift: float
    e_estimate: float


def init_state_u(prob: O.Problem, wu, wd) -> StateU:
    ov = overlap_u(wu, wd, prob.mo_coeff)
    e = float(np.mean(np.real(energy_u(wu, wd, prob.h0, prob.meas_ctx, prob.mo_coeff))))
    return StateU(wu=wu, wd=wd, weights=np.ones(wu.shape[0]), overlaps=ov, pop_control_ene_shift=e,
                  e_estimate=e)


def step_u(prob: O.Problem, params: O.Params, st: StateU, fields) -> StateU:
    """prop/afqmc.py:74-147 with unrestricted walkers."""
    fb = force_bias_u(st.wu, st.wd, prob.meas_ctx, prob.mo_coeff)
    ctx = prob.prop_ctx
    fs = -ctx.sqrt_dt * (1.0j * fb - ctx.mf_shifts)
    shifted = fields - fs
    wu, wd = apply_trotter_u(st.wu, st.wd, shifted, ctx, prob.chol_flat, params.n_exp_terms)
    ov_new = overlap_u(wu, wd, prob.mo_coeff)
    rst = O.State(walkers=st.wu, weights=st.weights, overlaps=st.overlaps,
                  pop_control_ene_shift=st.pop_control_ene_shift, e_estimate=st.e_estimate)
    _, w_new, pop = O.step_weights(prob, params, rst, fields, fb, ov_new)
    return StateU(wu=wu, wd=wd, weights=w_new, overlaps=ov_new, pop_control_ene_shift=pop,
                  e_estimate=st.e_estimate)


def orthonormalize_u(prob, st: StateU) -> StateU:
    wu, wd = O.orthonormalize(st.wu), O.orthonormalize(st.wd)
    return replace(st, wu=wu, wd=wd, overlaps=overlap_u(wu, wd, prob.mo_coeff))


def block_u(prob: O.Problem, params: O.Params, st: StateU, fields_steps, zeta):
    """prop/blocks.py:22-95 with unrestricted walkers.  Returns (state,
    {"energy", "weight"}, comb indices)."""
    for s in range(params.n_prop_steps):
        st = step_u(prob, params, st, fields_steps[s])
        if params.qr_every and (s + 1) % params.qr_every == 0 and s + 1 < params.n_prop_steps:
            st = orthonormalize_u(prob, st)
    st = orthonormalize_u(prob, st)
    e = np.real(energy_u(st.wu, st.wd, prob.h0, prob.meas_ctx, prob.mo_coeff))
    thresh = np.sqrt(2.0 / params.dt)
    e = np.where(np.abs(e - st.e_estimate) > thresh, st.e_estimate, e)
    wsum = np.sum(st.weights)
    e_block = np.sum(st.weights * e) / (1.0 if wsum == 0 else wsum)
    if wsum == 0:
        e_block = st.e_estimate
    alpha = params.shift_ema
    st = replace(st, pop_control_ene_shift=(1.0 - alpha) * st.pop_control_ene_shift + alpha * e_block)
    idx, cw = O.sr_indices(st.weights, zeta, st.wu.shape[0])
    st = replace(st, wu=st.wu[idx], wd=st.wd[idx], weights=np.full(st.weights.shape, cw[-1] / st.weights.shape[0]),
                 overlaps=st.overlaps[idx])
    return st, {"energy": float(e_block), "weight": float(wsum)}, idx


# --------------------------------------------------------------------------
# generalized walkers (W, 2n, 2o) with the RHF trial: meas/rhf.py:103-130,
# prop/chol_afqmc_ops.py:141-197 (the reference has no generalized energy)
# --------------------------------------------------------------------------


def _m_g(w, mo):
    n = mo.shape[0]
    cH = mo.conj().T
    return np.concatenate([cH[None] @ w[:, :n, :], cH[None] @ w[:, n:, :]], axis=1)


def overlap_g(w, mo):
    """det(vstack(C^H W_top, C^H W_bot)).  meas/rhf.py:103-109."""
    return np.linalg.det(_m_g(w, mo))


def force_bias_g(w, meas_ctx: O.MeasCtx, mo):
    """L~_flat vec(G_up + G_dn) of G_half = solve(m^T, W^T).  meas/rhf.py:112-130."""
    n, o = mo.shape
    g = np.linalg.solve(np.swapaxes(_m_g(w, mo), 1, 2), np.swapaxes(w, 1, 2))  # (W, 2o, 2n)
    gs = g[:, :o, :n] + g[:, o:, n:]
    return gs.reshape(gs.shape[0], -1) @ meas_ctx.rot_chol_flat.T


def apply_trotter_g(w, shifted, ctx: O.PropCtx, chol_flat, n_terms):
    """Both halves with the walker's V (prop/chol_afqmc_ops.py:141-197)."""
    n = ctx.exp_h1_half.shape[0]
    top = O.apply_trotter_r(w[:, :n, :], shifted, ctx, chol_flat, n_terms)
    bot = O.apply_trotter_r(w[:, n:, :], shifted, ctx, chol_flat, n_terms)
    return np.concatenate([top, bot], axis=1)


def step_g(prob: O.Problem, params: O.Params, st: O.State, fields) -> O.State:
    """prop/afqmc.py:74-147 with generalized walkers in st.walkers."""
    fb = force_bias_g(st.walkers, prob.meas_ctx, prob.mo_coeff)
    ctx = prob.prop_ctx
    fs = -ctx.sqrt_dt * (1.0j * fb - ctx.mf_shifts)
    w = apply_trotter_g(st.walkers, fields - fs, ctx, prob.chol_flat, params.n_exp_terms)
    ov_new = overlap_g(w, prob.mo_coeff)
    _, w_new, pop = O.step_weights(prob, params, st, fields, fb, ov_new)
    return O.State(walkers=w, weights=w_new, overlaps=ov_new, pop_control_ene_shift=pop, e_estimate=st.e_estimate)
