"""CPU FP64 oracle of the differentiated energy: the run of blocks with a
one-body perturbation h1 + lam D, recorded on a tape, and its reverse-mode
adjoint, which gives dL/dh1 (and dL/dlam = <dL/dh1, D>) for any loss L of
the block energies and block weights.

TEST INFRASTRUCTURE ONLY: the checker for the engine's adjoint kernels.

The reference ships no gradient of the energy.  The derivative computed here
is the one ``jax.grad`` of a wrapper around the reference's ``afqmc_block``
(prop/blocks.py:22-95) with respect to lam would give on the same fields:
the pathwise derivative with every discrete choice held at its value -- the
comb's indices (walkers.py:233-265, integer outputs of searchsorted), the
weight floor and cap (prop/afqmc.py:127-134) and the energy clip
(prop/blocks.py:59-66).  The initial state (walkers, weights, overlaps,
population shift, energy estimate) is an input and carries no derivative.

Where lam enters: E_half = expm(-dt/2 h1_eff) with h1_eff = h1 + lam D - v0
- v1 (prop/chol_afqmc_ops.py:86-94), and rot_h1 = C^H (h1 + lam D)
(meas/rhf.py:141-150).  The trial, the mean-field shifts and h0_prop do not
depend on h1.

Adjoint conventions: for a real loss L and a complex quantity z, the
adjoint is zb = dL/dRe z + i dL/dIm z; a holomorphic map z = f(u) gives
ub = conj(f'(u)) zb, a linear map z = A u gives ub = A^H zb.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Optional

import numpy as np
import scipy.linalg

from . import afqmc_oracle as O

# --------------------------------------------------------------------------
# forward pieces with their intermediates
# --------------------------------------------------------------------------


def _minv(walkers, mo):
    m = O.overlap_matrix(walkers, mo)
    return m, np.linalg.inv(m)


def green_adjoint(walkers, mo, gbar=None, kappa=None):
    """Adjoint of G_half = (W m^-1)^T and of ov = det(m)^2, m = C^H W, per
    walker: Wb = [Gb^T + C (kappa I - conj(G) Gb^T)] m^-H with kappa =
    2 conj(ov) ovb (the overlap's share).  meas/rhf.py:15-24."""
    m, mi = _minv(walkers, mo)
    nw, n, o = walkers.shape
    g = np.einsum("wba,wjb->waj", mi, walkers)  # G[a, j] = sum_b minv[b, a] W[j, b]
    if gbar is None:
        gbar = np.zeros((nw, o, n), complex)
    if kappa is None:
        kappa = np.zeros(nw, complex)
    P = kappa[:, None, None] * np.eye(o)[None] - np.einsum("waj,wbj->wab", np.conj(g), gbar)
    Z = np.swapaxes(gbar, 1, 2) + np.einsum("ic,wcb->wib", mo, P)
    return Z @ np.conj(np.swapaxes(mi, 1, 2))


def qr_adjoint(a, qbar):
    """Adjoint of the phase-fixed reduced QR (walkers.py:169-180), Q only:
    Ab = [(I - Q Q^H) Qb + Q Kb] R^-H, Kb = tril(S, -1) + diag(S)/2,
    S = Q^H Qb - Qb^H Q.  The diagonal half-weight comes from the gauge
    (diag R real positive), which makes diag(Q^H dQ) purely imaginary."""
    out = np.empty_like(a)
    for w in range(a.shape[0]):
        q, r = np.linalg.qr(a[w], mode="reduced")
        d = np.diag(r)
        ph = d / np.where(np.abs(d) == 0, 1.0, np.abs(d))
        q = q * np.conj(ph)[None, :]
        r = ph[:, None] * r
        b = q.conj().T @ qbar[w]
        s = b - b.conj().T
        kb = np.tril(s, -1) + 0.5 * np.diag(np.diag(s))
        z = qbar[w] - q @ b + q @ kb
        out[w] = scipy.linalg.solve_triangular(r, z.conj().T, lower=False).conj().T
    return out


@dataclass
class StepCache:
    walkers: np.ndarray      # pre-step
    weights: np.ndarray
    overlaps: np.ndarray
    pop_shift: float
    fields: np.ndarray
    fs: np.ndarray           # field shifts (W, G)
    xt: np.ndarray           # shifted fields
    vhs: np.ndarray          # (W, n, n)
    w1: np.ndarray
    terms: list              # t_0 .. t_K
    w2: np.ndarray
    walkers_new: np.ndarray
    overlaps_new: np.ndarray
    imp_ph: np.ndarray       # after floor / cap
    alive: np.ndarray        # imp_ph not floored/capped and w' not capped
    phi: np.ndarray
    rfac: np.ndarray
    weights_new: np.ndarray


def step_forward(prob: O.Problem, params: O.Params, st: O.State, x) -> tuple[O.State, StepCache]:
    """prop/afqmc.py:74-147, keeping what the adjoint needs."""
    ctx = prob.prop_ctx
    mo = prob.mo_coeff
    fb = O.force_bias_r(st.walkers, prob.meas_ctx, mo)
    fs = -ctx.sqrt_dt * (1.0j * fb - ctx.mf_shifts)
    xt = x - fs
    n = st.walkers.shape[1]
    E = ctx.exp_h1_half
    w1 = np.matmul(E[None], st.walkers)
    vhs = O.make_vhs(xt, prob.chol_flat, n)
    a = 1.0j * ctx.sqrt_dt
    terms = [w1]
    for k in range(1, params.n_exp_terms + 1):
        terms.append((a / k) * np.matmul(vhs, terms[-1]))
    w2 = sum(terms)
    wn = np.matmul(E[None], w2)
    ovn = O.overlap_r(wn, mo)
    shift_term = np.sum(xt * ctx.mf_shifts, axis=1)
    fb_term = np.sum(x * fs - 0.5 * fs * fs, axis=1)
    ratio = ovn / st.overlaps
    phi = np.exp(-ctx.sqrt_dt * shift_term) * ratio
    rfac = np.exp(fb_term.real + ctx.dt * (st.pop_control_ene_shift + ctx.h0_prop.real))
    # the reference's |imp| cos(theta), in its own arithmetic
    exponent = -ctx.sqrt_dt * shift_term + fb_term + ctx.dt * (st.pop_control_ene_shift + ctx.h0_prop)
    imp = np.exp(exponent) * ratio
    imp_ph = np.abs(imp) * np.cos(np.angle(phi))
    alive = ~((imp_ph < params.weight_floor) | (imp_ph > params.weight_cap))
    imp_ph = np.where(alive, imp_ph, 0.0)
    wpre = st.weights * imp_ph
    capped = wpre > params.weight_cap
    wnew = np.where(capped, 0.0, wpre)
    alive = alive & ~capped
    avg_w = np.clip(np.mean(wnew), 1.0e-300, None)
    pn = st.e_estimate - params.pop_control_damping * (np.log(avg_w) / ctx.dt)
    new = O.State(walkers=wn, weights=wnew, overlaps=ovn, pop_control_ene_shift=float(pn),
                  e_estimate=st.e_estimate)
    cache = StepCache(st.walkers, st.weights, st.overlaps, st.pop_control_ene_shift, x, fs, xt, vhs, w1, terms,
                      w2, wn, ovn, imp_ph, alive, phi, rfac, wnew)
    return new, cache


@dataclass
class Adj:
    """Adjoint of a state: walkers, weights, overlaps, population shift."""
    walkers: np.ndarray
    weights: np.ndarray
    overlaps: np.ndarray
    pop_shift: float = 0.0


@dataclass
class Accum:
    ebar: np.ndarray      # dL/dE_half (n, n) real
    sg: np.ndarray        # sum over measurements of Ebar_w G_half,w (o, n)


def step_adjoint(prob: O.Problem, params: O.Params, c: StepCache, adj: Adj, acc: Accum) -> Adj:
    ctx = prob.prop_ctx
    mo = prob.mo_coeff
    dt, sq = ctx.dt, ctx.sqrt_dt
    nw = c.walkers.shape[0]
    # population shift p' = e_est - damping log(mean w') / dt
    wbar_new = adj.weights.copy()
    if np.mean(c.weights_new) > 1.0e-300:
        wbar_new += adj.pop_shift * (-params.pop_control_damping / dt) / np.sum(c.weights_new)
    # w' = w imp_ph on live walkers
    wbar_new = np.where(c.alive, wbar_new, 0.0)
    wbar = wbar_new * c.imp_ph
    ibar = wbar_new * c.weights
    pbar = float(np.sum(ibar * dt * c.imp_ph))
    # imp_ph = rfac Re(phi): rfac = exp(Re fb_term + dt (p + h0p)), phi = exp(-sq shift) ovn / ov
    fbt_bar = ibar * c.imp_ph
    phibar = ibar * c.rfac
    shift_bar = np.conj(-sq * c.phi) * phibar
    ovn_bar = adj.overlaps + np.conj(c.phi / c.overlaps_new) * phibar
    ov_bar = np.conj(-c.phi / c.overlaps) * phibar
    fs_bar = (np.conj(c.fields - c.fs) * fbt_bar[:, None]
              + np.conj(-ctx.mf_shifts)[None, :] * shift_bar[:, None])
    # overlaps of the new walkers
    wn_bar = adj.walkers + green_adjoint(c.walkers_new, mo, kappa=2.0 * np.conj(c.overlaps_new) * ovn_bar)
    # W' = E W2, W2 = sum t_k, t_k = (a/k) V t_{k-1}, t_0 = W1 = E W
    E = ctx.exp_h1_half
    acc.ebar += np.real(np.einsum("wia,wja->ij", wn_bar, np.conj(c.w2)))
    w2_bar = np.matmul(E.T[None], wn_bar)
    a = 1.0j * sq
    K = len(c.terms) - 1
    tbar = w2_bar
    vbar = np.zeros_like(c.vhs)
    for k in range(K, 0, -1):
        # tbar is the adjoint of t_k
        vbar += np.conj(a / k) * np.matmul(tbar, np.conj(np.swapaxes(c.terms[k - 1], 1, 2)))
        tbar = w2_bar + np.conj(a / k) * np.matmul(np.conj(np.swapaxes(c.vhs, 1, 2)), tbar)
    w1_bar = tbar
    acc.ebar += np.real(np.einsum("wia,wja->ij", w1_bar, np.conj(c.walkers)))
    w_bar = np.matmul(E.T[None], w1_bar)
    # V = sum_g xt_g L_g
    xt_bar = vbar.reshape(nw, -1) @ prob.chol_flat.T
    fs_bar = fs_bar - xt_bar
    fb_bar = 1.0j * sq * fs_bar
    # fb = 2 L~ vec(G_half)
    gbar = (2.0 * fb_bar @ np.conj(prob.meas_ctx.rot_chol_flat)).reshape(c.walkers.shape[0], *prob.meas_ctx.rot_h1.shape)
    w_bar = w_bar + green_adjoint(c.walkers, mo, gbar=gbar)
    return Adj(walkers=w_bar, weights=wbar, overlaps=ov_bar, pop_shift=pbar)


def energy_gbar(prob: O.Problem, walkers, ebar_w):
    """Adjoint of Re E_loc (meas/rhf.py:36-50) with respect to G_half:
    Gb = Eb conj(2 rot_h1 + 4 sum_g c_g L~_g - 2 sum_g f_g L~_g)."""
    mc = prob.meas_ctx
    g = O.half_green(walkers, prob.mo_coeff)
    f = np.einsum("gij,wkj->wgik", mc.rot_chol, g)
    c = np.einsum("wgii->wg", f)
    d = (2.0 * mc.rot_h1[None] + 4.0 * np.einsum("wg,gij->wij", c, mc.rot_chol)
         - 2.0 * np.einsum("wgpq,gqj->wpj", f, mc.rot_chol))
    return ebar_w[:, None, None] * np.conj(d), g


# --------------------------------------------------------------------------
# the run of blocks
# --------------------------------------------------------------------------


@dataclass
class BlockTape:
    steps: list = field(default_factory=list)   # ('step', StepCache) / ('qr', pre walkers, post walkers)
    qr_pre: Optional[np.ndarray] = None
    measured: Optional[O.State] = None          # state after the block-end QR and overlap refresh
    energies: Optional[np.ndarray] = None       # clipped local energies
    unclipped: Optional[np.ndarray] = None
    e_block: float = 0.0
    w_sum: float = 0.0
    idx: Optional[np.ndarray] = None


def block_forward(prob, params, st: O.State, fields_steps, zeta, sr_idx=None):
    """prop/blocks.py:22-95 as afqmc_oracle.afqmc_block, recording a tape.
    sr_idx: comb indices to use instead of the comb's own (fixed-comb
    finite differences)."""
    tape = BlockTape()
    for s in range(params.n_prop_steps):
        st, c = step_forward(prob, params, st, fields_steps[s])
        tape.steps.append(("step", c))
        if params.qr_every and (s + 1) % params.qr_every == 0 and s + 1 < params.n_prop_steps:
            w = O.orthonormalize(st.walkers)
            tape.steps.append(("qr", st.walkers, w))
            st = O.replace(st, walkers=w, overlaps=O.overlap_r(w, prob.mo_coeff))
    tape.qr_pre = st.walkers
    w = O.orthonormalize(st.walkers)
    st = O.replace(st, walkers=w, overlaps=O.overlap_r(w, prob.mo_coeff))
    tape.measured = st
    e_block, w_sum, e = O.block_energy(prob, params, st)
    tape.energies = e
    tape.unclipped = np.real(O.energy_r(st.walkers, prob.h0, prob.meas_ctx, prob.mo_coeff))
    tape.e_block, tape.w_sum = e_block, w_sum
    alpha = params.shift_ema
    st = O.replace(st, pop_control_ene_shift=(1.0 - alpha) * st.pop_control_ene_shift + alpha * e_block)
    if sr_idx is None:
        w_sr, weights_sr, idx = O.stochastic_reconfiguration(st.walkers, st.weights, zeta)
    else:
        idx = np.asarray(sr_idx)
        cw = O.assoc_scan(np.abs(st.weights))
        w_sr, weights_sr = st.walkers[idx], np.full(st.weights.shape, cw[-1] / st.weights.shape[0])
    tape.idx = idx
    # overlaps of the copies are the copies of the overlaps
    st = O.replace(st, walkers=w_sr, weights=weights_sr, overlaps=st.overlaps[idx])
    return st, tape


def block_adjoint(prob, params, tape: BlockTape, adj: Adj, eb_bar: float, wb_bar: float, acc: Accum) -> Adj:
    nw = adj.walkers.shape[0]
    mo = prob.mo_coeff
    ms = tape.measured
    # comb: gather of walkers and overlaps, weights = sum |w| / N
    wk = np.zeros_like(adj.walkers)
    ob = np.zeros_like(adj.overlaps)
    np.add.at(wk, tape.idx, adj.walkers)
    np.add.at(ob, tape.idx, adj.overlaps)
    wbar = np.sign(ms.weights) * np.sum(adj.weights) / nw
    # population shift EMA: p = (1 - alpha) p_prev + alpha e_block
    alpha = params.shift_ema
    pbar = (1.0 - alpha) * adj.pop_shift
    eb_bar = eb_bar + alpha * adj.pop_shift
    # block energy e_b = sum w e / sum w, weight W_b = sum w
    wsum = np.sum(ms.weights)
    wbar = wbar + wb_bar
    if wsum != 0.0:
        live = tape.energies == tape.unclipped
        ebar_w = np.where(live, eb_bar * ms.weights / wsum, 0.0)
        wbar = wbar + eb_bar * (tape.energies - tape.e_block) / wsum
        gbar, g = energy_gbar(prob, ms.walkers, ebar_w)
        acc.sg += np.einsum("w,wij->ij", ebar_w, g)
        wk = wk + green_adjoint(ms.walkers, mo, gbar=gbar)
    # block-end QR and overlap refresh
    wk = wk + green_adjoint(ms.walkers, mo, kappa=2.0 * np.conj(ms.overlaps) * ob)
    wk = qr_adjoint(tape.qr_pre, wk)
    adj = Adj(walkers=wk, weights=wbar, overlaps=np.zeros_like(ob), pop_shift=pbar)
    for item in reversed(tape.steps):
        if item[0] == "step":
            adj = step_adjoint(prob, params, item[1], adj, acc)
        else:
            _, pre, post = item
            wk = adj.walkers + green_adjoint(post, mo, kappa=2.0 * np.conj(O.overlap_r(post, mo)) * adj.overlaps)
            adj = Adj(walkers=qr_adjoint(pre, wk), weights=adj.weights, overlaps=np.zeros_like(adj.overlaps),
                      pop_shift=adj.pop_shift)
    return adj


def run_forward(prob, params, st: O.State, fields_blocks, zetas, sr_fixed=None):
    """Blocks b = 0..B-1 with fields_blocks[b] (n_prop_steps, W, G) and comb
    uniforms zetas[b].  Returns (energies (B,), weights (B,), tapes)."""
    tapes, es, ws = [], [], []
    for b in range(len(fields_blocks)):
        st, t = block_forward(prob, params, st, fields_blocks[b], zetas[b],
                              None if sr_fixed is None else sr_fixed[b])
        tapes.append(t)
        es.append(t.e_block)
        ws.append(t.w_sum)
    return np.array(es), np.array(ws), tapes


def frechet_adjoint(h1_eff, dt, ebar):
    """dL/dh1_eff from dL/dE_half, E_half = expm(s h1_eff), s = -dt/2:
    s L_exp(s h1_eff^T, Ebar) (the adjoint of the Frechet derivative)."""
    s = -0.5 * dt
    return s * scipy.linalg.expm_frechet(s * h1_eff.T, ebar, compute_expm=False)


def h1_eff_of(prob: O.Problem):
    ctx = prob.prop_ctx
    v0m = 0.5 * np.einsum("gik,gkj->ij", prob.chol, prob.chol)
    v1m = np.einsum("g,gik->ik", (1.0j * ctx.mf_shifts).real, prob.chol)
    return prob.h1 - v0m - v1m


def run_backward(prob, params, tapes, eb_bar, wb_bar, n_walkers):
    """dL/dh1 (n, n) for the loss whose adjoints with respect to the block
    energies and weights are eb_bar, wb_bar."""
    n = prob.h1.shape[0]
    o = prob.mo_coeff.shape[1]
    acc = Accum(ebar=np.zeros((n, n)), sg=np.zeros((o, n), complex))
    adj = Adj(walkers=np.zeros((n_walkers, n, o), complex), weights=np.zeros(n_walkers),
              overlaps=np.zeros(n_walkers, complex), pop_shift=0.0)
    for b in range(len(tapes) - 1, -1, -1):
        adj = block_adjoint(prob, params, tapes[b], adj, float(eb_bar[b]), float(wb_bar[b]), acc)
    h1bar = frechet_adjoint(h1_eff_of(prob), params.dt, acc.ebar)
    # rot_h1 = C^H h1: E = Re(2 sum G_half o rot_h1) + ...
    h1bar = h1bar + 2.0 * np.real(np.conj(prob.mo_coeff) @ acc.sg)
    return h1bar, acc


def mixed_energy(es, ws):
    """The loss of the differentiated-energy checks: sum_b W_b e_b / sum_b W_b."""
    return float(np.sum(ws * es) / np.sum(ws))


def mixed_energy_bar(es, ws):
    tot = np.sum(ws)
    mu = np.sum(ws * es) / tot
    return ws / tot, (es - mu) / tot
