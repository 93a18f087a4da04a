"""CPU FP64 oracle for the phaseless-AFQMC step (restricted walkers, RHF trial).

TEST INFRASTRUCTURE ONLY.  Nothing in the product package imports this
module; it is the checker that tests, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py`` compare the CUDA engine against.

It restates, in NumPy float64/complex128, the arithmetic of the reference
package (ad_afqmc_prototype, a JAX program).  Every function cites the
reference file:line it follows.  Two deliberate interface differences:

* random numbers are INJECTED: ``fields`` (W, G) per step and the comb
  uniform ``zeta`` per reconfiguration are arguments, instead of being drawn
  from JAX's threefry stream (prop/afqmc.py:86-88, prop/blocks.py:81-82);
* the comb's prefix sum and search (walkers.py:236-239) restate the
  association order of ``jax.lax.associative_scan`` (what ``jnp.cumsum``
  lowers to on CPU/GPU) and the probe sequence of ``jnp.searchsorted``'s
  default method, so indices are compared bit-exactly.

Parity pins:
* outputs of the reference's own code: tests/golden/make_ref_golden.py runs
  the reference's hot-path modules unmodified on NumPy (a stand-in for the
  few JAX names they use; JAX itself cannot be installed here) and records
  contexts, overlaps, Green's functions, force biases, local energies, the
  Taylor action, apply_trotter, the phase-fixed QR, comb indices on dyadic
  weights, and whole afqmc_step / afqmc_block runs on injected draws (the
  12-orbital workload and the 200-orbital benchmark Hamiltonian);
  tests/test_ref_pins.py holds this oracle to them (1e-11 Ha per block);
* the reference's own known-answer tests (weights = exp(-dt) and population
  shift 0.1 with zero Hamiltonian; E_loc = h0 with zero h1/chol; force bias
  = 2 L~ vec(solve(m^T, w^T))), restated in tests/;
* first principles (Fock-space mixed estimators, exact exponentials).
The comb's association order (XLA's, restated by ``assoc_scan``) is the one
thing the NumPy run of the reference cannot show: its jnp.cumsum runs as a
sequential sum there, so comb indices are pinned on dyadic weights, whose
prefix sums are exact in every order.
"""
from __future__ import annotations

from dataclasses import dataclass, replace
from typing import Callable, Optional

import numpy as np
import scipy.linalg

# --------------------------------------------------------------------------
# trial / walkers set-up
# --------------------------------------------------------------------------


def natorbs(dm: np.ndarray, n_occ: int) -> np.ndarray:
    """Natural orbitals, descending occupation.  walkers.py:13-16."""
    dm = 0.5 * (dm + np.conj(dm.T))
    vecs = np.linalg.eigh(dm)[1][:, ::-1]
    return vecs[:, :n_occ]


def get_rdm1(mo_coeff: np.ndarray) -> np.ndarray:
    """Stacked [C C^H, C C^H].  trial/rhf.py:29-32."""
    dm = mo_coeff @ mo_coeff.conj().T
    return np.stack([dm, dm], axis=0)


def init_walkers_restricted(rdm1: np.ndarray, nocc: int, n_walkers: int) -> np.ndarray:
    """Restricted walkers from natural orbitals of the total rdm1.
    walkers.py:55-68."""
    if rdm1.ndim != 3 or rdm1.shape[0] != 2:
        raise ValueError("Expected rdm1 with shape (2, norb, norb).")
    dm_tot = rdm1[0] + rdm1[1]
    w0 = natorbs(dm_tot, nocc) + 0.0j
    return np.broadcast_to(w0, (n_walkers, *w0.shape)).copy()


# --------------------------------------------------------------------------
# propagator context  (prop/chol_afqmc_ops.py)
# --------------------------------------------------------------------------


def mf_shifts(chol: np.ndarray, rdm1: np.ndarray) -> np.ndarray:
    """mf_g = i tr(L_g dm_tot).  prop/chol_afqmc_ops.py:53-63."""
    dm = rdm1
    if dm.ndim == 3 and dm.shape[0] == 2:
        dm = dm[0] + dm[1]
    return 1.0j * np.einsum("gij,ji->g", chol, dm, optimize=True)


@dataclass
class PropCtx:
    dt: float
    sqrt_dt: float
    exp_h1_half: np.ndarray
    mf_shifts: np.ndarray
    h0_prop: complex


def build_prop_ctx(h0, h1, chol, rdm1, dt) -> PropCtx:
    """prop/chol_afqmc_ops.py:77-103 (restricted basis)."""
    sqrt_dt = np.sqrt(dt)
    mf = mf_shifts(chol, rdm1)
    h0_prop = -h0 - 0.5 * np.sum(mf**2)
    v0m = 0.5 * np.einsum("gik,gkj->ij", chol, chol, optimize=True)
    mf_r = (1.0j * mf).real
    v1m = np.einsum("g,gik->ik", mf_r, chol, optimize=True)
    h1_eff = h1 - v0m - v1m
    exp_h1_half = scipy.linalg.expm(-0.5 * dt * h1_eff)
    return PropCtx(dt=float(dt), sqrt_dt=float(sqrt_dt), exp_h1_half=exp_h1_half,
                   mf_shifts=mf, h0_prop=complex(h0_prop))


# --------------------------------------------------------------------------
# measurement context and kernels  (meas/rhf.py)
# --------------------------------------------------------------------------


@dataclass
class MeasCtx:
    rot_h1: np.ndarray        # (o, n)
    rot_chol: np.ndarray      # (G, o, n)
    rot_chol_flat: np.ndarray  # (G, o*n)


def build_meas_ctx(h1, chol, mo_coeff) -> MeasCtx:
    """meas/rhf.py:141-150."""
    cH = mo_coeff.conj().T
    rot_h1 = cH @ h1
    rot_chol = np.einsum("pi,gij->gpj", cH, chol, optimize=True)
    return MeasCtx(rot_h1=rot_h1, rot_chol=rot_chol,
                   rot_chol_flat=rot_chol.reshape(rot_chol.shape[0], -1))


def overlap_matrix(walkers, mo_coeff):
    """m = C^H W per walker (meas/rhf.py:23, trial/rhf.py:36)."""
    return np.matmul(mo_coeff.conj().T[None], walkers)


def overlap_r(walkers, mo_coeff):
    """det(C^H W)^2 per walker.  meas/rhf.py:22-24 = trial/rhf.py:35-37."""
    return np.linalg.det(overlap_matrix(walkers, mo_coeff)) ** 2


def half_green(walkers, mo_coeff):
    """G_half = solve(m^T, W^T), shape (W, o, n).  meas/rhf.py:15-19."""
    m = overlap_matrix(walkers, mo_coeff)
    return np.linalg.solve(np.swapaxes(m, 1, 2), np.swapaxes(walkers, 1, 2))


def force_bias_r(walkers, meas_ctx: MeasCtx, mo_coeff):
    """fb = 2 L~_flat vec(G_half).  meas/rhf.py:27-33."""
    g = half_green(walkers, mo_coeff)
    return 2.0 * (g.reshape(g.shape[0], -1) @ meas_ctx.rot_chol_flat.T)


def energy_r(walkers, h0, meas_ctx: MeasCtx, mo_coeff, chunk: int = 16):
    """Local energy e0 + e1 + 2 sum c^2 - exc.  meas/rhf.py:36-50."""
    out = np.empty(walkers.shape[0], dtype=np.complex128)
    for s in range(0, walkers.shape[0], chunk):
        g = half_green(walkers[s:s + chunk], mo_coeff)  # (w, o, n)
        e1 = 2.0 * np.sum(g * meas_ctx.rot_h1[None], axis=(1, 2))
        # f_g = rot_chol_g @ g^T  -> f[w,g,i,k] = sum_j rot_chol[g,i,j] g[w,k,j]
        f = np.einsum("gij,wkj->wgik", meas_ctx.rot_chol, g, optimize=True)
        c = np.einsum("wgii->wg", f)
        exc = np.einsum("wgij,wgji->w", f, f, optimize=True)
        e2 = 2.0 * np.sum(c * c, axis=1) - exc
        out[s:s + chunk] = h0 + e1 + e2
    return out


# --------------------------------------------------------------------------
# propagation  (prop/chol_afqmc_ops.py, prop/utils.py)
# --------------------------------------------------------------------------


def make_vhs(x, chol_flat, n):
    """V_w = Re(x) L + i Im(x) L, batched.  prop/chol_afqmc_ops.py:70-74."""
    v_re = np.real(x) @ chol_flat
    v_im = np.imag(x) @ chol_flat
    return (v_re + 1.0j * v_im).reshape(-1, n, n)


def taylor_expm_action(a, mat, vecs, n_terms):
    """sum_{k<=n_terms} (a mat)^k / k! vecs.  prop/utils.py:20-31."""
    out = vecs
    term = vecs
    for k in range(1, n_terms + 1):
        term = (a / k) * np.matmul(mat, term)
        out = out + term
    return out


def apply_trotter_r(walkers, shifted_fields, ctx: PropCtx, chol_flat, n_terms):
    """E_half . exp(i sqrt(dt) V) . E_half . W.
    prop/chol_afqmc_ops.py:173-183 with :106-107 and :127-137."""
    n = walkers.shape[1]
    e = ctx.exp_h1_half
    w1 = np.matmul(e[None], walkers)
    vhs = make_vhs(shifted_fields, chol_flat, n)
    a = 1.0j * ctx.sqrt_dt
    w2 = taylor_expm_action(a, vhs, w1, n_terms)
    return np.matmul(e[None], w2)


# --------------------------------------------------------------------------
# walker population operations  (walkers.py)
# --------------------------------------------------------------------------


def qr_phase(mat):
    """Reduced QR, Q scaled so diag(R) is real and >= 0.  walkers.py:169-180.
    Returns (Q, det(R))."""
    q, r = np.linalg.qr(mat, mode="reduced")
    d = np.diagonal(r, axis1=-2, axis2=-1)
    abs_d = np.abs(d)
    phase = d / np.where(abs_d == 0, 1.0 + 0.0j, abs_d)
    q = q * np.conj(phase)[..., None, :]
    r = phase[..., :, None] * r
    det_r = np.prod(np.diagonal(r, axis1=-2, axis2=-1), axis=-1)
    return q, det_r


def orthogonalize(walkers):
    """Restricted: (Q, det(R)^2).  walkers.py:183-203."""
    q, det_r = qr_phase(walkers)
    return q, det_r * det_r


def orthonormalize(walkers):
    """walkers.py:206-211."""
    return qr_phase(walkers)[0]


def assoc_scan(x: np.ndarray) -> np.ndarray:
    """Inclusive prefix sum in the association order of
    ``jax.lax.associative_scan`` with addition, which is what ``jnp.cumsum``
    lowers to on CPU and GPU (walkers.py:236, 252).

    Recursion: e' = e[0:-1:2] + e[1::2] (pairs), s' = scan(e'); then
    s[2k+1] = s'[k], s[0] = e[0], s[2k] = s'[k-1] + e[2k] for k >= 1.
    Every add is one IEEE binary64 round-to-nearest addition, so NumPy and
    the CUDA kernel produce the same bits.  For non-negative input the
    result is non-decreasing up to an ulp (the tree is not sequential).
    """
    e = np.asarray(x, dtype=np.float64)
    n = e.shape[0]
    if n < 2:
        return e.copy()
    red = e[0:-1:2] + e[1::2]
    odd = assoc_scan(red)
    out = np.empty(n, dtype=np.float64)
    out[1::2] = odd
    out[0] = e[0]
    m = (n + 1) // 2  # number of even positions
    if m > 1:
        out[2::2] = odd[:m - 1] + e[2::2]
    return out


def searchsorted_left(cw: np.ndarray, z: np.ndarray) -> np.ndarray:
    """Binary search with the probe sequence of ``jnp.searchsorted``'s
    default method ('scan', side='left'): ceil(log2(n+1)) rounds of
    mid = (lo+hi)//2; z <= cw[mid] ? hi = mid : lo = mid; result hi.
    On a non-decreasing array this is the number of entries < z."""
    n = cw.shape[0]
    lo = np.zeros(z.shape, dtype=np.int64)
    hi = np.full(z.shape, n, dtype=np.int64)
    for _ in range(int(np.ceil(np.log2(n + 1)))):
        mid = (lo + hi) // 2
        left = z <= cw[np.minimum(mid, n - 1)]
        lo = np.where(left, lo, mid)
        hi = np.where(left, mid, hi)
    return hi


def sr_indices(weights, zeta, n_walkers, cumsum: Callable = assoc_scan):
    """Comb indices.  walkers.py:233-240.  ``cumsum`` selects the association
    order of the prefix sum (default: the reference's, see assoc_scan).
    Indices are clamped to n_walkers-1 like an out-of-range gather in the
    reference."""
    cw = cumsum(np.abs(weights))
    tot = cw[-1]
    z = tot * (np.arange(n_walkers) + zeta) / n_walkers
    idx = searchsorted_left(cw, z)
    return np.minimum(idx, n_walkers - 1), cw


def stochastic_reconfiguration(walkers, weights, zeta, cumsum: Callable = assoc_scan):
    """walkers.py:243-265 (restricted).  Returns (walkers, weights, idx)."""
    n = walkers.shape[0]
    idx, cw = sr_indices(weights, zeta, n, cumsum=cumsum)
    avg = cw[-1] / n
    weights_new = np.full((n,), avg, dtype=np.float64)
    return walkers[idx], weights_new, idx


# --------------------------------------------------------------------------
# step / block  (prop/afqmc.py, prop/blocks.py)
# --------------------------------------------------------------------------


@dataclass
class Params:
    """prop/types.py:19-32, plus ``qr_every`` (an extra orthonormalisation
    inside a block after every qr_every steps; 0 = only at block end)."""
    dt: float = 0.005
    n_chunks: int = 1
    n_exp_terms: int = 6
    pop_control_damping: float = 0.1
    weight_floor: float = 1.0e-3
    weight_cap: float = 100.0
    n_prop_steps: int = 50
    shift_ema: float = 0.1
    n_eql_blocks: int = 50
    n_blocks: int = 500
    n_walkers: int = 200
    seed: int = 42
    qr_every: int = 0


@dataclass
class State:
    """prop/types.py:10-16 without the rng key (randomness is injected)."""
    walkers: np.ndarray
    weights: np.ndarray
    overlaps: np.ndarray
    pop_control_ene_shift: float
    e_estimate: float


@dataclass
class Problem:
    h0: float
    h1: np.ndarray
    chol: np.ndarray
    mo_coeff: np.ndarray
    prop_ctx: PropCtx
    meas_ctx: MeasCtx

    @property
    def chol_flat(self):
        return self.chol.reshape(self.chol.shape[0], -1)


def make_problem(h0, h1, chol, mo_coeff, dt) -> Problem:
    rdm1 = get_rdm1(mo_coeff)
    return Problem(h0=float(h0), h1=h1, chol=chol, mo_coeff=mo_coeff,
                   prop_ctx=build_prop_ctx(h0, h1, chol, rdm1, dt),
                   meas_ctx=build_meas_ctx(h1, chol, mo_coeff))


def init_prop_state(prob: Problem, n_walkers: int,
                    initial_walkers: Optional[np.ndarray] = None) -> State:
    """prop/afqmc.py:17-71 (e_estimate = unweighted mean of Re E_loc)."""
    if initial_walkers is None:
        initial_walkers = init_walkers_restricted(
            get_rdm1(prob.mo_coeff), prob.mo_coeff.shape[1], n_walkers)
    w = np.asarray(initial_walkers, dtype=np.complex128)
    ov = overlap_r(w, prob.mo_coeff)
    e = np.real(energy_r(w, prob.h0, prob.meas_ctx, prob.mo_coeff))
    e_est = float(np.mean(e))
    return State(walkers=w, weights=np.ones(w.shape[0]), overlaps=ov,
                 pop_control_ene_shift=e_est, e_estimate=e_est)


def step_weights(prob: Problem, params: Params, state: State, fields,
                 force_bias, overlaps_new):
    """The weight-update arithmetic of prop/afqmc.py:97-101,116-138."""
    ctx = prob.prop_ctx
    field_shifts = -ctx.sqrt_dt * (1.0j * force_bias - ctx.mf_shifts)
    shifted = fields - field_shifts
    shift_term = np.sum(shifted * ctx.mf_shifts, axis=1)
    fb_term = np.sum(fields * field_shifts - 0.5 * field_shifts * field_shifts, axis=1)
    ratio = overlaps_new / state.overlaps
    exponent = (-ctx.sqrt_dt * shift_term + fb_term
                + ctx.dt * (state.pop_control_ene_shift + ctx.h0_prop))
    imp_fun = np.exp(exponent) * ratio
    theta = np.angle(np.exp(-ctx.sqrt_dt * shift_term) * ratio)
    imp_ph = np.abs(imp_fun) * np.cos(theta)
    imp_ph = np.where(imp_ph < params.weight_floor, 0.0, imp_ph)
    imp_ph = np.where(imp_ph > params.weight_cap, 0.0, imp_ph)
    weights_new = state.weights * imp_ph
    weights_new = np.where(weights_new > params.weight_cap, 0.0, weights_new)
    avg_w = np.clip(np.mean(weights_new), 1.0e-300, None)
    pop_shift_new = state.e_estimate - params.pop_control_damping * (np.log(avg_w) / ctx.dt)
    return shifted, weights_new, float(pop_shift_new)


def afqmc_step(prob: Problem, params: Params, state: State, fields,
               force_bias_fn: Optional[Callable] = None,
               overlap_fn: Optional[Callable] = None) -> State:
    """prop/afqmc.py:74-147 with injected fields (W, G) float64.
    ``force_bias_fn(walkers)`` / ``overlap_fn(walkers)`` replace the RHF
    kernels, like the fake meas/trial ops of the reference's tests."""
    fields = np.asarray(fields, dtype=np.float64)
    if force_bias_fn is None:
        fb = force_bias_r(state.walkers, prob.meas_ctx, prob.mo_coeff)
    else:
        fb = force_bias_fn(state.walkers)
    ctx = prob.prop_ctx
    field_shifts = -ctx.sqrt_dt * (1.0j * fb - ctx.mf_shifts)
    shifted = fields - field_shifts
    walkers_new = apply_trotter_r(state.walkers, shifted, ctx, prob.chol_flat,
                                  params.n_exp_terms)
    if overlap_fn is None:
        overlaps_new = overlap_r(walkers_new, prob.mo_coeff)
    else:
        overlaps_new = overlap_fn(walkers_new)
    _, weights_new, pop_new = step_weights(prob, params, state, fields, fb, overlaps_new)
    return State(walkers=walkers_new, weights=weights_new, overlaps=overlaps_new,
                 pop_control_ene_shift=pop_new, e_estimate=state.e_estimate)


def block_energy(prob: Problem, params: Params, state: State):
    """Mixed energy with clipping and weighted mean.  prop/blocks.py:59-73."""
    e = np.real(energy_r(state.walkers, prob.h0, prob.meas_ctx, prob.mo_coeff))
    thresh = np.sqrt(2.0 / params.dt)
    e_ref = state.e_estimate
    e = np.where(np.abs(e - e_ref) > thresh, e_ref, e)
    w_sum = np.sum(state.weights)
    w_sum_safe = 1.0 if w_sum == 0 else w_sum
    e_block = np.sum(state.weights * e) / w_sum_safe
    if w_sum == 0:
        e_block = e_ref
    return float(e_block), float(w_sum), e


def afqmc_block(prob: Problem, params: Params, state: State, fields_steps, zeta,
                cumsum: Callable = assoc_scan):
    """prop/blocks.py:22-95 with injected fields (n_prop_steps, W, G) and comb
    uniform ``zeta``.  With params.qr_every > 0 an extra orthonormalisation
    (and overlap refresh, as at prop/blocks.py:53-57) follows every
    qr_every-th step that is not the last one.
    Returns (state, {"energy", "weight"}, sr_indices)."""
    for s in range(params.n_prop_steps):
        state = afqmc_step(prob, params, state, fields_steps[s])
        if params.qr_every and (s + 1) % params.qr_every == 0 and s + 1 < params.n_prop_steps:
            w = orthonormalize(state.walkers)
            state = replace(state, walkers=w, overlaps=overlap_r(w, prob.mo_coeff))
    w = orthonormalize(state.walkers)
    state = replace(state, walkers=w, overlaps=overlap_r(w, prob.mo_coeff))
    e_block, w_sum, _ = block_energy(prob, params, state)
    alpha = params.shift_ema
    state = replace(state, pop_control_ene_shift=(1.0 - alpha) * state.pop_control_ene_shift
                    + alpha * e_block)
    w_sr, weights_sr, idx = stochastic_reconfiguration(state.walkers, state.weights, zeta,
                                                       cumsum=cumsum)
    state = replace(state, walkers=w_sr, weights=weights_sr,
                    overlaps=overlap_r(w_sr, prob.mo_coeff))
    return state, {"energy": e_block, "weight": w_sum}, idx
