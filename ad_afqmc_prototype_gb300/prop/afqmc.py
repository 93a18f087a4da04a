"""Propagation step (prop/afqmc.py:17-147 of the reference).

``afqmc_step`` keeps the reference's keyword-only signature.  When the ops
are this package's RHF/Cholesky ops it runs the fused CUDA step (one C-ABI
call, ``afq_step``); with other ops (user callables, as in the reference's
tests) it composes the same CUDA pieces around them: field draw, force bias,
field shifts, propagation, overlaps and the weight update.  The input state
is never modified: the result lives in new tensors (``inplace=True`` skips
the copies for callers that discard the old state)."""
from __future__ import annotations

from typing import Any, Optional

import torch

from .. import engine, _lib
from .. import walkers as wk
from ..core.ops import k_energy, k_force_bias, meas_ops
from ..core.system import system
from ..ham.chol import ham_chol
from ..meas.rhf import energy_kernel_r, energy_kernel_u, force_bias_kernel_r, force_bias_kernel_u, rhf_meas_ctx
from ..trial.rhf import overlap_r, overlap_u, rhf_trial
from .chol_afqmc_ops import chol_afqmc_ctx, chol_afqmc_ops
from .types import PRNGKey, afqmc_params, prop_state, split

_PREC = {"fp64": _lib.AFQ_PREC_FP64, "mixed": _lib.AFQ_PREC_MIXED, "mixed_fast": _lib.AFQ_PREC_MIXED_FAST}


def init_prop_state(*, sys: system, n_walkers: int, seed: int, ham_data: ham_chol, trial_ops_,
                    trial_data: Any, meas_ops: meas_ops, initial_walkers: Any | None = None,
                    initial_e_estimate: Any | None = None) -> prop_state:
    """Walkers, unit weights, overlaps and the unweighted mean energy
    (prop/afqmc.py:17-71)."""
    key = PRNGKey(seed)
    weights = torch.ones((n_walkers,), dtype=engine.F64, device=engine.device())
    if initial_walkers is None:
        initial_walkers = wk.init_walkers(sys=sys, rdm1=trial_ops_.get_rdm1(trial_data), n_walkers=n_walkers)
    if isinstance(initial_walkers, (tuple, list)):
        walkers = engine.pair_views(engine.as_pair(initial_walkers))
    else:
        walkers = engine.as_device(initial_walkers, engine.C128)
    overlaps = wk.apply_chunked(walkers, trial_ops_.overlap, 1, trial_data=trial_data)
    if initial_e_estimate is not None:
        e_est = engine.as_device(torch.as_tensor(initial_e_estimate).reshape(()), engine.F64)
    else:
        meas_ctx = meas_ops.build_meas_ctx(ham_data, trial_data)
        e_kernel = meas_ops.require_kernel(k_energy)
        e = wk.apply_chunked(walkers, e_kernel, 1, ham_data=ham_data, meas_ctx=meas_ctx, trial_data=trial_data)
        e_est = torch.real(e).to(engine.F64).mean()
    return prop_state(walkers=walkers, weights=weights, overlaps=overlaps.to(engine.C128), rng_key=key,
                      pop_control_ene_shift=e_est.clone(), e_estimate=e_est)


_KIND_OPS = {"restricted": (overlap_r, force_bias_kernel_r, energy_kernel_r),
             "unrestricted": (overlap_u, force_bias_kernel_u, energy_kernel_u)}


def engine_problem(*, params, ham_data, trial_data, meas_ops, prop_ops, prop_ctx, meas_ctx, n_walkers: int,
                   need_energy: bool = False, walker_kind: str = "restricted") -> Optional[engine.Problem]:
    """The fused-engine view of the arguments, or None when any op is not
    one of this package's RHF/Cholesky ops for `walker_kind`."""
    if not isinstance(trial_data, rhf_trial) or not isinstance(meas_ctx, rhf_meas_ctx):
        return None
    if not isinstance(prop_ctx, chol_afqmc_ctx) or not isinstance(ham_data, ham_chol):
        return None
    ov, fb, en = _KIND_OPS[walker_kind]
    if meas_ops.overlap is not ov or meas_ops.kernels.get(k_force_bias) is not fb:
        return None
    if need_energy and meas_ops.kernels.get(k_energy) is not en:
        return None
    if getattr(prop_ops.apply_trotter, "ham_data", None) is not ham_data:
        return None
    prec = _PREC.get(str(getattr(params, "precision", "fp64")).lower())
    if prec is None:
        raise ValueError(f"unknown precision {params.precision!r}; expected 'fp64', 'mixed' or 'mixed_fast'")
    if walker_kind == "unrestricted" and prec != _lib.AFQ_PREC_FP64:
        raise ValueError("unrestricted walkers run the binary64 form (precision='fp64')")
    lowp = None
    if prec != _lib.AFQ_PREC_FP64:
        # cached on the measurement context: it depends on chol, rot_chol and the precision only
        cached = getattr(meas_ctx, "_lowp", None)
        if cached is None or cached[0] is not ham_data.chol or cached[1] < n_walkers or cached[3] != prec:
            buf = engine.prepare_lowp(n_walkers, trial_data.norb, trial_data.nocc, int(ham_data.chol.shape[0]),
                                      ham_data.chol, meas_ctx.rot_chol, prec)
            cached = (ham_data.chol, n_walkers, buf, prec)
            object.__setattr__(meas_ctx, "_lowp", cached)
        lowp = cached[2]
    return engine.Problem(
        n_walkers=n_walkers, norb=trial_data.norb, nocc=trial_data.nocc, nchol=int(ham_data.chol.shape[0]),
        trial_is_real=trial_data.is_real, h0=ham_data.h0, chol=ham_data.chol, mo=trial_data.mo_coeff,
        dt=float(prop_ctx.dt), sqrt_dt=float(prop_ctx.sqrt_dt), exp_h1_half=prop_ctx.exp_h1_half,
        mf_shifts=prop_ctx.mf_shifts, h0_prop=complex(prop_ctx.h0_prop.item()), rot_h1=meas_ctx.rot_h1,
        rot_chol=meas_ctx.rot_chol, precision=prec, lowp=lowp)


def device_state(state: prop_state, inplace: bool) -> engine.DeviceState:
    def own(t, dtype):
        t = engine.as_device(t, dtype)
        return t if inplace else t.clone()
    if wk.is_unrestricted(state.walkers):
        p = engine.as_pair(state.walkers)
        walk = p if inplace else p.clone()
    else:
        walk = own(state.walkers, engine.C128)
    return engine.DeviceState(walkers=walk, weights=own(state.weights, engine.F64),
                              overlaps=own(state.overlaps, engine.C128),
                              pop_shift=own(torch.as_tensor(state.pop_control_ene_shift).reshape(1), engine.F64),
                              e_estimate=engine.as_device(torch.as_tensor(state.e_estimate).reshape(1), engine.F64))


def afqmc_step(state: prop_state, *, params: afqmc_params, ham_data: ham_chol, trial_data: Any,
               meas_ops: meas_ops, prop_ops: chol_afqmc_ops, prop_ctx: chol_afqmc_ctx, meas_ctx: Any,
               fields: Any = None, inplace: bool = False) -> prop_state:
    """One phaseless step (prop/afqmc.py:74-147).  ``fields`` (W, G) float64
    may be injected; otherwise they are drawn from state.rng_key."""
    key, subkey = split(state.rng_key)
    seed, counter = int(subkey[0]), int(subkey[1])
    nw = wk.n_walkers(state.walkers)
    if wk.is_unrestricted(state.walkers):
        prob = engine_problem(params=params, ham_data=ham_data, trial_data=trial_data, meas_ops=meas_ops,
                              prop_ops=prop_ops, prop_ctx=prop_ctx, meas_ctx=meas_ctx, n_walkers=nw,
                              walker_kind="unrestricted")
        if prob is None:
            raise ValueError("unrestricted walkers run with this package's RHF/Cholesky ops only")
        st = device_state(state, inplace)
        engine.step_u(prob, params, st, seed, counter, fields=fields)
        return prop_state(walkers=engine.pair_views(st.walkers), weights=st.weights, overlaps=st.overlaps,
                          rng_key=key, pop_control_ene_shift=st.pop_shift.reshape(()),
                          e_estimate=st.e_estimate.reshape(()))
    prob = engine_problem(params=params, ham_data=ham_data, trial_data=trial_data, meas_ops=meas_ops,
                          prop_ops=prop_ops, prop_ctx=prop_ctx, meas_ctx=meas_ctx, n_walkers=nw)
    if prob is not None:
        st = device_state(state, inplace)
        engine.step(prob, params, st, seed, counter, fields=fields)
    else:
        if fields is None:
            fields = engine.fill_normal((nw, prop_ops.n_fields()), seed, counter)
        fields = engine.as_device(fields, engine.F64)
        fb_kernel = meas_ops.require_kernel(k_force_bias)
        force_bias = wk.apply_chunked(state.walkers, fb_kernel, params.n_chunks, ham_data, meas_ctx, trial_data)
        xs, shift_term, fb_term = engine.field_shift(fields, force_bias, prop_ctx.mf_shifts,
                                                     float(prop_ctx.sqrt_dt))
        walkers_new = wk.apply_chunked_prop(state.walkers, xs, prop_ops.apply_trotter, params.n_chunks, prop_ctx,
                                            params.n_exp_terms)
        overlaps_new = engine.as_device(
            wk.apply_chunked(walkers_new, meas_ops.overlap, params.n_chunks, trial_data), engine.C128)
        st = device_state(state, inplace=False)
        st.walkers = engine.as_device(walkers_new, engine.C128)
        nf = prop_ops.n_fields()
        lite = engine.Problem(n_walkers=nw, norb=st.walkers.shape[1], nocc=st.walkers.shape[2], nchol=nf,
                              trial_is_real=True, h0=0.0, chol=None, mo=None, dt=float(prop_ctx.dt),
                              sqrt_dt=float(prop_ctx.sqrt_dt), exp_h1_half=None, mf_shifts=None,
                              h0_prop=complex(prop_ctx.h0_prop.item()), rot_h1=None, rot_chol=None)
        engine.weight_update(lite, params, shift_term, fb_term, overlaps_new, st)
    return prop_state(walkers=st.walkers, weights=st.weights, overlaps=st.overlaps, rng_key=key,
                      pop_control_ene_shift=st.pop_shift.reshape(()), e_estimate=st.e_estimate.reshape(()))
