"""Propagation block (prop/blocks.py:18-95 of the reference): n_prop_steps
steps, QR, mixed energy, shift update and comb reconfiguration.  With this
package's RHF/Cholesky ops the whole block is one C-ABI call (``afq_block``)."""
from __future__ import annotations

from typing import Any, NamedTuple

import torch

from .. import engine
from .. import walkers as wk
from ..core.ops import k_energy, meas_ops
from ..core.system import system
from ..ham.chol import ham_chol
from .afqmc import afqmc_step, device_state, engine_problem
from .chol_afqmc_ops import chol_afqmc_ctx, chol_afqmc_ops
from .types import afqmc_params, prop_state


class block_obs(NamedTuple):
    scalars: dict


def afqmc_block(state: prop_state, *, sys: system, params: afqmc_params, ham_data: ham_chol, trial_data: Any,
                meas_ops: meas_ops, prop_ops: chol_afqmc_ops, prop_ctx: chol_afqmc_ctx, meas_ctx: Any,
                fields: Any = None, zeta: Any = None, inplace: bool = False,
                cv: Any = None) -> tuple[prop_state, block_obs]:
    """propagation + measurement.  ``fields`` (n_prop_steps, W, G) and the comb
    uniform ``zeta`` may be injected; otherwise both are drawn from the key.
    ``cv`` (a ``prop.cv.ExchangeControlVariate``, mixed precisions only)
    selects the control-variate measurement of the exchange energy."""
    nw = wk.n_walkers(state.walkers)
    seed, counter = int(state.rng_key[0]), int(state.rng_key[1])
    key = torch.tensor([seed, counter + params.n_prop_steps + 1], dtype=torch.int64)
    if sys.walker_kind.lower() == "unrestricted":
        if cv is not None:
            raise ValueError("the control-variate measurement needs restricted walkers")
        prob = engine_problem(params=params, ham_data=ham_data, trial_data=trial_data, meas_ops=meas_ops,
                              prop_ops=prop_ops, prop_ctx=prop_ctx, meas_ctx=meas_ctx, n_walkers=nw,
                              need_energy=True, walker_kind="unrestricted")
        if prob is None:
            raise ValueError("unrestricted walkers run with this package's RHF/Cholesky ops only")
        st = device_state(state, inplace)
        e, wsum = engine.block_u(prob, params, st, seed, counter, fields=fields, zeta=zeta)
        new = prop_state(walkers=engine.pair_views(st.walkers), weights=st.weights, overlaps=st.overlaps,
                         rng_key=key, pop_control_ene_shift=st.pop_shift.reshape(()),
                         e_estimate=st.e_estimate.reshape(()))
        return new, block_obs(scalars={"energy": e.reshape(()), "weight": wsum.reshape(())})
    if sys.walker_kind.lower() == "restricted":
        prob = engine_problem(params=params, ham_data=ham_data, trial_data=trial_data, meas_ops=meas_ops,
                              prop_ops=prop_ops, prop_ctx=prop_ctx, meas_ctx=meas_ctx, n_walkers=nw,
                              need_energy=True)
    else:
        prob = None
    if prob is not None:
        st = device_state(state, inplace)
        cvs = cv.block_args(nw) if cv is not None else None
        e, wsum = engine.block(prob, params, st, seed, counter, fields=fields, zeta=zeta, cv=cvs)
        if cv is not None:
            cv.after_block()
        new = prop_state(walkers=st.walkers, weights=st.weights, overlaps=st.overlaps, rng_key=key,
                         pop_control_ene_shift=st.pop_shift.reshape(()), e_estimate=st.e_estimate.reshape(()))
        return new, block_obs(scalars={"energy": e.reshape(()), "weight": wsum.reshape(())})

    if cv is not None:
        raise ValueError("the control-variate measurement needs the engine's restricted RHF path")
    kw = dict(params=params, ham_data=ham_data, trial_data=trial_data, meas_ops=meas_ops, prop_ops=prop_ops,
              prop_ctx=prop_ctx, meas_ctx=meas_ctx)
    for s in range(params.n_prop_steps):
        state = afqmc_step(state, fields=None if fields is None else fields[s], **kw)
        if params.qr_every and (s + 1) % params.qr_every == 0 and s + 1 < params.n_prop_steps:
            w = wk.orthonormalize(state.walkers, sys.walker_kind)
            state = state._replace(walkers=w, overlaps=wk.apply_chunked(w, meas_ops.overlap, params.n_chunks,
                                                                         trial_data))
    w = wk.orthonormalize(state.walkers, sys.walker_kind)
    state = state._replace(walkers=w, overlaps=wk.apply_chunked(w, meas_ops.overlap, params.n_chunks, trial_data))
    e_kernel = meas_ops.require_kernel(k_energy)
    e = engine.as_device(wk.apply_chunked(state.walkers, e_kernel, params.n_chunks, ham_data, meas_ctx,
                                          trial_data), engine.C128)
    st = device_state(state, inplace=False)
    e_blk, wsum = engine.block_measure(st.weights, e, st.e_estimate, st.pop_shift, params.dt, params.shift_ema)
    if zeta is None:
        zeta = float(engine.fill_uniform((1,), seed, counter + params.n_prop_steps).item())
    w_sr, weights_sr = wk.stochastic_reconfiguration(st.walkers, st.weights, zeta, sys.walker_kind)
    overlaps_sr = wk.apply_chunked(w_sr, meas_ops.overlap, params.n_chunks, trial_data)
    new = prop_state(walkers=w_sr, weights=weights_sr, overlaps=overlaps_sr, rng_key=key,
                     pop_control_ene_shift=st.pop_shift.reshape(()), e_estimate=st.e_estimate.reshape(()))
    return new, block_obs(scalars={"energy": e_blk.reshape(()), "weight": wsum.reshape(())})
