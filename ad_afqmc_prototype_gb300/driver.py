"""Energy driver (driver.py of the reference): equilibration blocks, sampling
blocks, outlier rejection and blocking analysis, with the same signature,
progress lines and return values.

The reference compiles chunks of blocks with ``jax.lax.scan`` under
``jax.jit`` (driver.py:22-38) so that they stay on the GPU; here, when
``block_fn`` is this package's ``afqmc_block`` on the engine's restricted
RHF path, a chunk is one ``afq_run_blocks`` call: the block loop replayed as
a CUDA graph with the random stream's counter on the device (the same stream
as calling ``afqmc_block`` block by block).  Any other ``block_fn`` is called
block by block, as the reference's scan would.
"""
from __future__ import annotations

import time
from functools import partial
from typing import Any, Callable

import numpy as np
import torch

from . import engine
from .core.ops import meas_ops, trial_ops
from .core.system import system
from .ham.chol import ham_chol
from .prop.afqmc import device_state, engine_problem, init_prop_state
from .prop.blocks import afqmc_block, block_obs
from .prop.chol_afqmc_ops import make_chol_afqmc_ops
from .prop.types import afqmc_params, prop_state
from .stat_utils import blocking_analysis_ratio, reject_outliers

print = partial(print, flush=True)


def make_run_blocks(block, engine_args: dict | None = None):
    """run_blocks(state, n_blocks) -> (state, energies (n,), weights (n,)).
    engine_args (keyword arguments of afqmc_block) selects the graph-replayed
    engine loop."""

    def run_blocks(state0: prop_state, *, n_blocks: int):
        if engine_args is not None:
            kw = engine_args
            nw = int(state0.walkers.shape[0])
            prob = engine_problem(params=kw["params"], ham_data=kw["ham_data"], trial_data=kw["trial_data"],
                                  meas_ops=kw["meas_ops"], prop_ops=kw["prop_ops"], prop_ctx=kw["prop_ctx"],
                                  meas_ctx=kw["meas_ctx"], n_walkers=nw, need_energy=True)
            if prob is not None:
                params = kw["params"]
                seed, counter = int(state0.rng_key[0]), int(state0.rng_key[1])
                st = device_state(state0, inplace=False)
                ctr = torch.tensor([counter], dtype=torch.int64, device=st.walkers.device)
                e, w = engine.run_blocks(prob, params, st, n_blocks, seed, ctr)
                key = torch.tensor([seed, counter + n_blocks * (params.n_prop_steps + 1)], dtype=torch.int64)
                new = prop_state(walkers=st.walkers, weights=st.weights, overlaps=st.overlaps, rng_key=key,
                                 pop_control_ene_shift=st.pop_shift.reshape(()),
                                 e_estimate=st.e_estimate.reshape(()))
                return new, e.cpu(), w.cpu()
        es, ws = [], []
        state = state0
        for _ in range(n_blocks):
            state, obs = block(state)
            es.append(float(obs.scalars["energy"]))
            ws.append(float(obs.scalars["weight"]))
        return state, torch.tensor(es, dtype=torch.float64), torch.tensor(ws, dtype=torch.float64)

    return run_blocks


def run_afqmc_energy(*, sys: system, params: afqmc_params, ham_data: ham_chol, trial_data: Any,
                     meas_ops: meas_ops, trial_ops: trial_ops,
                     block_fn: Callable[..., tuple[prop_state, block_obs]]):
    """equilibration blocks then sampling blocks.

    Returns:
      (mean_energy, stderr, block_energies, block_weights)
    """
    prop_ops = make_chol_afqmc_ops(ham_data, sys.walker_kind)
    prop_ctx = prop_ops.build_prop_ctx(trial_ops.get_rdm1(trial_data), params.dt)
    meas_ctx = meas_ops.build_meas_ctx(ham_data, trial_data)
    state = init_prop_state(sys=sys, n_walkers=params.n_walkers, seed=params.seed, ham_data=ham_data,
                            trial_ops_=trial_ops, trial_data=trial_data, meas_ops=meas_ops)
    kw = dict(sys=sys, params=params, ham_data=ham_data, trial_data=trial_data, meas_ops=meas_ops,
              prop_ops=prop_ops, prop_ctx=prop_ctx, meas_ctx=meas_ctx)

    def block(state_in):
        return block_fn(state_in, **kw)

    use_engine = block_fn is afqmc_block and sys.walker_kind.lower() == "restricted"
    run_blocks = make_run_blocks(block, kw if use_engine else None)

    t0 = time.perf_counter()
    t_mark = t0
    print_every = params.n_eql_blocks // 5 if params.n_eql_blocks >= 5 else 0
    e_eq = [float(state.e_estimate)]
    w_eq = [float(torch.as_tensor(state.weights).sum())]
    print("\nEquilibration:\n")
    if print_every:
        print(f"{'':4s}{'block':>9s}  {'E_blk':>14s}  {'W':>12s}  {'t[s]':>8s}")
    print(f"[eql {0:4d}/{params.n_eql_blocks}]  {e_eq[0]:14.10f}  {w_eq[0]:12.6e}  {0.0:8.1f}")
    chunk = print_every if print_every else params.n_eql_blocks
    for start in range(0, params.n_eql_blocks, max(chunk, 1)):
        n = min(chunk, params.n_eql_blocks - start)
        state, e_c, w_c = run_blocks(state, n_blocks=n)
        e_eq.extend(e_c.tolist())
        w_eq.extend(w_c.tolist())
        if start > 0:
            print(f"[eql {start:4d}/{params.n_eql_blocks}]  {float(e_c.mean()):14.10f}  "
                  f"{float(w_c.mean()):12.6e}  {time.perf_counter() - t0:8.1f}")

    print("\nSampling:\n")
    print_every = params.n_blocks // 10 if params.n_blocks >= 10 else 0
    e_s, w_s = [], []
    if print_every:
        print(f"{'':4s}{'block':>9s}  {'E_avg':>14s}  {'E_err':>10s}  {'E_block':>14s}  "
              f"{'W':>12s}  {'dt[s/bl]':>9s}  {'t[s]':>8s}")
    chunk = print_every if print_every else params.n_blocks
    for start in range(0, params.n_blocks, max(chunk, 1)):
        n = min(chunk, params.n_blocks - start)
        state, e_c, w_c = run_blocks(state, n_blocks=n)
        e_s.extend(e_c.tolist())
        w_s.extend(w_c.tolist())
        if start > 0:
            now = time.perf_counter()
            per = (now - t_mark) / float(n)
            t_mark = now
            st = blocking_analysis_ratio(np.asarray(e_s), np.asarray(w_s), print_q=False)
            print(f"[blk {start:4d}/{params.n_blocks}]  {float(st['mu']):14.10f}  {float(st['se_star']):10.3e}  "
                  f"{float(e_c.mean()):14.10f}  {float(w_c.mean()):12.6e}  {per:9.3f}  {now - t0:8.1f}")

    data = np.column_stack((np.asarray(e_s), np.asarray(w_s)))
    clean, _ = reject_outliers(data, obs=0)
    print(f"\nRejected {data.shape[0] - clean.shape[0]} outlier blocks.")
    print("\nFinal blocking analysis:")
    st = blocking_analysis_ratio(clean[:, 0], clean[:, 1], print_q=True)
    e_all = torch.tensor(np.concatenate([e_eq, clean[:, 0]]), dtype=torch.float64)
    w_all = torch.tensor(np.concatenate([w_eq, clean[:, 1]]), dtype=torch.float64)
    return st["mu"], st["se_star"], e_all, w_all
