"""Differentiated energy: block energies and weights of a run of AFQMC
blocks as a differentiable function of the one-body Hamiltonian h1.

An engine form beside the reference's drop-in (the reference ships no
gradient).  ``block_energies(h1, ...)`` is a ``torch.autograd.Function``:
its forward runs ``n_blocks`` binary64 blocks through the engine
(``afq_grad_forward``, the same arithmetic as ``afqmc_block``) and its
backward runs the engine's hand-written adjoint kernels
(``afq_grad_backward``) with step checkpointing, returning dL/dh1 for any
loss L of the block energies and weights.  For a one-body perturbation
h1 + lam D, autograd gives dL/dlam = sum_ij dL/dh1[i, j] D[i, j]::

    lam = torch.zeros((), dtype=torch.float64, device="cuda", requires_grad=True)
    e, w = block_energies(ham.h1 + lam * D, ham_data=ham, trial_data=trial, params=params,
                          state=state, n_blocks=20, seed=7, checkpoint_every=20)
    E = (w * e).sum() / w.sum()
    E.backward()                      # lam.grad = dE/dlam

The derivative is the pathwise one that ``jax.grad`` of a wrapper around
the reference's ``afqmc_block`` (prop/blocks.py:22-95) gives on the same
fields: comb indices (walkers.py:233-265), the weight floor/cap
(prop/afqmc.py:127-134) and the energy clip (prop/blocks.py:59-66) held at
their values, the initial state a constant.  ``sr_fixed`` runs the blocks
with given comb indices, which is how finite differences of that same
function are taken.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any, Optional

import torch

from . import engine
from .ham.chol import ham_chol
from .prop.types import afqmc_params, prop_state
from .trial.rhf import get_rdm1, rhf_trial


def make_problem(h1: torch.Tensor, *, ham_data: ham_chol, trial_data: rhf_trial, params: afqmc_params,
                 n_walkers: int) -> engine.Problem:
    """The engine's binary64 problem for one-body matrix h1 (the propagator
    and measurement contexts of prop/chol_afqmc_ops.py:77-103 and
    meas/rhf.py:141-150 built on the device)."""
    if not trial_data.is_real:
        raise ValueError("the differentiated energy supports real trial orbitals")
    h1 = engine.as_device(h1.detach() if isinstance(h1, torch.Tensor) else h1, engine.F64)
    n = trial_data.norb
    if h1.shape != (n, n):
        raise ValueError(f"h1 must be ({n}, {n}); got {tuple(h1.shape)}")
    e_half, mf, h0p = engine.build_prop_ctx(ham_data.h0, h1, ham_data.chol, get_rdm1(trial_data), params.dt)
    rot_h1, rot_chol = engine.build_meas_ctx(h1, ham_data.chol, trial_data.mo_coeff, True)
    return engine.Problem(n_walkers=n_walkers, norb=n, nocc=trial_data.nocc, nchol=int(ham_data.chol.shape[0]),
                          trial_is_real=True, h0=ham_data.h0, chol=ham_data.chol, mo=trial_data.mo_coeff,
                          dt=float(params.dt), sqrt_dt=float(params.dt) ** 0.5, exp_h1_half=e_half, mf_shifts=mf,
                          h0_prop=complex(h0p.item()), rot_h1=rot_h1, rot_chol=rot_chol)


@dataclass
class GradRun:
    """Inputs of a differentiated run, and what the forward leaves behind:
    the final state, the comb indices (n_blocks, W) and the tape."""
    ham_data: ham_chol
    trial_data: rhf_trial
    params: afqmc_params
    state: prop_state
    n_blocks: int
    seed: int
    counter: int
    checkpoint_blocks: int
    sr_fixed: Optional[torch.Tensor] = None
    final_state: Optional[engine.DeviceState] = None
    sr_idx: Optional[torch.Tensor] = None
    tape: Optional[torch.Tensor] = field(default=None, repr=False)
    problem: Optional[engine.Problem] = field(default=None, repr=False)
    h1: Optional[torch.Tensor] = field(default=None, repr=False)


def _device_state(state: prop_state) -> engine.DeviceState:
    return engine.DeviceState(
        walkers=engine.as_device(state.walkers, engine.C128).clone(),
        weights=engine.as_device(state.weights, engine.F64).clone(),
        overlaps=engine.as_device(state.overlaps, engine.C128).clone(),
        pop_shift=engine.as_device(state.pop_control_ene_shift, engine.F64).reshape(1).clone(),
        e_estimate=engine.as_device(state.e_estimate, engine.F64).reshape(1).clone())


class AfqmcBlocksFunction(torch.autograd.Function):
    """(energies, weights) = f(h1) for a run of blocks; see the module doc."""

    @staticmethod
    def forward(ctx, h1: torch.Tensor, run: GradRun):
        W = int(run.state.walkers.shape[0])
        prob = make_problem(h1, ham_data=run.ham_data, trial_data=run.trial_data, params=run.params, n_walkers=W)
        st = _device_state(run.state)
        e, w, idx, tape = engine.grad_forward(prob, run.params, st, run.n_blocks, run.seed, run.counter,
                                              run.checkpoint_blocks, run.sr_fixed)
        run.final_state, run.sr_idx, run.tape, run.problem = st, idx, tape, prob
        run.h1 = engine.as_device(h1.detach(), engine.F64).clone()
        ctx.run = run
        return e, w

    @staticmethod
    def backward(ctx, e_bar, w_bar):
        run: GradRun = ctx.run
        B = run.n_blocks
        dev = run.h1.device
        eb = torch.zeros((B,), dtype=engine.F64, device=dev) if e_bar is None else e_bar.to(engine.F64)
        wb = torch.zeros((B,), dtype=engine.F64, device=dev) if w_bar is None else w_bar.to(engine.F64)
        h1_bar = engine.grad_backward(run.problem, run.params, run.h1, B, run.seed, run.counter,
                                      run.checkpoint_blocks, run.tape, eb.contiguous(), wb.contiguous())
        engine.workspace_status()
        return h1_bar, None


def block_energies(h1: torch.Tensor, *, ham_data: ham_chol, trial_data: rhf_trial, params: afqmc_params,
                   state: prop_state, n_blocks: int, seed: Optional[int] = None, counter: Optional[int] = None,
                   checkpoint_every: int = 20, sr_fixed: Optional[torch.Tensor] = None,
                   run_out: Optional[list] = None):
    """Block energies and weights (device (n_blocks,) f64 each) of n_blocks
    blocks from `state` with one-body matrix h1, differentiable in h1.

    Fields and comb uniforms come from the engine's Philox stream: seed and
    counter default to state.rng_key; block b uses counter + b (n_prop_steps
    + 1), as the driver's block loop does.  checkpoint_every (steps, rounded
    down to whole blocks, at least one) sets how often the forward keeps the
    state for the backward's replay.  run_out (a list) receives the GradRun
    (final state, comb indices)."""
    if str(getattr(params, "precision", "fp64")).lower() != "fp64":
        raise ValueError("the differentiated energy runs the binary64 form (params.precision='fp64')")
    key = torch.as_tensor(state.rng_key).reshape(-1)
    seed = int(key[0]) if seed is None else int(seed)
    counter = int(key[1]) if counter is None else int(counter)
    ck = min(int(n_blocks), max(1, int(checkpoint_every) // max(1, int(params.n_prop_steps))))
    run = GradRun(ham_data=ham_data, trial_data=trial_data, params=params, state=state, n_blocks=int(n_blocks),
                  seed=seed, counter=counter, checkpoint_blocks=ck, sr_fixed=sr_fixed)
    if run_out is not None:
        run_out.append(run)
    if not isinstance(h1, torch.Tensor):
        h1 = torch.as_tensor(h1)
    return AfqmcBlocksFunction.apply(h1, run)


def mixed_energy(energies: torch.Tensor, weights: torch.Tensor) -> torch.Tensor:
    """sum_b W_b e_b / sum_b W_b (the weighted mean over blocks)."""
    return (weights * energies).sum() / weights.sum()


def energy_and_derivative(D, *, ham_data: ham_chol, trial_data: rhf_trial, params: afqmc_params,
                          state: prop_state, n_blocks: int, lam: float = 0.0, seed: Optional[int] = None,
                          counter: Optional[int] = None, checkpoint_every: int = 20) -> dict[str, Any]:
    """E(lam) = mixed_energy of the run with h1 + lam D, and dE/dlam by the
    adjoint.  Returns dict(energy, derivative, h1_grad, run)."""
    D = engine.as_device(D, engine.F64)
    h1 = (ham_data.h1 + float(lam) * D).detach().requires_grad_(True)
    runs: list = []
    e, w = block_energies(h1, ham_data=ham_data, trial_data=trial_data, params=params, state=state,
                          n_blocks=n_blocks, seed=seed, counter=counter, checkpoint_every=checkpoint_every,
                          run_out=runs)
    E = mixed_energy(e, w)
    E.backward()
    g = h1.grad.detach()
    return {"energy": float(E.detach()), "derivative": float((g * D).sum()), "h1_grad": g, "run": runs[0],
            "block_energies": e.detach(), "block_weights": w.detach()}
