"""Cholesky propagator ops (prop/chol_afqmc_ops.py:15-262 of the reference),
restricted walkers, on the CUDA engine."""
from __future__ import annotations

from dataclasses import dataclass
from typing import Any, Callable, NamedTuple

import torch

from .. import engine
from ..ham.chol import ham_chol


@dataclass(frozen=True)
class chol_afqmc_ctx:
    """dt, sqrt_dt (0-d f64), exp_h1_half (n, n) f64 device, mf_shifts (G,)
    c128 device, h0_prop (0-d c128)."""

    dt: torch.Tensor
    sqrt_dt: torch.Tensor
    exp_h1_half: torch.Tensor
    mf_shifts: torch.Tensor
    h0_prop: torch.Tensor


class chol_afqmc_ops(NamedTuple):
    n_fields: Callable[[], int]
    build_prop_ctx: Callable[[Any, float], chol_afqmc_ctx]  # (rdm1, dt) -> ctx
    apply_trotter: Callable[[Any, Any, chol_afqmc_ctx, int], Any]  # (w, field, ctx, n_terms) -> w


def _build_prop_ctx(ham_data: ham_chol, trial_rdm1, dt: float) -> chol_afqmc_ctx:
    """mf shifts, h0_prop, expm(-dt/2 h1_eff) on the device (:77-103)."""
    e, mf, h0p = engine.build_prop_ctx(ham_data.h0, ham_data.h1, ham_data.chol, trial_rdm1, dt)
    dt_t = torch.tensor(float(dt), dtype=torch.float64)
    return chol_afqmc_ctx(dt=dt_t, sqrt_dt=torch.sqrt(dt_t), exp_h1_half=e, mf_shifts=mf,
                          h0_prop=h0p.cpu().reshape(()))


def make_chol_afqmc_ops(ham_data: ham_chol, walker_kind: str) -> chol_afqmc_ops:
    """prop/chol_afqmc_ops.py:215-262; restricted basis and walkers only."""
    walker_kind = walker_kind.lower()
    nf = int(ham_data.chol.shape[0])

    def n_fields_() -> int:
        return nf

    def build_prop_ctx(trial_rdm1, dt):
        return _build_prop_ctx(ham_data, trial_rdm1, dt)

    if ham_data.basis == "generalized" and walker_kind != "generalized":
        raise ValueError("ham_data.basis='generalized' requires walker_kind='generalized'")
    if walker_kind not in ("restricted", "unrestricted", "generalized"):
        raise ValueError(f"unknown walker_kind: {walker_kind}")
    if ham_data.basis != "restricted":
        raise ValueError("the CUDA engine propagates walkers with a restricted-basis Hamiltonian only")

    if walker_kind == "generalized":
        def apply_trotter_g_batched(walkers, fields, ctx: chol_afqmc_ctx, n_terms: int, n_chunks: int = 1):
            """Top and bottom halves with the walker's V (:141-197)."""
            return engine.apply_trotter_g(walkers, fields, ham_data.chol, ctx.exp_h1_half, float(ctx.sqrt_dt),
                                          int(n_terms), n_chunks=n_chunks)

        def apply_trotter_g(w, field, ctx: chol_afqmc_ctx, n_terms: int):
            f = torch.as_tensor(field)[None].to(torch.complex128)
            return apply_trotter_g_batched(torch.as_tensor(w)[None], f, ctx, n_terms)[0]

        apply_trotter_g.batched = apply_trotter_g_batched
        apply_trotter_g.ham_data = ham_data
        return chol_afqmc_ops(n_fields_, build_prop_ctx, apply_trotter_g)

    if walker_kind == "unrestricted":
        def apply_trotter_u_batched(walkers, fields, ctx: chol_afqmc_ctx, n_terms: int, n_chunks: int = 1):
            """Both spins with the same V (:118-183); returns the (up, down) pair."""
            p = engine.apply_trotter_u(walkers, fields, ham_data.chol, ctx.exp_h1_half, float(ctx.sqrt_dt),
                                       int(n_terms), n_chunks=n_chunks)
            return engine.pair_views(p)

        def apply_trotter_u(w, field, ctx: chol_afqmc_ctx, n_terms: int):
            wu, wd = w
            f = torch.as_tensor(field)[None].to(torch.complex128)
            pu, pd = apply_trotter_u_batched((torch.as_tensor(wu)[None], torch.as_tensor(wd)[None]), f, ctx,
                                             n_terms)
            return (pu[0], pd[0])

        apply_trotter_u.batched = apply_trotter_u_batched
        apply_trotter_u.ham_data = ham_data
        return chol_afqmc_ops(n_fields_, build_prop_ctx, apply_trotter_u)

    def apply_trotter_batched(walkers, fields, ctx: chol_afqmc_ctx, n_terms: int, n_chunks: int = 1):
        """E_half exp(i sqrt_dt V(x)) E_half W for a batch (:173-183)."""
        return engine.apply_trotter(walkers, fields, ham_data.chol, ctx.exp_h1_half, float(ctx.sqrt_dt),
                                    int(n_terms), n_chunks=n_chunks)

    def apply_trotter(w, field, ctx: chol_afqmc_ctx, n_terms: int):
        w = torch.as_tensor(w)
        f = torch.as_tensor(field)
        return apply_trotter_batched(w[None], f[None].to(torch.complex128), ctx, n_terms)[0]

    apply_trotter.batched = apply_trotter_batched
    apply_trotter.ham_data = ham_data
    return chol_afqmc_ops(n_fields_, build_prop_ctx, apply_trotter)
