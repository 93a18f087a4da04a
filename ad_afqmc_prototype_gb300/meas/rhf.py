"""RHF measurement kernels (meas/rhf.py:15-176 of the reference),
restricted walkers, on the CUDA engine.  Per-walker functions keep the
reference's signatures; their ``batched`` attribute runs a chunk of walkers
in one launch (used by walkers.apply_chunked and the fused step)."""
from __future__ import annotations

from dataclasses import dataclass
from typing import Any

import torch

from .. import engine
from ..core.ops import k_energy, k_force_bias, meas_ops
from ..core.system import system
from ..ham.chol import ham_chol
from ..trial.rhf import overlap_g, overlap_r, overlap_u, rhf_trial


@dataclass(frozen=True)
class rhf_meas_ctx:
    rot_h1: torch.Tensor         # (nocc, norb) complex128
    rot_chol: torch.Tensor       # (n_chol, nocc, norb) float64 (real trial) or complex128
    rot_chol_flat: torch.Tensor  # (n_chol, nocc*norb) view of rot_chol


def build_meas_ctx(ham_data: ham_chol, trial_data: rhf_trial) -> rhf_meas_ctx:
    """Half-rotated h1 and Cholesky vectors (meas/rhf.py:141-150)."""
    if ham_data.basis != "restricted":
        raise ValueError("RHF meas_ops currently assumes ham_chol.basis == 'restricted'.")
    rot_h1, rot_chol = engine.build_meas_ctx(ham_data.h1, ham_data.chol, trial_data.mo_coeff,
                                             trial_data.is_real)
    return rhf_meas_ctx(rot_h1=rot_h1, rot_chol=rot_chol,
                        rot_chol_flat=rot_chol.reshape(rot_chol.shape[0], -1))


def half_green_batched(walkers, trial_data: rhf_trial):
    """G_half = solve((C^H W)^T, W^T) per walker (meas/rhf.py:15-19)."""
    return engine.half_green(walkers, trial_data.mo_coeff, trial_data.is_real)


def _fb_batched(walkers, _ham, meas_ctx: rhf_meas_ctx, trial_data: rhf_trial):
    return engine.force_bias(walkers, trial_data.mo_coeff, meas_ctx.rot_chol, trial_data.is_real)


def force_bias_kernel_r(walker, _ham: Any, meas_ctx: rhf_meas_ctx, trial_data: rhf_trial):
    """2 L~_flat vec(G_half) (meas/rhf.py:27-33)."""
    return _fb_batched(torch.as_tensor(walker)[None], _ham, meas_ctx, trial_data)[0]


force_bias_kernel_r.batched = _fb_batched


def _energy_batched(walkers, ham_data: ham_chol, meas_ctx: rhf_meas_ctx, trial_data: rhf_trial):
    return engine.energy(walkers, ham_data.h0, trial_data.mo_coeff, meas_ctx.rot_h1, meas_ctx.rot_chol,
                         trial_data.is_real)


def energy_kernel_r(walker, ham_data: ham_chol, meas_ctx: rhf_meas_ctx, trial_data: rhf_trial):
    """h0 + e1 + 2 sum_g c_g^2 - exc (meas/rhf.py:36-50)."""
    return _energy_batched(torch.as_tensor(walker)[None], ham_data, meas_ctx, trial_data)[0]


energy_kernel_r.batched = _energy_batched


def _pair1(walker):
    wu, wd = walker
    return (torch.as_tensor(wu)[None], torch.as_tensor(wd)[None])


def _fb_u_batched(walkers, _ham, meas_ctx: rhf_meas_ctx, trial_data: rhf_trial):
    return engine.force_bias_u(walkers, trial_data.mo_coeff, meas_ctx.rot_chol, trial_data.is_real)


def force_bias_kernel_u(walker, _ham: Any, meas_ctx: rhf_meas_ctx, trial_data: rhf_trial):
    """L~_flat vec(G_up + G_dn) for one pair (meas/rhf.py:60-72)."""
    return _fb_u_batched(_pair1(walker), _ham, meas_ctx, trial_data)[0]


force_bias_kernel_u.batched = _fb_u_batched


def _energy_u_batched(walkers, ham_data: ham_chol, meas_ctx: rhf_meas_ctx, trial_data: rhf_trial):
    return engine.energy_u(walkers, ham_data.h0, trial_data.mo_coeff, meas_ctx.rot_h1, meas_ctx.rot_chol,
                           trial_data.is_real)


def energy_kernel_u(walker, ham_data: ham_chol, meas_ctx: rhf_meas_ctx, trial_data: rhf_trial):
    """h0 + e1 + [sum_g (c_up + c_dn)^2 - exc_up - exc_dn] / 2 for one pair
    (meas/rhf.py:75-100)."""
    return _energy_u_batched(_pair1(walker), ham_data, meas_ctx, trial_data)[0]


energy_kernel_u.batched = _energy_u_batched


def _fb_g_batched(walkers, _ham, meas_ctx: rhf_meas_ctx, trial_data: rhf_trial):
    return engine.force_bias_g(walkers, trial_data.mo_coeff, meas_ctx.rot_chol, trial_data.is_real)


def force_bias_kernel_g(walker, _ham: Any, meas_ctx: rhf_meas_ctx, trial_data: rhf_trial):
    """L~_flat vec(G_uu + G_dd) for one (2n, 2o) walker (meas/rhf.py:112-130)."""
    return _fb_g_batched(torch.as_tensor(walker)[None], _ham, meas_ctx, trial_data)[0]


force_bias_kernel_g.batched = _fb_g_batched


def make_rhf_meas_ops(sys: system) -> meas_ops:
    """meas/rhf.py:153-176.  Generalized walkers have a force bias but, as in
    the reference, no energy kernel."""
    wk = sys.walker_kind.lower()
    if wk == "restricted":
        return meas_ops(overlap=overlap_r, build_meas_ctx=build_meas_ctx,
                        kernels={k_force_bias: force_bias_kernel_r, k_energy: energy_kernel_r})
    if wk == "unrestricted":
        return meas_ops(overlap=overlap_u, build_meas_ctx=build_meas_ctx,
                        kernels={k_force_bias: force_bias_kernel_u, k_energy: energy_kernel_u})
    if wk == "generalized":
        return meas_ops(overlap=overlap_g, build_meas_ctx=build_meas_ctx, kernels={k_force_bias: force_bias_kernel_g})
    raise ValueError(f"unknown walker_kind: {sys.walker_kind}")
