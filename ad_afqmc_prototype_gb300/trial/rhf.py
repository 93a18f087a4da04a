"""RHF trial (trial/rhf.py:12-71 of the reference), restricted walkers.

``rhf_trial.mo_coeff`` is kept on the device as complex128; ``is_real``
records that the imaginary part is zero, which selects the engine's
real-trial kernels (half-rotated Cholesky vectors stored real)."""
from __future__ import annotations

from dataclasses import dataclass

import torch

from .. import engine
from ..core.ops import trial_ops
from ..core.system import system


@dataclass(frozen=True)
class rhf_trial:
    mo_coeff: torch.Tensor  # (norb, nocc)

    def __post_init__(self):
        m = self.mo_coeff if isinstance(self.mo_coeff, torch.Tensor) else torch.as_tensor(self.mo_coeff)
        if m.dim() != 2:
            raise ValueError(f"mo_coeff must be (norb, nocc); got {tuple(m.shape)}")
        is_real = (not m.is_complex()) or bool(torch.all(m.imag == 0))
        object.__setattr__(self, "mo_coeff", engine.as_device(m, engine.C128))
        object.__setattr__(self, "is_real", is_real)

    @property
    def norb(self) -> int:
        return int(self.mo_coeff.shape[0])

    @property
    def nocc(self) -> int:
        return int(self.mo_coeff.shape[1])


def get_rdm1(trial_data: rhf_trial) -> torch.Tensor:
    """Stacked [C C^H, C C^H] (trial/rhf.py:29-32), formed by the engine's kernel."""
    return engine.trial_rdm1(trial_data.mo_coeff)


def _overlap_batched(walkers, trial_data: rhf_trial):
    return engine.overlap(walkers, trial_data.mo_coeff, trial_data.is_real)


def overlap_r(walker, trial_data: rhf_trial):
    """det(C^H W)^2 for one walker (trial/rhf.py:35-37)."""
    return _overlap_batched(torch.as_tensor(walker).unsqueeze(0) if isinstance(walker, torch.Tensor)
                            else torch.as_tensor(walker)[None], trial_data)[0]


overlap_r.batched = _overlap_batched


def _overlap_u_batched(walkers, trial_data: rhf_trial):
    return engine.overlap_u(walkers, trial_data.mo_coeff, trial_data.is_real)


def overlap_u(walker, trial_data: rhf_trial):
    """det(C^H W_up) det(C^H W_dn) for one pair (trial/rhf.py:40-44)."""
    wu, wd = walker
    return _overlap_u_batched((torch.as_tensor(wu)[None], torch.as_tensor(wd)[None]), trial_data)[0]


overlap_u.batched = _overlap_u_batched


def _overlap_g_batched(walkers, trial_data: rhf_trial):
    return engine.overlap_g(walkers, trial_data.mo_coeff, trial_data.is_real)


def overlap_g(walker, trial_data: rhf_trial):
    """det(vstack(C^H W_top, C^H W_bot)) for one (2n, 2o) walker (trial/rhf.py:47-53)."""
    return _overlap_g_batched(torch.as_tensor(walker)[None], trial_data)[0]


overlap_g.batched = _overlap_g_batched


def make_rhf_trial_ops(sys: system) -> trial_ops:
    """trial/rhf.py:56-71."""
    if sys.nup != sys.ndn:
        raise ValueError("RHF requires nelec[0] == nelec[1].")
    wk = sys.walker_kind.lower()
    if wk == "restricted":
        return trial_ops(overlap=overlap_r, get_rdm1=get_rdm1)
    if wk == "unrestricted":
        return trial_ops(overlap=overlap_u, get_rdm1=get_rdm1)
    if wk == "generalized":
        return trial_ops(overlap=overlap_g, get_rdm1=get_rdm1)
    raise ValueError(f"unknown walker_kind: {sys.walker_kind}")
