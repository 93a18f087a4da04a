"""Cholesky Hamiltonian container (ham/chol.py:12-65 of the reference).

Arrays are moved to the current CUDA device as float64 on construction.
The CUDA engine handles the restricted basis with real h1 and chol;
complex integrals raise ValueError."""
from __future__ import annotations

from dataclasses import dataclass
from typing import Any, Literal

import torch

ham_basis = Literal["restricted", "generalized"]


def _to_dev(x):
    from ..engine import as_device, F64
    t = x if isinstance(x, torch.Tensor) else torch.as_tensor(x)
    if t.is_complex():
        if torch.any(t.imag != 0):
            raise ValueError("complex Hamiltonian integrals are not supported by the CUDA engine")
        t = t.real
    return as_device(t, F64)


@dataclass(frozen=True)
class ham_chol:
    """basis="restricted": h1 (norb, norb), chol (n_fields, norb, norb)."""

    h0: Any
    h1: Any
    chol: Any
    basis: ham_basis = "restricted"

    def __post_init__(self):
        if self.basis not in ("restricted", "generalized"):
            raise ValueError(f"unknown basis: {self.basis}")
        h1 = self.h1 if isinstance(self.h1, torch.Tensor) else torch.as_tensor(self.h1)
        chol = self.chol if isinstance(self.chol, torch.Tensor) else torch.as_tensor(self.chol)
        if h1.dim() != 2:
            raise ValueError(f"h1 must be rank-2; got ndim={h1.dim()}")
        if h1.shape[0] != h1.shape[1]:
            raise ValueError(f"h1 must be square; got {tuple(h1.shape)}")
        if chol.dim() != 3:
            raise ValueError(f"chol must be rank-3; got ndim={chol.dim()}")
        if tuple(chol.shape[1:]) != tuple(h1.shape):
            raise ValueError(
                f"chol trailing dims must match h1; got chol {tuple(chol.shape)}, h1 {tuple(h1.shape)}")
        object.__setattr__(self, "h1", _to_dev(h1))
        object.__setattr__(self, "chol", _to_dev(chol))
        object.__setattr__(self, "h0", float(torch.as_tensor(self.h0).real.item()))

    @property
    def norb(self) -> int:
        return int(self.h1.shape[0])


def n_fields(ham: ham_chol) -> int:
    return int(ham.chol.shape[0])
