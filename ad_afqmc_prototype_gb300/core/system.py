"""Static system configuration (core/system.py:6-32 of the reference)."""
from __future__ import annotations

from dataclasses import dataclass
from typing import Literal, Tuple

walker_kind = Literal["restricted", "unrestricted", "generalized"]


@dataclass(frozen=True)
class system:
    """norb spatial orbitals, nelec = (n_up, n_dn), walker representation."""

    norb: int
    nelec: Tuple[int, int]
    walker_kind: walker_kind

    @property
    def nup(self) -> int:
        return self.nelec[0]

    @property
    def ndn(self) -> int:
        return self.nelec[1]

    @property
    def ne(self) -> int:
        return self.nelec[0] + self.nelec[1]
