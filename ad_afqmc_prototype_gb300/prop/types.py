"""State and parameters (prop/types.py:10-32 of the reference)."""
from __future__ import annotations

from dataclasses import dataclass
from typing import Any, NamedTuple

import torch


class prop_state(NamedTuple):
    """walkers (W, n, o) c128, weights (W,) f64, overlaps (W,) c128 on the
    device; rng_key = int64 CPU tensor [seed, counter] of the engine's
    Philox stream; pop_control_ene_shift and e_estimate are 0-d f64 device
    tensors."""

    walkers: Any
    weights: torch.Tensor
    overlaps: torch.Tensor
    rng_key: torch.Tensor
    pop_control_ene_shift: torch.Tensor
    e_estimate: torch.Tensor


def PRNGKey(seed: int) -> torch.Tensor:
    """Key of the engine's counter-based stream: [seed, counter = 0]."""
    return torch.tensor([int(seed), 0], dtype=torch.int64)


def split(key: torch.Tensor):
    """(next key, subkey): the subkey draws with the current counter."""
    nxt = key.clone()
    nxt[1] += 1
    return nxt, key.clone()


@dataclass(frozen=True)
class afqmc_params:
    """Defaults as prop/types.py:19-32.  Extra fields: ``qr_every`` (an
    orthonormalisation after every qr_every-th step inside a block, 0 = only
    at block end) and ``precision`` ("fp64", "mixed" or "mixed_fast")."""

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
    precision: str = "fp64"
