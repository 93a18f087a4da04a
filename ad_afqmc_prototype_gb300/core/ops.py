"""Operation bundles: the plugin interfaces of the step (core/ops.py:11-90
of the reference).  Kernels are per-walker callables, as in the reference;
the engine's own kernels additionally carry a ``batched`` attribute that
``walkers.apply_chunked`` uses to run a whole chunk in one CUDA launch."""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any, Callable, Mapping, NamedTuple, Optional


class trial_ops(NamedTuple):
    """overlap(walker, trial_data), get_rdm1(trial_data), optional greens."""

    overlap: Callable[[Any, Any], Any]
    get_rdm1: Callable[[Any], Any]
    greens: Optional[Callable[[Any, Any], Any]] = None


class ham_ops(NamedTuple):
    n_fields: Callable[[Any], int]


meas_kernel = Callable[[Any, Any, Any, Any], Any]

k_energy = "energy"
k_force_bias = "force_bias"


@dataclass(frozen=True)
class meas_ops:
    """Measurement ops: overlap, context builder, kernels and observables."""

    overlap: Callable[[Any, Any], Any]
    build_meas_ctx: Callable[[Any, Any], Any] = lambda ham_data, trial_data: None
    kernels: Mapping[str, meas_kernel] = field(default_factory=dict)
    observables: Mapping[str, meas_kernel] = field(default_factory=dict)

    def has_kernel(self, name: str) -> bool:
        return name in self.kernels

    def has_observable(self, name: str) -> bool:
        return name in self.observables

    def require_kernel(self, name: str) -> meas_kernel:
        try:
            return self.kernels[name]
        except KeyError as e:
            avail = ", ".join(sorted(self.kernels.keys()))
            raise KeyError(f"missing required kernel '{name}'. available: [{avail}]") from e

    def require_observable(self, name: str) -> meas_kernel:
        try:
            return self.observables[name]
        except KeyError as e:
            avail = ", ".join(sorted(self.observables.keys()))
            raise KeyError(f"missing requested observable '{name}'. available: [{avail}]") from e

    def available_kernels(self) -> tuple[str, ...]:
        return tuple(sorted(self.kernels.keys()))

    def available_observables(self) -> tuple[str, ...]:
        return tuple(sorted(self.observables.keys()))
