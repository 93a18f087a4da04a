"""Seeded synthetic Cholesky Hamiltonians, RHF trials and perturbations.

The workloads (there is no public dataset for this path) are defined as:

* h1 = diag(linspace(-2, 0.5, n)) + off-diagonal part of sym(N(0, 0.1)),
  sym(B) = (B + B^T)/2 as in the reference's test generator
  (tests/test_auto.py:29-45);
* L_g = sym(N(0, 1)) * scale * exp(-g / decay), g = 0..G-1, real symmetric;
  the 12-orbital workload uses scale 0.3 and decay 12 = G/4; scaled-up
  workloads keep the same decay profile (decay = G/4) and the per-entry
  scale 0.3*12/n.  With that rule the local-energy spread across walkers
  stays near 1 Ha and no walker energy is clipped at sqrt(2/dt) at any of
  the five sizes; keeping 0.3 per entry at n >= 60 drives every walker's
  energy past the clip within ten steps (weights collapse to one walker);
* h0 = 0; the trial is the lowest nocc eigenvectors of h1 (real);
* D = sym(N(0, 0.05)) for the one-body perturbation lambda*D.

Draw order from ``numpy.random.default_rng(seed)``: h1 off-diagonal, chol, D.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class Workload:
    name: str
    nbasis: int
    nocc: int
    nchol: int
    n_walkers: int
    n_steps: int
    seed: int = 0


# The five workloads of the benchmark description, smallest first.
WORKLOADS = {
    "c1_n12_o6_g48_w256": Workload("c1_n12_o6_g48_w256", 12, 6, 48, 256, 100, 0),
    "c2_n120_o20_g600_w2048": Workload("c2_n120_o20_g600_w2048", 120, 20, 600, 2048, 200, 1),
    "c3_n60_o10_g300_w1024": Workload("c3_n60_o10_g300_w1024", 60, 10, 300, 1024, 200, 2),
    "c4_n200_o30_g1000_w4096": Workload("c4_n200_o30_g1000_w4096", 200, 30, 1000, 4096, 400, 3),
    "c5_n400_o50_g2000_w1024": Workload("c5_n400_o50_g2000_w1024", 400, 50, 2000, 1024, 200, 4),
}


def _sym(b):
    return 0.5 * (b + np.swapaxes(b, -1, -2))


def make_hamiltonian(nbasis: int, nocc: int, nchol: int, seed: int = 0,
                     scale: float | None = None, decay: float | None = None):
    """Returns dict(h0, h1, chol, mo_coeff, D) as NumPy float64 arrays."""
    n, g = nbasis, nchol
    rng = np.random.default_rng(seed)
    off = _sym(rng.normal(0.0, 0.1, size=(n, n)))
    off = off - np.diag(np.diag(off))
    h1 = np.diag(np.linspace(-2.0, 0.5, n)) + off
    if scale is None:
        scale = 0.3 * 12.0 / n
    if decay is None:
        decay = g / 4.0
    b = _sym(rng.normal(0.0, 1.0, size=(g, n, n)))
    chol = b * (scale * np.exp(-np.arange(g) / decay))[:, None, None]
    d = _sym(rng.normal(0.0, 0.05, size=(n, n)))
    evals, evecs = np.linalg.eigh(h1)
    mo = np.ascontiguousarray(evecs[:, :nocc])
    return {"h0": 0.0, "h1": np.ascontiguousarray(h1), "chol": np.ascontiguousarray(chol),
            "mo_coeff": mo, "D": np.ascontiguousarray(d),
            "scale": float(scale), "decay": float(decay)}


def make_workload(w: Workload, **kw):
    return make_hamiltonian(w.nbasis, w.nocc, w.nchol, seed=w.seed, **kw)


def trial_walkers(mo_coeff: np.ndarray, n_walkers: int) -> np.ndarray:
    """All walkers start at the trial (complex128, (W, n, o))."""
    w0 = np.asarray(mo_coeff, dtype=np.complex128)
    return np.ascontiguousarray(np.broadcast_to(w0, (n_walkers, *w0.shape)))
