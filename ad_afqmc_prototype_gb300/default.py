"""Restricted AFQMC from a mean-field object (default.py of the reference).

``Rhf(mf).kernel()`` has the reference's behaviour (default.py:15-47): MO-basis
one-body integrals and nuclear repulsion from ``mf``, the two-electron
integrals in the MO basis as a 4-fold packed matrix, their modified Cholesky
vectors (max_error 1e-6, on the GPU here: ``integrals.modified_cholesky``),
the RHF trial ``eye(nao, nelectron // 2)``, restricted walkers, and
``driver.run_afqmc_energy`` with 20 equilibration and 200 sampling blocks.

The reference builds the MO integrals with pyscf (``ao2mo.kernel`` and
``ao2mo.restore(4, ...)``).  pyscf is optional here: pass the MO-basis
integrals yourself with ``eri=`` (full (n, n, n, n), 4-fold packed
(npair, npair) or 8-fold packed (npair (npair + 1) / 2,), pairs i >= j in
row-major triangle order, as pyscf stores them), or have pyscf importable
and ``Rhf(mf)`` calls it as the reference does.  ``mf`` needs only ``mol``
(``nao``, ``nelec``, ``nelectron``), ``mo_coeff``, ``get_hcore()`` and
``energy_nuc()``.
"""
from __future__ import annotations

from typing import Optional

import numpy as np
import torch

from . import driver, integrals
from .core import system
from .ham.chol import ham_chol
from .meas.rhf import make_rhf_meas_ops
from .prop.blocks import afqmc_block
from .prop.chol_afqmc_ops import make_chol_afqmc_ops
from .prop.types import afqmc_params
from .trial.rhf import make_rhf_trial_ops, rhf_trial


def restore_4fold(eri, norb: int) -> np.ndarray:
    """The (npair, npair) 4-fold packed form of MO-basis integrals given full,
    4-fold or 8-fold packed (pyscf's ``ao2mo.restore(4, eri, norb)``)."""
    eri = np.asarray(eri, dtype=np.float64)
    npair = norb * (norb + 1) // 2
    if eri.shape == (norb, norb, norb, norb):
        ii, jj = np.tril_indices(norb)
        return np.ascontiguousarray(eri[ii, jj][:, ii, jj])
    if eri.shape == (npair, npair):
        return np.ascontiguousarray(eri)
    if eri.ndim == 1 and eri.shape[0] == npair * (npair + 1) // 2:
        out = np.zeros((npair, npair))
        r, c = np.tril_indices(npair)
        out[r, c] = eri
        out[c, r] = eri
        return out
    raise ValueError(f"eri of shape {eri.shape} is not full, 4-fold or 8-fold packed for norb={norb}")


def _mo_eri_from_pyscf(mf) -> np.ndarray:
    try:
        from pyscf import ao2mo
    except ImportError as e:  # the reference needs pyscf here; this package takes eri= instead
        raise ImportError("pyscf is not installed: pass the MO-basis two-electron integrals as Rhf(mf, eri=...)") from e
    mol = mf.mol
    eri = np.array(ao2mo.kernel(mol, mf.mo_coeff))
    return ao2mo.restore(4, eri, mol.nao)


class Rhf:
    def __init__(self, mf, eri: Optional[np.ndarray] = None, max_error: float = 1e-6):
        mol = mf.mol
        h0 = float(mf.energy_nuc())
        mo = np.asarray(mf.mo_coeff)
        h1 = np.array(mo.T @ np.asarray(mf.get_hcore()) @ mo)
        norb = int(mol.nao)
        eri4 = restore_4fold(_mo_eri_from_pyscf(mf) if eri is None else eri, norb)
        chol = integrals.modified_cholesky_device(eri4, max_error=max_error)

        sys_ = system.system(norb=norb, nelec=tuple(mol.nelec), walker_kind="restricted")
        dev = chol.device
        ham_data = ham_chol(h0=torch.tensor(h0, dtype=torch.float64, device=dev),
                            h1=torch.as_tensor(h1, dtype=torch.float64, device=dev), chol=chol)
        self.trial_data = rhf_trial(torch.eye(norb, int(mol.nelectron) // 2, dtype=torch.float64, device=dev))
        self.trial_ops = make_rhf_trial_ops(sys=sys_)
        self.meas_ops = make_rhf_meas_ops(sys=sys_)
        self.prop_ops = make_chol_afqmc_ops(ham_data, sys_.walker_kind)
        self.params = afqmc_params(n_eql_blocks=20, n_blocks=200, seed=np.random.randint(0, int(1e6)))
        self.block_fn = afqmc_block

        self.sys = sys_
        self.ham_data = ham_data

    def kernel(self):
        return driver.run_afqmc_energy(
            sys=self.sys,
            params=self.params,
            ham_data=self.ham_data,
            trial_ops=self.trial_ops,
            trial_data=self.trial_data,
            meas_ops=self.meas_ops,
            block_fn=self.block_fn,
        )
