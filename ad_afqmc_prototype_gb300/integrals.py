"""Integrals (integrals.py of the reference): the modified Cholesky
decomposition of the two-electron integrals, on the GPU.

``modified_cholesky(mat, max_error)`` has the reference's signature and
result (integrals.py:3-46): ``mat`` is the 4-fold symmetric ERI matrix over
orbital pairs i >= j (as ``pyscf.ao2mo.restore(4, eri, norb)`` returns it),
the result a NumPy array (nchol, norb, norb) of symmetric Cholesky vectors.
The pivoted loop runs in the engine (``afq_modified_cholesky``, binary64);
``modified_cholesky_device`` returns the vectors as a device tensor.
"""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np
import torch

from . import _lib, engine


def modified_cholesky_device(mat, max_error: float = 1e-6, max_vectors: Optional[int] = None) -> torch.Tensor:
    """Cholesky vectors (nchol, norb, norb) float64 on the device.
    max_vectors bounds the memory (default: size, the reference's bound)."""
    m = engine.as_device(mat, engine.F64)
    if m.dim() != 2 or m.shape[0] != m.shape[1]:
        raise ValueError(f"mat must be square; got {tuple(m.shape)}")
    size = int(m.shape[0])
    norb = int(((-1 + (1 + 8 * size) ** 0.5) / 2))
    if norb * (norb + 1) // 2 != size:
        raise ValueError(f"mat size {size} is not norb (norb + 1) / 2")
    mv = size if max_vectors is None else int(max_vectors)
    lib = _lib.load()
    nb = int(lib.afq_modified_cholesky_workspace(size, mv))
    ws = torch.empty((max(nb, 256),), dtype=torch.uint8, device=m.device)
    out = torch.empty((mv, norb, norb), dtype=engine.F64, device=m.device)
    nchol = ctypes.c_int32(0)
    _lib.call("afq_modified_cholesky", size, engine.ptr(m), float(max_error), mv, engine.ptr(out),
              ctypes.byref(nchol), engine.ptr(ws), ws.numel(), engine.stream_ptr())
    return out[:nchol.value].clone()


def modified_cholesky(mat: np.ndarray, max_error: float = 1e-6) -> np.ndarray:
    """Modified cholesky decomposition for a given matrix (integrals.py:3-46)."""
    return modified_cholesky_device(mat, max_error).cpu().numpy()
