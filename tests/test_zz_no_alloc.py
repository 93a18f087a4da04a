"""afq_sr_indices_static -- the comb indices with the scan's scratch in a
file-scope device array, for callers that cannot allocate device memory
(for example a plug-in inside a JAX process, whose runtime reserves most of
the GPU's memory at start-up) -- against afq_sr_indices, which takes a
caller workspace.  Both run the same arithmetic, so indices and prefix sums
must agree bit for bit; two calls in a row check that the shared array's
leftover contents from the first call do not leak into the second.  The
file sorts last so that a run stopping at the first failure has already run
every other test."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _static_indices(weights, zeta):
    from ad_afqmc_prototype_gb300 import _lib, engine
    W = weights.shape[0]
    idx = torch.full((W,), -1, dtype=torch.int32, device=weights.device)
    cw = torch.full((W,), float("nan"), dtype=torch.float64, device=weights.device)
    _lib.call("afq_sr_indices_static", W, ctypes.c_void_p(weights.data_ptr()), float(zeta),
              ctypes.c_void_p(idx.data_ptr()), ctypes.c_void_p(cw.data_ptr()), engine.stream_ptr())
    return idx.long(), cw


def test_static_scratch_matches_workspace_version(cuda):
    from ad_afqmc_prototype_gb300 import engine
    rng = np.random.default_rng(2024)
    # two calls in a row: a larger call first leaves its levels in the array
    for W, zeta in ((5000, 0.37), (1000, 0.81)):
        w = rng.random(W) * rng.choice([0.0, 1.0, 1e-3, 9.0], size=W)
        wd = engine.as_device(w, engine.F64)
        ref_idx, ref_cw = engine.sr_indices(wd, zeta)
        idx, cw = _static_indices(wd, zeta)
        torch.cuda.synchronize()
        assert torch.equal(idx, ref_idx)
        assert torch.equal(cw, ref_cw)


def test_static_scratch_rejects_oversize(cuda):
    from ad_afqmc_prototype_gb300 import _lib
    lib = _lib.load()
    w = torch.ones((65537,), dtype=torch.float64, device="cuda")
    idx = torch.empty((65537,), dtype=torch.int32, device="cuda")
    rc = lib.afq_sr_indices_static(65537, ctypes.c_void_p(w.data_ptr()), 0.5, ctypes.c_void_p(idx.data_ptr()),
                                   None, None)
    assert rc == _lib.AFQ_E_UNSUPPORTED
    assert b"65536" in lib.afq_last_error()
