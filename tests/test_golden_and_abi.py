"""CPU tests: the oracle reproduces the committed golden fixtures, and the
C-ABI library loads, exports every function include/afqmc_gb300.h declares
and rejects bad arguments before touching a device."""
import ctypes
import os
import re

import numpy as np
import pytest

from oracle import afqmc_oracle as O
from ad_afqmc_prototype_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


def test_oracle_reproduces_block_golden():
    g = np.load(os.path.join(GOLD, "c1_block.npz"))
    H = synth.make_workload(synth.WORKLOADS["c1_n12_o6_g48_w256"])
    W = g["fields"].shape[2]
    prob = O.make_problem(H["h0"], H["h1"], H["chol"], H["mo_coeff"], 0.005)
    P = O.Params(dt=0.005, n_prop_steps=10, qr_every=5)
    st = O.init_prop_state(prob, W, synth.trial_walkers(H["mo_coeff"], W))
    assert abs(st.e_estimate - float(g["e_estimate"])) < 1e-12
    for b in range(g["fields"].shape[0]):
        st, obs, idx = O.afqmc_block(prob, P, st, g["fields"][b], float(g["zetas"][b]))
        assert abs(obs["energy"] - g["block_energy"][b]) < 1e-10
        np.testing.assert_array_equal(idx, g["sr_idx"][b])
    np.testing.assert_allclose(st.walkers, g["final_walkers"], atol=1e-10)


def test_oracle_reproduces_kernel_golden():
    g = np.load(os.path.join(GOLD, "kernels.npz"))
    for tag in ("real", "cplx"):
        c = g[f"{tag}_mo"]
        ctx = O.build_meas_ctx(g["h1"], g["chol"], c)
        np.testing.assert_allclose(O.energy_r(g["walkers"], float(g["h0"]), ctx, c), g[f"{tag}_energy"],
                                   rtol=1e-12)
        np.testing.assert_allclose(O.force_bias_r(g["walkers"], ctx, c), g[f"{tag}_fb"], rtol=1e-12)


def _declared_functions():
    src = open(os.path.join(ROOT, "include", "afqmc_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(afq_\w+)\s*\(", src)))


def test_library_exports_every_declared_function(engine_lib):
    names = _declared_functions()
    assert len(names) >= 25
    for name in names:
        assert hasattr(engine_lib, name), name
    from ad_afqmc_prototype_gb300 import _lib
    assert sorted(_lib.exported_symbols()) == names


def test_abi_version_and_status_strings(engine_lib):
    assert engine_lib.afq_abi_version() == 2
    assert engine_lib.afq_status_string(0) == b"ok"
    assert engine_lib.afq_status_string(-4) == b"workspace too small"


def test_argument_validation_needs_no_device(engine_lib):
    from ad_afqmc_prototype_gb300 import _lib
    d = _lib.afq_dims(0, 12, 6, 48, 1, 0)  # zero walkers
    rc = engine_lib.afq_overlap(ctypes.byref(d), None, None, None, None)
    assert rc == _lib.AFQ_E_INVALID_ARGUMENT
    assert b"n_walkers" in engine_lib.afq_last_error()
    d = _lib.afq_dims(4, 12, 13, 48, 1, 0)  # nocc > norb
    assert engine_lib.afq_overlap(ctypes.byref(d), None, None, None, None) == _lib.AFQ_E_INVALID_ARGUMENT
    d = _lib.afq_dims(4, 600, 6, 48, 1, 0)  # norb beyond the kernels' limit
    assert engine_lib.afq_overlap(ctypes.byref(d), None, None, None, None) == _lib.AFQ_E_UNSUPPORTED
    assert engine_lib.afq_step(None, None, None, None, 0, 0, None, 0, None) == _lib.AFQ_E_INVALID_ARGUMENT
    d = _lib.afq_dims(4, 12, 6, 48, 1, 0)
    assert engine_lib.afq_step_workspace(ctypes.byref(d), 1) > 0
    # workspace grows with walkers; chunking shrinks the V workspace
    d2 = _lib.afq_dims(64, 12, 6, 48, 1, 0)
    assert engine_lib.afq_step_workspace(ctypes.byref(d2), 1) > engine_lib.afq_step_workspace(ctypes.byref(d), 1)
    assert engine_lib.afq_step_workspace(ctypes.byref(d2), 4) < engine_lib.afq_step_workspace(ctypes.byref(d2), 1)


def test_python_layer_raises_without_cuda():
    import torch
    if torch.cuda.is_available():
        pytest.skip("CUDA present")
    from ad_afqmc_prototype_gb300 import engine
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        engine.device()
