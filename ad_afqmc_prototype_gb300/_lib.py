"""ctypes binding of libafqmc_gb300.so (the C ABI in include/afqmc_gb300.h).

The library is the only compute path of this package: if it is missing or
cannot be loaded, every operation raises; there is no CPU or PyTorch
fallback.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, Structure, c_double, c_int32, c_int64, c_size_t, c_uint64, c_void_p

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libafqmc_gb300.so")

AFQ_OK = 0
AFQ_E_INVALID_ARGUMENT = -1
AFQ_E_UNSUPPORTED = -2
AFQ_E_CUDA = -3
AFQ_E_WORKSPACE = -4
AFQ_E_DEVICE_CHECK = -5

AFQ_PREC_FP64 = 0
AFQ_PREC_MIXED = 1
AFQ_PREC_MIXED_FAST = 2

AFQ_STATUS_WAIT_EXPIRED = 1
AFQ_STATUS_SINGULAR = 2
AFQ_STATUS_BAD_INDEX = 3
AFQ_STATUS_NONFINITE = 4

AFQ_CV_OFF = 0
AFQ_CV_RECORD = 1
AFQ_CV_ESTIMATE = 2
AFQ_CV_FEATURES = 64


class afq_dims(Structure):
    _fields_ = [("n_walkers", c_int32), ("norb", c_int32), ("nocc", c_int32), ("nchol", c_int32),
                ("trial_is_real", c_int32), ("precision", c_int32)]


class afq_params(Structure):
    _fields_ = [("dt", c_double), ("pop_control_damping", c_double), ("weight_floor", c_double),
                ("weight_cap", c_double), ("shift_ema", c_double), ("n_exp_terms", c_int32),
                ("n_prop_steps", c_int32), ("qr_every", c_int32), ("n_chunks", c_int32)]


class afq_problem(Structure):
    _fields_ = [("dims", afq_dims), ("h0", c_double), ("chol", c_void_p), ("mo_coeff", c_void_p),
                ("dt", c_double), ("sqrt_dt", c_double), ("exp_h1_half", c_void_p),
                ("mf_shifts", c_void_p), ("h0_prop_re", c_double), ("h0_prop_im", c_double),
                ("rot_h1", c_void_p), ("rot_chol", c_void_p), ("lowp", c_void_p)]


class afq_state(Structure):
    _fields_ = [("walkers", c_void_p), ("weights", c_void_p), ("overlaps", c_void_p),
                ("pop_control_ene_shift", c_void_p), ("e_estimate", c_void_p)]


class afq_cv(Structure):
    _fields_ = [("mode", c_int32), ("hidden", c_int32), ("n_sample", c_int32), ("pad_", c_int32),
                ("net", c_void_p), ("feat_shift", c_void_p), ("feat_scale", c_void_p), ("y_shift", c_double),
                ("y_scale", c_double), ("rec_features", c_void_p), ("rec_exchange", c_void_p),
                ("stats", c_void_p)]


P = c_void_p
_SIGS = {
    "afq_abi_version": (c_int32, []),
    "afq_status_string": (ctypes.c_char_p, [c_int32]),
    "afq_last_error": (ctypes.c_char_p, []),
    "afq_build_prop_ctx_workspace": (c_size_t, [c_int32, c_int32]),
    "afq_build_prop_ctx": (c_int32, [c_int32, c_int32, c_double, c_double, P, P, P, c_int32, P, P, P,
                                     P, c_size_t, P]),
    "afq_trial_rdm1": (c_int32, [c_int32, c_int32, P, P, P]),
    "afq_build_meas_ctx": (c_int32, [c_int32, c_int32, c_int32, P, P, P, c_int32, P, P, P]),
    "afq_lowp_bytes": (c_size_t, [POINTER(afq_dims)]),
    "afq_prepare_lowp": (c_int32, [POINTER(afq_dims), P, P, P, c_size_t, P]),
    "afq_lowp_gemm_tn": (c_int32, [c_int32, c_int32, c_int32, P, c_int64, P, c_int64, P, c_int64, P, c_int32, P]),
    "afq_workspace_status": (c_int32, [P, POINTER(c_int32), P]),
    "afq_workspace_counters": (c_int32, [P, POINTER(c_int32), POINTER(c_int32), P]),
    "afq_selftest_wait": (c_int32, [c_int64, c_int32, P, P]),
    "afq_overlap": (c_int32, [POINTER(afq_dims), P, P, P, P]),
    "afq_half_green": (c_int32, [POINTER(afq_dims), P, P, P, P, P]),
    "afq_force_bias_workspace": (c_size_t, [POINTER(afq_dims)]),
    "afq_force_bias": (c_int32, [POINTER(afq_dims), P, P, P, P, P, c_size_t, P]),
    "afq_energy_workspace": (c_size_t, [POINTER(afq_dims)]),
    "afq_energy": (c_int32, [POINTER(afq_dims), c_double, P, P, P, P, P, P, c_size_t, P]),
    "afq_apply_trotter_workspace": (c_size_t, [POINTER(afq_dims), c_int32]),
    "afq_apply_trotter": (c_int32, [POINTER(afq_dims), c_int32, c_double, c_int32, P, P, P, P, P, P,
                                    c_size_t, P]),
    "afq_orthogonalize": (c_int32, [POINTER(afq_dims), P, P, P, P]),
    "afq_sr_workspace": (c_size_t, [c_int32]),
    "afq_sr_indices": (c_int32, [c_int32, P, c_double, P, P, P, c_size_t, P]),
    "afq_sr_indices_static": (c_int32, [c_int32, P, c_double, P, P, P]),
    "afq_stochastic_reconfiguration": (c_int32, [POINTER(afq_dims), P, c_double, P, P, P, P, P,
                                                 c_size_t, P]),
    "afq_fill_normal": (c_int32, [c_int64, c_uint64, c_uint64, P, P]),
    "afq_fill_uniform": (c_int32, [c_int64, c_uint64, c_uint64, P, P]),
    "afq_field_shift": (c_int32, [POINTER(afq_dims), c_double, P, P, P, P, P, P, P]),
    "afq_field_shift_lowp_bytes": (c_size_t, [c_int32, c_int32, c_int32]),
    "afq_field_shift_lowp": (c_int32, [c_int32, c_int32, c_int32, c_double, P, P, P, P, P, P, c_size_t, P]),
    "afq_weight_update": (c_int32, [POINTER(afq_dims), POINTER(afq_params), POINTER(afq_problem), P, P,
                                    P, POINTER(afq_state), P]),
    "afq_block_measure": (c_int32, [c_int32, c_double, c_double, P, P, P, P, P, P, P]),
    "afq_step_workspace": (c_size_t, [POINTER(afq_dims), c_int32]),
    "afq_step": (c_int32, [POINTER(afq_problem), POINTER(afq_params), POINTER(afq_state), P, c_uint64,
                           c_uint64, P, c_size_t, P]),
    "afq_block_workspace": (c_size_t, [POINTER(afq_dims), c_int32]),
    "afq_block": (c_int32, [POINTER(afq_problem), POINTER(afq_params), POINTER(afq_state), P, c_double,
                            c_uint64, c_uint64, P, P, P, P, c_size_t, P]),
    "afq_block_cv": (c_int32, [POINTER(afq_problem), POINTER(afq_params), POINTER(afq_state), P, c_double,
                               c_uint64, c_uint64, P, P, P, POINTER(afq_cv), P, c_size_t, P]),
    "afq_run_blocks_workspace": (c_size_t, [POINTER(afq_dims), c_int32]),
    "afq_run_blocks": (c_int32, [POINTER(afq_problem), POINTER(afq_params), POINTER(afq_state), c_int32, c_uint64,
                                 P, P, P, P, c_size_t, P]),
    "afq_grad_tape_bytes": (c_size_t, [POINTER(afq_dims), c_int32, c_int32]),
    "afq_grad_workspace": (c_size_t, [POINTER(afq_dims), POINTER(afq_params), c_int32]),
    "afq_grad_forward": (c_int32, [POINTER(afq_problem), POINTER(afq_params), POINTER(afq_state), c_int32, c_uint64,
                                   c_uint64, c_int32, P, P, P, P, P, c_size_t, P, c_size_t, P]),
    "afq_grad_backward": (c_int32, [POINTER(afq_problem), POINTER(afq_params), P, c_int32, c_uint64, c_uint64,
                                    c_int32, P, c_size_t, P, P, P, P, c_size_t, P]),
    "afq_u_workspace": (c_size_t, [POINTER(afq_dims), c_int32]),
    "afq_overlap_u": (c_int32, [POINTER(afq_dims), P, P, P, P, c_size_t, P]),
    "afq_force_bias_u": (c_int32, [POINTER(afq_dims), P, P, P, P, P, c_size_t, P]),
    "afq_energy_u": (c_int32, [POINTER(afq_dims), c_double, P, P, P, P, P, P, c_size_t, P]),
    "afq_apply_trotter_u": (c_int32, [POINTER(afq_dims), c_int32, c_double, c_int32, P, P, P, P, P, P, c_size_t, P]),
    "afq_stochastic_reconfiguration_u": (c_int32, [POINTER(afq_dims), P, c_double, P, P, P, P, P, c_size_t, P]),
    "afq_step_u": (c_int32, [POINTER(afq_problem), POINTER(afq_params), POINTER(afq_state), P, c_uint64, c_uint64,
                             P, c_size_t, P]),
    "afq_block_u": (c_int32, [POINTER(afq_problem), POINTER(afq_params), POINTER(afq_state), P, c_double,
                              c_uint64, c_uint64, P, P, P, P, c_size_t, P]),
    "afq_g_workspace": (c_size_t, [POINTER(afq_dims), c_int32]),
    "afq_overlap_g": (c_int32, [POINTER(afq_dims), P, P, P, P, c_size_t, P]),
    "afq_force_bias_g": (c_int32, [POINTER(afq_dims), P, P, P, P, P, c_size_t, P]),
    "afq_apply_trotter_g": (c_int32, [POINTER(afq_dims), c_int32, c_double, c_int32, P, P, P, P, P, P, c_size_t, P]),
    "afq_modified_cholesky_workspace": (c_size_t, [c_int32, c_int32]),
    "afq_modified_cholesky": (c_int32, [c_int32, P, c_double, c_int32, P, POINTER(c_int32), P, c_size_t, P]),
    "afq_mlp_param_count": (c_size_t, [c_int32, c_int32]),
    "afq_mlp_forward": (c_int32, [c_int32, c_int32, c_int32, P, P, P, P]),
    "afq_mlp_train_workspace": (c_size_t, [c_int32, c_int32, c_int32]),
    "afq_mlp_gradient": (c_int32, [c_int32, c_int32, c_int32, P, P, P, P, P, P, c_size_t, P]),
    "afq_mlp_train_step": (c_int32, [c_int32, c_int32, c_int32, P, P, P, P, P, P, ctypes.c_float, c_int32, P,
                                     c_size_t, P, P]),
    "afq_mlp_sync": (c_int32, [c_int32, c_int32, P, P, P]),
    "afq_launch_count": (ctypes.c_longlong, []),
    "afq_timing_enable": (c_int32, [c_int32]),
    "afq_timing_report": (c_int32, [ctypes.c_char_p, c_size_t]),
    "afq_timing_reset": (c_int32, []),
    "afq_probe_fma_peak": (c_int32, [c_int32, POINTER(c_double)]),
}


def timing_report() -> dict:
    """{phase: (calls, total_ms)} accumulated since the last reset."""
    lib = load()
    buf = ctypes.create_string_buffer(1 << 16)
    check(lib.afq_timing_report(buf, len(buf)), "afq_timing_report")
    out = {}
    for line in buf.value.decode().splitlines():
        name, calls, ms = line.split()
        out[name] = (int(calls), float(ms))
    return out

_lib = None


class EngineError(RuntimeError):
    """A failure reported by the CUDA engine through its C ABI."""

    def __init__(self, status: int, func: str, message: str):
        super().__init__(f"{func} failed with status {status}: {message}")
        self.status = status


def load(path: str | None = None) -> ctypes.CDLL:
    """Loads (once) and returns the engine library; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(
            f"CUDA engine library not found at {p}; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` (there is no CPU fallback)")
    lib = ctypes.CDLL(p)
    for name, (res, args) in _SIGS.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def exported_symbols():
    return sorted(_SIGS)


def check(status: int, func: str):
    if status == AFQ_OK:
        return
    lib = load()
    msg = lib.afq_last_error().decode(errors="replace")
    if status in (AFQ_E_INVALID_ARGUMENT,):
        raise ValueError(f"{func}: {msg}")
    raise EngineError(status, func, msg)


def call(name: str, *args):
    f = getattr(load(), name)
    check(f(*args), name)
