"""Typed wrappers over the C ABI: device tensors in, device tensors out.

PyTorch supplies device memory, the current CUDA stream and the caller's
tensors; all arithmetic happens in libafqmc_gb300.so.  Scratch memory for
the hot calls comes from a per-device workspace arena that grows (outside
the C calls) when a larger problem arrives, so the C calls never allocate.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Optional

import numpy as np
import torch

from . import _lib
from ._lib import afq_dims, afq_params, afq_problem, afq_state

F64 = torch.float64
C128 = torch.complex128


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("the AFQMC engine needs a CUDA device (there is no CPU fallback)")


def device() -> torch.device:
    require_cuda()
    return torch.device("cuda", torch.cuda.current_device())


def stream_ptr() -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def as_device(x, dtype) -> torch.Tensor:
    """Host or device array -> contiguous device tensor of `dtype`."""
    dev = device()
    if isinstance(x, torch.Tensor):
        t = x
    else:
        t = torch.as_tensor(np.asarray(x))
    if t.is_complex() and not dtype.is_complex:
        raise ValueError("complex input where a real array is required")
    return t.to(device=dev, dtype=dtype).contiguous()


def ptr(t: Optional[torch.Tensor]) -> ctypes.c_void_p:
    if t is None:
        return ctypes.c_void_p(None)
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError("expected a contiguous tensor")
    return ctypes.c_void_p(t.data_ptr())


class _Arena:
    def __init__(self):
        self.buf: dict[int, torch.Tensor] = {}

    def get(self, nbytes: int) -> torch.Tensor:
        dev = torch.cuda.current_device()
        b = self.buf.get(dev)
        if b is None or b.numel() < nbytes:
            self.buf.pop(dev, None)
            b = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=dev)
            b[:256].zero_()  # the step / block status word lives at offset 0
            self.buf[dev] = b
        return b


_arena = _Arena()


def workspace(nbytes: int) -> tuple[ctypes.c_void_p, int]:
    b = _arena.get(nbytes)
    return ctypes.c_void_p(b.data_ptr()), b.numel()


def make_dims(n_walkers, norb, nocc, nchol, trial_is_real, precision=_lib.AFQ_PREC_FP64) -> afq_dims:
    return afq_dims(int(n_walkers), int(norb), int(nocc), int(nchol), int(bool(trial_is_real)),
                    int(precision))


def _check_walkers(w: torch.Tensor, norb: int, nocc: int) -> torch.Tensor:
    if w.dim() != 3 or w.shape[1] != norb or w.shape[2] != nocc:
        raise ValueError(f"walkers must be (n_walkers, {norb}, {nocc}); got {tuple(w.shape)}")
    return as_device(w, C128)


# ------------------------------------------------------------------ set-up


def build_prop_ctx(h0: float, h1: torch.Tensor, chol: torch.Tensor, rdm1: torch.Tensor, dt: float):
    """prop/chol_afqmc_ops.py:77-103.  Returns (exp_h1_half, mf_shifts, h0_prop)."""
    n, G = h1.shape[0], chol.shape[0]
    rdm1 = as_device(rdm1, C128)
    if rdm1.dim() == 3 and rdm1.shape[0] == 2:
        spin = 1
    elif rdm1.dim() == 2:
        spin = 0
    else:
        raise ValueError(f"rdm1 must be (2, n, n) or (n, n); got {tuple(rdm1.shape)}")
    if rdm1.shape[-1] != n or rdm1.shape[-2] != n:
        raise ValueError("rdm1 trailing dims must match h1")
    e = torch.empty((n, n), dtype=F64, device=h1.device)
    mf = torch.empty((G,), dtype=C128, device=h1.device)
    h0p = torch.empty((1,), dtype=C128, device=h1.device)
    lib = _lib.load()
    nb = lib.afq_build_prop_ctx_workspace(n, G)
    wsp, wsn = workspace(nb)
    _lib.call("afq_build_prop_ctx", n, G, float(h0), float(dt), ptr(h1), ptr(chol), ptr(rdm1), spin,
              ptr(e), ptr(mf), ptr(h0p), wsp, wsn, stream_ptr())
    return e, mf, h0p


def trial_rdm1(mo: torch.Tensor) -> torch.Tensor:
    """(2, n, n) complex128 [C C^H, C C^H] of the trial orbitals (n, o)."""
    mo = as_device(mo, C128)
    n, o = mo.shape
    out = torch.empty((2, n, n), dtype=C128, device=mo.device)
    _lib.call("afq_trial_rdm1", int(n), int(o), ptr(mo), ptr(out), stream_ptr())
    return out


def build_meas_ctx(h1: torch.Tensor, chol: torch.Tensor, mo: torch.Tensor, trial_is_real: bool):
    """meas/rhf.py:141-150.  Returns (rot_h1 (o,n) c128, rot_chol (G,o,n))."""
    n, o, G = h1.shape[0], mo.shape[1], chol.shape[0]
    rot_h1 = torch.empty((o, n), dtype=C128, device=h1.device)
    rot_chol = torch.empty((G, o, n), dtype=F64 if trial_is_real else C128, device=h1.device)
    _lib.call("afq_build_meas_ctx", n, o, G, ptr(h1), ptr(chol), ptr(mo), int(trial_is_real), ptr(rot_h1),
              ptr(rot_chol), stream_ptr())
    return rot_h1, rot_chol


# ---------------------------------------------------------- walker kernels


def overlap(walkers, mo: torch.Tensor, trial_is_real: bool) -> torch.Tensor:
    n, o = mo.shape
    w = _check_walkers(walkers, n, o)
    out = torch.empty((w.shape[0],), dtype=C128, device=w.device)
    d = make_dims(w.shape[0], n, o, 1, trial_is_real)
    _lib.call("afq_overlap", ctypes.byref(d), ptr(mo), ptr(w), ptr(out), stream_ptr())
    return out


def half_green(walkers, mo: torch.Tensor, trial_is_real: bool, with_overlap: bool = False):
    n, o = mo.shape
    w = _check_walkers(walkers, n, o)
    g = torch.empty((w.shape[0], o, n), dtype=C128, device=w.device)
    ov = torch.empty((w.shape[0],), dtype=C128, device=w.device) if with_overlap else None
    d = make_dims(w.shape[0], n, o, 1, trial_is_real)
    _lib.call("afq_half_green", ctypes.byref(d), ptr(mo), ptr(w), ptr(g), ptr(ov), stream_ptr())
    return (g, ov) if with_overlap else g


def force_bias(walkers, mo, rot_chol, trial_is_real: bool) -> torch.Tensor:
    n, o = mo.shape
    G = rot_chol.shape[0]
    w = _check_walkers(walkers, n, o)
    out = torch.empty((w.shape[0], G), dtype=C128, device=w.device)
    d = make_dims(w.shape[0], n, o, G, trial_is_real)
    lib = _lib.load()
    wsp, wsn = workspace(lib.afq_force_bias_workspace(ctypes.byref(d)))
    _lib.call("afq_force_bias", ctypes.byref(d), ptr(mo), ptr(rot_chol), ptr(w), ptr(out), wsp, wsn,
              stream_ptr())
    return out


def energy(walkers, h0: float, mo, rot_h1, rot_chol, trial_is_real: bool) -> torch.Tensor:
    n, o = mo.shape
    G = rot_chol.shape[0]
    w = _check_walkers(walkers, n, o)
    out = torch.empty((w.shape[0],), dtype=C128, device=w.device)
    d = make_dims(w.shape[0], n, o, G, trial_is_real)
    lib = _lib.load()
    wsp, wsn = workspace(lib.afq_energy_workspace(ctypes.byref(d)))
    _lib.call("afq_energy", ctypes.byref(d), float(h0), ptr(mo), ptr(rot_h1), ptr(rot_chol), ptr(w), ptr(out),
              wsp, wsn, stream_ptr())
    return out


def apply_trotter(walkers, shifted_fields, chol, exp_h1_half, sqrt_dt: float, n_terms: int,
                  n_chunks: int = 1, out: Optional[torch.Tensor] = None) -> torch.Tensor:
    G, n, _ = chol.shape
    if walkers.dim() != 3 or walkers.shape[1] != n:
        raise ValueError(f"walkers must be (n_walkers, {n}, nocc); got {tuple(walkers.shape)}")
    o = walkers.shape[2]
    w = as_device(walkers, C128)
    x = as_device(shifted_fields, C128)
    if x.shape != (w.shape[0], G):
        raise ValueError(f"fields must be ({w.shape[0]}, {G}); got {tuple(x.shape)}")
    if out is None:
        out = torch.empty_like(w)
    d = make_dims(w.shape[0], n, o, G, True)
    lib = _lib.load()
    wsp, wsn = workspace(lib.afq_apply_trotter_workspace(ctypes.byref(d), int(n_chunks)))
    _lib.call("afq_apply_trotter", ctypes.byref(d), int(n_terms), float(sqrt_dt), int(n_chunks), ptr(chol),
              ptr(exp_h1_half), ptr(w), ptr(x), ptr(out), wsp, wsn, stream_ptr())
    return out


def orthogonalize(walkers, out: Optional[torch.Tensor] = None, precision: int = _lib.AFQ_PREC_FP64):
    """Returns (Q, det_r) with diag(R) >= 0 (walkers.py:169-203); Householder
    for the FP64 precision, CholeskyQR2 for the mixed ones."""
    w = as_device(walkers, C128)
    if w.dim() != 3:
        raise ValueError("walkers must be (n_walkers, norb, nocc)")
    W, n, o = w.shape
    if out is None:
        out = torch.empty_like(w)
    det = torch.empty((W,), dtype=C128, device=w.device)
    d = make_dims(W, n, o, 1, True, precision)
    _lib.call("afq_orthogonalize", ctypes.byref(d), ptr(w), ptr(out), ptr(det), stream_ptr())
    return out, det


def sr_indices(weights, zeta: float):
    """Comb indices (int64) and the prefix sum of |w| (walkers.py:233-240)."""
    w = as_device(weights, F64)
    W = w.shape[0]
    idx = torch.empty((W,), dtype=torch.int32, device=w.device)
    cw = torch.empty((W,), dtype=F64, device=w.device)
    lib = _lib.load()
    wsp, wsn = workspace(lib.afq_sr_workspace(W))
    _lib.call("afq_sr_indices", W, ptr(w), float(zeta), ptr(idx), ptr(cw), wsp, wsn, stream_ptr())
    return idx.long(), cw


def stochastic_reconfiguration(walkers, weights, zeta: float):
    """walkers.py:243-265 (restricted): returns (walkers, weights, idx)."""
    w = as_device(walkers, C128)
    wt = as_device(weights, F64)
    W, n, o = w.shape
    out = torch.empty_like(w)
    wout = torch.empty_like(wt)
    idx = torch.empty((W,), dtype=torch.int32, device=w.device)
    d = make_dims(W, n, o, 1, True)
    lib = _lib.load()
    wsp, wsn = workspace(lib.afq_sr_workspace(W))
    _lib.call("afq_stochastic_reconfiguration", ctypes.byref(d), ptr(wt), float(zeta), ptr(w), ptr(out),
              ptr(wout), ptr(idx), wsp, wsn, stream_ptr())
    return out, wout, idx.long()


def fill_normal(shape, seed: int, counter: int) -> torch.Tensor:
    out = torch.empty(shape, dtype=F64, device=device())
    _lib.call("afq_fill_normal", out.numel(), int(seed) & (2**64 - 1), int(counter) & (2**64 - 1), ptr(out),
              stream_ptr())
    return out


def fill_uniform(shape, seed: int, counter: int) -> torch.Tensor:
    out = torch.empty(shape, dtype=F64, device=device())
    _lib.call("afq_fill_uniform", out.numel(), int(seed) & (2**64 - 1), int(counter) & (2**64 - 1), ptr(out),
              stream_ptr())
    return out


def field_shift(fields, force_bias_, mf_shifts, sqrt_dt: float):
    x = as_device(fields, F64)
    fb = as_device(force_bias_, C128)
    mf = as_device(mf_shifts, C128)
    W, G = x.shape
    if fb.shape != (W, G) or mf.shape != (G,):
        raise ValueError("field_shift: shape mismatch")
    xs = torch.empty((W, G), dtype=C128, device=x.device)
    st = torch.empty((W,), dtype=C128, device=x.device)
    ft = torch.empty((W,), dtype=C128, device=x.device)
    d = make_dims(W, 1, 1, G, True)
    _lib.call("afq_field_shift", ctypes.byref(d), float(sqrt_dt), ptr(x), ptr(fb), ptr(mf), ptr(xs), ptr(st),
              ptr(ft), stream_ptr())
    return xs, st, ft


@dataclass
class Problem:
    """Device views of Hamiltonian, trial and both contexts (afq_problem)."""
    n_walkers: int
    norb: int
    nocc: int
    nchol: int
    trial_is_real: bool
    h0: float
    chol: torch.Tensor
    mo: torch.Tensor
    dt: float
    sqrt_dt: float
    exp_h1_half: torch.Tensor
    mf_shifts: torch.Tensor
    h0_prop: complex
    rot_h1: torch.Tensor
    rot_chol: torch.Tensor
    precision: int = _lib.AFQ_PREC_FP64
    lowp: Optional[torch.Tensor] = None

    def c(self) -> afq_problem:
        return afq_problem(make_dims(self.n_walkers, self.norb, self.nocc, self.nchol, self.trial_is_real,
                                     self.precision),
                           float(self.h0), ptr(self.chol), ptr(self.mo), float(self.dt), float(self.sqrt_dt),
                           ptr(self.exp_h1_half), ptr(self.mf_shifts), float(self.h0_prop.real),
                           float(self.h0_prop.imag), ptr(self.rot_h1), ptr(self.rot_chol),
                           ptr(self.lowp) if self.lowp is not None else None)


def prepare_lowp(n_walkers: int, norb: int, nocc: int, nchol: int, chol: torch.Tensor,
                 rot_chol: torch.Tensor, precision: int = _lib.AFQ_PREC_MIXED) -> torch.Tensor:
    """bf16 split copies of chol and rot_chol in tensor-core operand order,
    for a mixed-precision step (real trial orbitals only); the layout depends
    on the precision (six or three sections)."""
    if rot_chol.is_complex():
        raise ValueError("the mixed-precision form supports real trial orbitals only")
    if precision not in (_lib.AFQ_PREC_MIXED, _lib.AFQ_PREC_MIXED_FAST):
        raise ValueError(f"precision {precision} has no low-precision operands")
    d = make_dims(n_walkers, norb, nocc, nchol, True, precision)
    lib = _lib.load()
    nb = int(lib.afq_lowp_bytes(ctypes.byref(d)))
    buf = torch.empty((nb,), dtype=torch.uint8, device=chol.device)
    _lib.call("afq_prepare_lowp", ctypes.byref(d), ptr(chol), ptr(rot_chol), ptr(buf), nb, stream_ptr())
    return buf


def workspace_status():
    """Reads and clears the device status word of the step / block workspace
    (synchronises the stream); raises EngineError if a bounded wait expired."""
    b = _arena.buf.get(torch.cuda.current_device())
    if b is None:
        return 0
    v = ctypes.c_int32(0)
    _lib.call("afq_workspace_status", ptr(b), ctypes.byref(v), stream_ptr())
    return v.value


def workspace_counters():
    """(status, nonfinite): the status word of the step / block workspace and
    the number of walker updates that produced a NaN or infinite overlap or
    weight since the last read; both are cleared (synchronises the stream).
    Does not raise on a set status."""
    b = _arena.buf.get(torch.cuda.current_device())
    if b is None:
        return 0, 0
    v, nf = ctypes.c_int32(0), ctypes.c_int32(0)
    _lib.load().afq_workspace_counters(ptr(b), ctypes.byref(v), ctypes.byref(nf), stream_ptr())
    return v.value, nf.value


def selftest_wait(limit_ns: int, arrive: bool) -> int:
    """Runs the bounded-wait self-test (afq_selftest_wait) and returns the
    device status it wrote: AFQ_STATUS_WAIT_EXPIRED when nothing arrived."""
    out = torch.full((1,), -1, dtype=torch.int32, device=device())
    _lib.call("afq_selftest_wait", int(limit_ns), 1 if arrive else 0, ptr(out), stream_ptr())
    return int(out.item())


def make_params(params, n_prop_steps: Optional[int] = None) -> afq_params:
    return afq_params(float(params.dt), float(params.pop_control_damping), float(params.weight_floor),
                      float(params.weight_cap), float(params.shift_ema), int(params.n_exp_terms),
                      int(params.n_prop_steps if n_prop_steps is None else n_prop_steps),
                      int(getattr(params, "qr_every", 0) or 0), int(params.n_chunks))


@dataclass
class DeviceState:
    walkers: torch.Tensor
    weights: torch.Tensor
    overlaps: torch.Tensor
    pop_shift: torch.Tensor  # (1,) f64
    e_estimate: torch.Tensor  # (1,) f64

    def c(self) -> afq_state:
        return afq_state(ptr(self.walkers), ptr(self.weights), ptr(self.overlaps), ptr(self.pop_shift),
                         ptr(self.e_estimate))


def block_measure(weights, energy_, e_estimate, pop_shift, dt: float, shift_ema: float):
    """prop/blocks.py:59-79; updates pop_shift ((1,) f64) in place, returns (E_blk, W_sum)."""
    W = weights.shape[0]
    e = torch.empty((1,), dtype=F64, device=weights.device)
    wsum = torch.empty((1,), dtype=F64, device=weights.device)
    _lib.call("afq_block_measure", int(W), float(dt), float(shift_ema), ptr(weights), ptr(energy_),
              ptr(e_estimate), ptr(pop_shift), ptr(e), ptr(wsum), stream_ptr())
    return e, wsum


def weight_update(prob: Problem, params, shift_term, fb_term, overlaps_new, st: DeviceState):
    d = make_dims(st.walkers.shape[0], prob.norb, prob.nocc, prob.nchol, prob.trial_is_real)
    p = make_params(params)
    pb = prob.c()
    cs = st.c()
    _lib.call("afq_weight_update", ctypes.byref(d), ctypes.byref(p), ctypes.byref(pb), ptr(shift_term),
              ptr(fb_term), ptr(overlaps_new), ctypes.byref(cs), stream_ptr())


def step(prob: Problem, params, st: DeviceState, seed: int, counter: int, fields=None):
    """One afqmc_step on `st`, in place."""
    if fields is not None:
        fields = as_device(fields, F64)
        if fields.shape != (st.walkers.shape[0], prob.nchol):
            raise ValueError("fields shape mismatch")
    d = make_dims(st.walkers.shape[0], prob.norb, prob.nocc, prob.nchol, prob.trial_is_real, prob.precision)
    lib = _lib.load()
    wsp, wsn = workspace(lib.afq_step_workspace(ctypes.byref(d), int(params.n_chunks)))
    p = make_params(params)
    pb = prob.c()
    cs = st.c()
    _lib.call("afq_step", ctypes.byref(pb), ctypes.byref(p), ctypes.byref(cs), ptr(fields),
              int(seed) & (2**64 - 1), int(counter) & (2**64 - 1), wsp, wsn, stream_ptr())


def block(prob: Problem, params, st: DeviceState, seed: int, counter: int, fields=None, zeta=None,
          return_idx: bool = False, cv=None):
    """One afqmc_block on `st`, in place.  Returns device (energy, weight[, idx]).
    cv: an `afq_cv` structure (the control-variate measurement), or None."""
    W = st.walkers.shape[0]
    if fields is not None:
        fields = as_device(fields, F64)
        if fields.shape != (params.n_prop_steps, W, prob.nchol):
            raise ValueError("fields must be (n_prop_steps, n_walkers, nchol)")
    d = make_dims(W, prob.norb, prob.nocc, prob.nchol, prob.trial_is_real, prob.precision)
    lib = _lib.load()
    wsp, wsn = workspace(lib.afq_block_workspace(ctypes.byref(d), int(params.n_chunks)))
    p = make_params(params)
    pb = prob.c()
    cs = st.c()
    e = torch.empty((1,), dtype=F64, device=st.walkers.device)
    wsum = torch.empty((1,), dtype=F64, device=st.walkers.device)
    idx = torch.empty((W,), dtype=torch.int32, device=st.walkers.device) if return_idx else None
    z = -1.0 if zeta is None else float(zeta)
    if zeta is not None and not (0.0 <= z < 1.0):
        raise ValueError("zeta must be in [0, 1)")
    if cv is None:
        _lib.call("afq_block", ctypes.byref(pb), ctypes.byref(p), ctypes.byref(cs), ptr(fields), z,
                  int(seed) & (2**64 - 1), int(counter) & (2**64 - 1), ptr(e), ptr(wsum), ptr(idx), wsp, wsn,
                  stream_ptr())
    else:
        _lib.call("afq_block_cv", ctypes.byref(pb), ctypes.byref(p), ctypes.byref(cs), ptr(fields), z,
                  int(seed) & (2**64 - 1), int(counter) & (2**64 - 1), ptr(e), ptr(wsum), ptr(idx),
                  ctypes.byref(cv), wsp, wsn, stream_ptr())
    if return_idx:
        return e, wsum, idx.long()
    return e, wsum


def run_blocks(prob: Problem, params, st: DeviceState, n_blocks: int, seed: int, counter):
    """n_blocks afqmc_blocks on `st` in place (driver.py:22-38), the block
    loop replayed as a CUDA graph.  `counter`: device (1,) int64 Philox
    counter, advanced by n_prop_steps + 1 per block.  Returns device
    (energies (n_blocks,), weights (n_blocks,))."""
    W = st.walkers.shape[0]
    if counter.dtype != torch.int64 or counter.numel() != 1 or not counter.is_cuda:
        raise ValueError("counter must be a device (1,) int64 tensor")
    d = make_dims(W, prob.norb, prob.nocc, prob.nchol, prob.trial_is_real, prob.precision)
    lib = _lib.load()
    wsp, wsn = workspace(lib.afq_run_blocks_workspace(ctypes.byref(d), int(params.n_chunks)))
    p = make_params(params)
    pb = prob.c()
    cs = st.c()
    e = torch.empty((max(n_blocks, 1),), dtype=F64, device=st.walkers.device)
    w = torch.empty_like(e)
    _lib.call("afq_run_blocks", ctypes.byref(pb), ctypes.byref(p), ctypes.byref(cs), int(n_blocks),
              int(seed) & (2**64 - 1), ptr(counter), ptr(e), ptr(w), wsp, wsn, stream_ptr())
    return e[:n_blocks], w[:n_blocks]


# ------------------------------------------------- unrestricted walkers
def as_pair(w) -> torch.Tensor:
    """(2, W, n, o) complex128 device tensor of a (w_up, w_dn) pair; no copy
    when the two are the halves of one such tensor (as as_pair returns and
    pair_views splits), else the two are stacked."""
    if isinstance(w, torch.Tensor):
        if w.dim() != 4 or w.shape[0] != 2:
            raise ValueError(f"unrestricted walkers must be (2, W, n, o) or a pair; got {tuple(w.shape)}")
        return as_device(w, C128)
    if not (isinstance(w, (tuple, list)) and len(w) == 2):
        raise ValueError("unrestricted walkers must be a pair (w_up, w_dn)")
    wu, wd = w
    if isinstance(wu, torch.Tensor) and isinstance(wd, torch.Tensor) and wu.is_cuda and wd.is_cuda:
        base = getattr(wu, "_base", None)
        if (base is not None and base is getattr(wd, "_base", None) and base.dim() == 4 and base.shape[0] == 2
                and base.dtype == C128 and base.is_contiguous() and wu.data_ptr() == base.data_ptr()
                and wd.data_ptr() == base[1].data_ptr()):
            return base
    wu, wd = as_device(wu, C128), as_device(wd, C128)
    if wu.shape != wd.shape:
        raise ValueError(f"up and down walkers differ in shape: {tuple(wu.shape)} vs {tuple(wd.shape)}")
    return torch.stack([wu, wd]).contiguous()


def pair_views(p: torch.Tensor):
    """(w_up, w_dn) views of a (2, W, n, o) tensor."""
    return p[0], p[1]


def _u_dims(p: torch.Tensor, nchol: int, trial_is_real: bool):
    return make_dims(p.shape[1], p.shape[2], p.shape[3], nchol, trial_is_real)


def _u_ws(d, n_chunks: int = 1):
    return workspace(_lib.load().afq_u_workspace(ctypes.byref(d), int(n_chunks)))


def overlap_u(walkers, mo: torch.Tensor, trial_is_real: bool) -> torch.Tensor:
    """det(C^H W_up) det(C^H W_dn) per pair (meas/rhf.py:53-57)."""
    p = as_pair(walkers)
    d = _u_dims(p, 1, trial_is_real)
    out = torch.empty((p.shape[1],), dtype=C128, device=p.device)
    wsp, wsn = _u_ws(d)
    _lib.call("afq_overlap_u", ctypes.byref(d), ptr(mo), ptr(p), ptr(out), wsp, wsn, stream_ptr())
    return out


def force_bias_u(walkers, mo, rot_chol, trial_is_real: bool) -> torch.Tensor:
    """L~_flat vec(G_up + G_dn) per pair (meas/rhf.py:60-72)."""
    p = as_pair(walkers)
    d = _u_dims(p, rot_chol.shape[0], trial_is_real)
    out = torch.empty((p.shape[1], rot_chol.shape[0]), dtype=C128, device=p.device)
    wsp, wsn = _u_ws(d)
    _lib.call("afq_force_bias_u", ctypes.byref(d), ptr(mo), ptr(rot_chol), ptr(p), ptr(out), wsp, wsn,
              stream_ptr())
    return out


def energy_u(walkers, h0: float, mo, rot_h1, rot_chol, trial_is_real: bool) -> torch.Tensor:
    """Local energy of each pair (meas/rhf.py:75-100)."""
    p = as_pair(walkers)
    d = _u_dims(p, rot_chol.shape[0], trial_is_real)
    out = torch.empty((p.shape[1],), dtype=C128, device=p.device)
    wsp, wsn = _u_ws(d)
    _lib.call("afq_energy_u", ctypes.byref(d), float(h0), ptr(mo), ptr(rot_h1), ptr(rot_chol), ptr(p), ptr(out),
              wsp, wsn, stream_ptr())
    return out


def apply_trotter_u(walkers, shifted_fields, chol, exp_h1_half, sqrt_dt: float, n_terms: int,
                    n_chunks: int = 1) -> torch.Tensor:
    """Both spins propagated with the same V (prop/chol_afqmc_ops.py:118-183);
    returns a new (2, W, n, o) tensor."""
    p = as_pair(walkers)
    xs = as_device(shifted_fields, C128)
    d = _u_dims(p, chol.shape[0], True)
    out = torch.empty_like(p)
    wsp, wsn = _u_ws(d, n_chunks)
    _lib.call("afq_apply_trotter_u", ctypes.byref(d), int(n_terms), float(sqrt_dt), int(n_chunks), ptr(chol),
              ptr(exp_h1_half), ptr(p), ptr(xs), ptr(out), wsp, wsn, stream_ptr())
    return out


def stochastic_reconfiguration_u(walkers, weights, zeta: float):
    """Comb with one set of indices for both spins (walkers.py:243-265).
    Returns ((2, W, n, o), weights, idx)."""
    p = as_pair(walkers)
    w = as_device(weights, F64)
    d = _u_dims(p, 1, True)
    out = torch.empty_like(p)
    wout = torch.empty_like(w)
    idx = torch.empty((p.shape[1],), dtype=torch.int32, device=p.device)
    wsp, wsn = _u_ws(d)
    _lib.call("afq_stochastic_reconfiguration_u", ctypes.byref(d), ptr(w), float(zeta), ptr(p), ptr(out),
              ptr(wout), ptr(idx), wsp, wsn, stream_ptr())
    return out, wout, idx


def step_u(prob: Problem, params, st: DeviceState, seed: int, counter: int, fields=None):
    """One afqmc_step of unrestricted walkers (st.walkers (2, W, n, o)), in place."""
    W = st.walkers.shape[1]
    if fields is not None:
        fields = as_device(fields, F64)
        if fields.shape != (W, prob.nchol):
            raise ValueError("fields shape mismatch")
    pb = prob.c()
    p = make_params(params)
    wsp, wsn = _u_ws(pb.dims, int(params.n_chunks))
    cs = st.c()
    _lib.call("afq_step_u", ctypes.byref(pb), ctypes.byref(p), ctypes.byref(cs), ptr(fields),
              int(seed) & (2**64 - 1), int(counter) & (2**64 - 1), wsp, wsn, stream_ptr())


def block_u(prob: Problem, params, st: DeviceState, seed: int, counter: int, fields=None, zeta=None,
            return_idx: bool = False):
    """One afqmc_block of unrestricted walkers, in place.  Returns device
    (energy, weight[, idx])."""
    W = st.walkers.shape[1]
    if fields is not None:
        fields = as_device(fields, F64)
        if fields.shape != (params.n_prop_steps, W, prob.nchol):
            raise ValueError("fields must be (n_prop_steps, n_walkers, nchol)")
    pb = prob.c()
    p = make_params(params)
    wsp, wsn = _u_ws(pb.dims, int(params.n_chunks))
    cs = st.c()
    e = torch.empty((1,), dtype=F64, device=st.walkers.device)
    wsum = torch.empty((1,), dtype=F64, device=st.walkers.device)
    idx = torch.empty((W,), dtype=torch.int32, device=st.walkers.device) if return_idx else None
    z = -1.0 if zeta is None else float(zeta)
    if zeta is not None and not (0.0 <= z < 1.0):
        raise ValueError("zeta must be in [0, 1)")
    _lib.call("afq_block_u", ctypes.byref(pb), ctypes.byref(p), ctypes.byref(cs), ptr(fields), z,
              int(seed) & (2**64 - 1), int(counter) & (2**64 - 1), ptr(e), ptr(wsum), ptr(idx), wsp, wsn,
              stream_ptr())
    if return_idx:
        return e, wsum, idx.long()
    return e, wsum


# ------------------------------------------------- generalized walkers
def _g_dims(w: torch.Tensor, mo: torch.Tensor, nchol: int, trial_is_real: bool):
    n, o = mo.shape
    if w.dim() != 3 or w.shape[1] != 2 * n or w.shape[2] != 2 * o:
        raise ValueError(f"generalized walkers must be (W, {2 * n}, {2 * o}); got {tuple(w.shape)}")
    return make_dims(w.shape[0], n, o, nchol, trial_is_real)


def _g_ws(d, n_chunks: int = 1):
    return workspace(_lib.load().afq_g_workspace(ctypes.byref(d), int(n_chunks)))


def overlap_g(walkers, mo: torch.Tensor, trial_is_real: bool) -> torch.Tensor:
    """det(vstack(C^H W_top, C^H W_bot)) per walker (meas/rhf.py:103-109)."""
    w = as_device(walkers, C128)
    d = _g_dims(w, mo, 1, trial_is_real)
    out = torch.empty((w.shape[0],), dtype=C128, device=w.device)
    wsp, wsn = _g_ws(d)
    _lib.call("afq_overlap_g", ctypes.byref(d), ptr(mo), ptr(w), ptr(out), wsp, wsn, stream_ptr())
    return out


def force_bias_g(walkers, mo, rot_chol, trial_is_real: bool) -> torch.Tensor:
    """L~_flat vec(G_uu + G_dd) per walker (meas/rhf.py:112-130)."""
    w = as_device(walkers, C128)
    d = _g_dims(w, mo, rot_chol.shape[0], trial_is_real)
    out = torch.empty((w.shape[0], rot_chol.shape[0]), dtype=C128, device=w.device)
    wsp, wsn = _g_ws(d)
    _lib.call("afq_force_bias_g", ctypes.byref(d), ptr(mo), ptr(rot_chol), ptr(w), ptr(out), wsp, wsn,
              stream_ptr())
    return out


def apply_trotter_g(walkers, shifted_fields, chol, exp_h1_half, sqrt_dt: float, n_terms: int,
                    n_chunks: int = 1) -> torch.Tensor:
    """Both halves of each (2n, 2o) walker with its V (prop/chol_afqmc_ops.py:141-197)."""
    w = as_device(walkers, C128)
    xs = as_device(shifted_fields, C128)
    n = int(chol.shape[1])
    if w.dim() != 3 or w.shape[1] != 2 * n or w.shape[2] % 2:
        raise ValueError(f"generalized walkers must be (W, {2 * n}, 2 nocc); got {tuple(w.shape)}")
    d = make_dims(w.shape[0], n, w.shape[2] // 2, chol.shape[0], True)
    out = torch.empty_like(w)
    wsp, wsn = _g_ws(d, n_chunks)
    _lib.call("afq_apply_trotter_g", ctypes.byref(d), int(n_terms), float(sqrt_dt), int(n_chunks), ptr(chol),
              ptr(exp_h1_half), ptr(w), ptr(xs), ptr(out), wsp, wsn, stream_ptr())
    return out


# ------------------------------------------------- differentiated energy
def grad_forward(prob: Problem, params, st: DeviceState, n_blocks: int, seed: int, counter: int,
                 checkpoint_blocks: int, sr_fixed: Optional[torch.Tensor] = None):
    """n_blocks binary64 blocks on `st` in place with the tape kept for
    grad_backward.  Returns device (energies (B,), weights (B,), comb
    indices (B, W) int32, tape)."""
    W = st.walkers.shape[0]
    d = make_dims(W, prob.norb, prob.nocc, prob.nchol, prob.trial_is_real, prob.precision)
    p = make_params(params)
    lib = _lib.load()
    tb = int(lib.afq_grad_tape_bytes(ctypes.byref(d), int(n_blocks), int(checkpoint_blocks)))
    tape = torch.empty((max(tb, 256),), dtype=torch.uint8, device=st.walkers.device)
    wsp, wsn = workspace(lib.afq_grad_workspace(ctypes.byref(d), ctypes.byref(p), 0))
    if sr_fixed is not None:
        sr_fixed = sr_fixed.to(device=st.walkers.device, dtype=torch.int32).contiguous()
        if sr_fixed.shape != (n_blocks, W):
            raise ValueError(f"sr_fixed must be (n_blocks, n_walkers) = ({n_blocks}, {W})")
    e = torch.empty((n_blocks,), dtype=F64, device=st.walkers.device)
    w = torch.empty_like(e)
    idx = torch.empty((n_blocks, W), dtype=torch.int32, device=st.walkers.device)
    pb = prob.c()
    cs = st.c()
    _lib.call("afq_grad_forward", ctypes.byref(pb), ctypes.byref(p), ctypes.byref(cs), int(n_blocks),
              int(seed) & (2**64 - 1), int(counter) & (2**64 - 1), int(checkpoint_blocks), ptr(sr_fixed), ptr(e),
              ptr(w), ptr(idx), ptr(tape), tape.numel(), wsp, wsn, stream_ptr())
    return e, w, idx, tape


def grad_backward(prob: Problem, params, h1: torch.Tensor, n_blocks: int, seed: int, counter: int,
                  checkpoint_blocks: int, tape: torch.Tensor, energies_bar: torch.Tensor,
                  weights_bar: torch.Tensor) -> torch.Tensor:
    """dL/dh1 (n, n) from dL/de_b and dL/dW_b of the run grad_forward taped."""
    d = make_dims(prob.n_walkers, prob.norb, prob.nocc, prob.nchol, prob.trial_is_real, prob.precision)
    p = make_params(params)
    lib = _lib.load()
    wsp, wsn = workspace(lib.afq_grad_workspace(ctypes.byref(d), ctypes.byref(p), int(checkpoint_blocks)))
    eb = as_device(energies_bar, F64)
    wb = as_device(weights_bar, F64)
    if eb.shape != (n_blocks,) or wb.shape != (n_blocks,):
        raise ValueError("energies_bar and weights_bar must be (n_blocks,)")
    h1 = as_device(h1, F64)
    out = torch.empty((prob.norb, prob.norb), dtype=F64, device=h1.device)
    pb = prob.c()
    _lib.call("afq_grad_backward", ctypes.byref(pb), ctypes.byref(p), ptr(h1), int(n_blocks),
              int(seed) & (2**64 - 1), int(counter) & (2**64 - 1), int(checkpoint_blocks), ptr(tape), tape.numel(),
              ptr(eb), ptr(wb), ptr(out), wsp, wsn, stream_ptr())
    return out


# ------------------------------------------------------------- the network
def mlp_param_count(n_features: int, hidden: int) -> int:
    n = int(_lib.load().afq_mlp_param_count(int(n_features), int(hidden)))
    if n == 0:
        raise ValueError(f"network shape F={n_features} H={hidden} (F a multiple of 16, H a multiple of 32, <= 256)")
    return n


def mlp_forward(params_bf16: torch.Tensor, x: torch.Tensor, hidden: int) -> torch.Tensor:
    """y (B,) fp32 = network(x (B, F) fp32) with the bf16 parameters."""
    x = x.to(torch.float32).contiguous()
    B, F = x.shape
    y = torch.empty((B,), dtype=torch.float32, device=x.device)
    _lib.call("afq_mlp_forward", int(B), int(F), int(hidden), ptr(params_bf16), ptr(x), ptr(y), stream_ptr())
    return y


def mlp_sync(master: torch.Tensor, params_bf16: torch.Tensor, n_features: int, hidden: int):
    _lib.call("afq_mlp_sync", int(n_features), int(hidden), ptr(master), ptr(params_bf16), stream_ptr())


def mlp_gradient(params_bf16, x, target, hidden: int, ws=None):
    """(gradient (P,) fp32, loss (1,), workspace) of mean (y - t)^2 / 2 at the bf16 parameters."""
    x = x.to(torch.float32).contiguous()
    target = target.to(torch.float32).contiguous()
    B, F = x.shape
    need = int(_lib.load().afq_mlp_train_workspace(int(B), int(F), int(hidden)))
    if ws is None or ws.numel() * 4 < need:
        ws = torch.empty((need + 3) // 4, dtype=torch.float32, device=x.device)
    g = torch.empty((mlp_param_count(F, hidden),), dtype=torch.float32, device=x.device)
    loss = torch.empty((1,), dtype=torch.float32, device=x.device)
    _lib.call("afq_mlp_gradient", int(B), int(F), int(hidden), ptr(params_bf16), ptr(x), ptr(target), ptr(g),
              ptr(loss), ptr(ws), ws.numel() * 4, stream_ptr())
    return g, loss, ws


def mlp_train_step(master, params_bf16, m, v, x, target, lr: float, step: int, hidden: int, ws=None,
                   loss_out=None):
    """One Adam step on a batch; returns (device loss (1,), workspace tensor).
    loss_out: a device float32 slot for the loss (default: a new tensor)."""
    x = x.to(torch.float32).contiguous()
    target = target.to(torch.float32).contiguous()
    B, F = x.shape
    need = int(_lib.load().afq_mlp_train_workspace(int(B), int(F), int(hidden)))
    if ws is None or ws.numel() * 4 < need:
        ws = torch.empty((need + 3) // 4, dtype=torch.float32, device=x.device)
    loss = torch.empty((1,), dtype=torch.float32, device=x.device) if loss_out is None else loss_out
    _lib.call("afq_mlp_train_step", int(B), int(F), int(hidden), ptr(master), ptr(params_bf16), ptr(m), ptr(v),
              ptr(x), ptr(target), float(lr), int(step), ptr(ws), ws.numel() * 4, ptr(loss), stream_ptr())
    return loss, ws
