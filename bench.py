"""Throughput benchmark of the AFQMC block on GB300.

One bench step = one AFQMC block of the benchmark workload: 10 propagation
steps with a QR after step 5, then QR, mixed energy, shift update and comb
reconfiguration (QR every 5 steps, energy and comb every 10).  The metric is
walker-steps/s = n_walkers * 10 / (seconds per block), summed over ranks.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--precision fp64|mixed] [--workload NAME]

--impl reference times the CPU restatement of the reference's algorithm
(the JAX reference cannot be installed here) on the host cores.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "walker-steps/s at |ΔE|≤0.1 mHa vs FP64 oracle: chosen form vs plain FP64 GPU"
UNIT = "walker-steps/s"
STEPS_PER_BLOCK = 10
QR_EVERY = 5
# bf16 sections of a split tensor-core operand row, per precision (split_sections in the CUDA sources)
SPLIT_SECTIONS = {"mixed": 6, "mixed_fast": 3}
# DRAM bytes (read + write) per launch of a kernel, from one ncu capture of this bench's own command
# (profiles/launches_block_c4_n200_o30_g1000_w4096_mixed_fast.md), keyed by (workload, precision,
# walkers, phase); the roofline reports them beside the algorithmic bytes
MEASURED_TRAFFIC = {("c4_n200_o30_g1000_w4096", "mixed_fast", 4096, "vbuild_gemm"): 564473600 + 1283924736,
                    ("c4_n200_o30_g1000_w4096", "mixed_fast", 4096, "trotter"): 1741291520 + 368705536,
                    ("c4_n200_o30_g1000_w4096", "mixed_fast", 4096, "fb_gemm"): 368115712 + 19635200}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed_fast", choices=["fp64", "mixed", "mixed_fast"])
    ap.add_argument("--workload", default="c4_n200_o30_g1000_w4096")
    ap.add_argument("--walkers", type=int, default=0, help="override the workload's walker count")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="budget of the CPU baseline sample")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-e2e-numa", dest="e2e_numa", action="store_false",
                    help="leave the process affinity alone for the end-to-end line")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip the plain-FP64 comparison block")
    ap.add_argument("--no-cv", action="store_true", help="skip the control-variate line")
    ap.add_argument("--no-grad", action="store_true", help="skip the differentiated-energy line")
    ap.add_argument("--grad-only", action="store_true",
                    help="print only the differentiated-energy measurement (60-orbital workload)")
    ap.add_argument("--grad-blocks", type=int, default=20, help="blocks of the differentiated run")
    ap.add_argument("--no-large", action="store_true", help="skip the 400-orbital workload line")
    return ap.parse_args()


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return None


# ----------------------------------------------------------------- clocks ---
class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------- algorithmic work model ---
def _r64(x):
    return (x + 63) // 64 * 64


def phase_work(n, o, G, W, trial_real=True, precision="fp64", n_terms=6):
    """(work per launch, pipe) of each timed phase.  FP64 form: algorithmic
    real flops.  Mixed forms: the tensor-core phases count the flops of the
    bf16 split operands (2 M N K with K the split row length; the energy GEMM
    without the padding of its exchange-fused layout; the Taylor kernel's
    128 x N x 16 MMAs, N = norb rounded up to 16, two a K step (V's hi and mid
    pieces) over K = 2 N per V product and N per E - I product: 256 (4
    n_terms + 4) N^2 per walker), the exchange step the bytes it must read.  The overlap
    and Green's-function phases of the mixed forms form m = C^T W on the tensor
    cores from integer digit slices and run the LU, the inverse and G_half on
    the fp32 pipe; they and the QR (double-float arithmetic) are "df32": their
    algorithmic flops are taken against the fp32 SIMT peak."""
    cm = 4 if trial_real else 8  # complex x real vs complex x complex multiply-add
    work = {
        "vbuild_gemm": (4.0 * G * n * n * W, "fp64"),
        "trotter": ((48.0 + 8.0) * n * n * o * W, "fp64"),
        "fb_gemm": (cm * G * o * n * W, "fp64"),
        "green": ((cm * o * o * n + 16.0 * o ** 3 + 8.0 * n * o * o) * W, "fp64"),
        "overlap": ((cm * o * o * n + 16.0 * o ** 3) * W, "fp64"),
        "energy": ((cm * G * o * o * n + 8.0 * G * o * o) * W, "fp64"),
        "qr": ((32.0 * n * o * o - 10.7 * o ** 3) * W, "fp64"),
    }
    if precision in SPLIT_SECTIONS:
        ks = SPLIT_SECTIONS[precision]
        work["vbuild_gemm"] = (2.0 * (2 * W) * n * n * _r64(ks * G), "tensor")
        work["fb_gemm"] = (2.0 * (2 * W) * G * _r64(ks * o * n), "tensor")
        del work["energy"]  # composite phase: e_green_rows + e_gemm + e_exchange
        work["e_gemm"] = (2.0 * (G * o) * (2 * o * W) * _r64(ks * n), "tensor")
        if 24 < o <= 32:  # exchange contracted in the GEMM's epilogue: the finish reads its fp32 sums
            work["e_exchange"] = (4.0 * W * (2 * 2 * ((32 * G + 127) // 128) + 2 * G), "hbm")
        else:  # the reduction reads F (G o x 2 o W fp32)
            work["e_exchange"] = (4.0 * (2 * o * W) * (G * o), "hbm")
        work["trotter"] = ((48.0 + 8.0) * n * n * o * W, "fp32")
        if precision == "mixed_fast" and n % 8 == 0 and n <= 256 and o <= 32:  # tensor-core Taylor products
            nn = (n + 15) // 16 * 16
            work["trotter"] = (256.0 * (4 * n_terms + 4) * nn * nn * W, "tensor")
        for k in ("overlap", "green", "qr"):
            work[k] = (work[k][0], "df32")
    return work


def algorithmic_work(n, o, G, W, trial_real=True, n_terms=6):
    """Algorithmic work per logical call over all walkers: the real-flop
    counts of the reference's formulas (complex x real multiply-add = 4,
    complex x complex = 8), whatever precision form executes them -- the
    three-section bf16 products execute 3x these flops on the tensor cores,
    the double-float phases ~10 fp32 instructions per flop.  Per walker:
    V-build 4 G n^2, Taylor + E_half products (8 n_terms + 8) n^2 o, force
    bias 4 G o n, m = C^H W with its LU cm o^2 n + 16 o^3 (+ 8 n o^2 for
    G_half), energy cm G o^2 n + 8 G o^2, QR 32 n o^2 - 10.7 o^3.  The
    exchange finish is counted in bytes (it reads the GEMM's sums)."""
    cm = 4 if trial_real else 8
    e_total = (cm * G * o * o * n + 8.0 * G * o * o) * W
    return {
        "vbuild_gemm": 4.0 * G * n * n * W,
        "trotter": (8.0 * n_terms + 8.0) * n * n * o * W,
        "fb_gemm": cm * G * o * n * W,
        "green": (cm * o * o * n + 16.0 * o ** 3 + 8.0 * n * o * o) * W,
        "overlap": (cm * o * o * n + 16.0 * o ** 3) * W,
        "energy": e_total,
        "e_gemm": e_total,
        "qr": (32.0 * n * o * o - 10.7 * o ** 3) * W,
    }


def _peak_for(pipe, lib):
    peaks = load_peaks() or {}
    if pipe == "hbm":
        peak = peaks.get("hbm_gbs")
        return (peak, "MEASURED_PEAKS.json hbm_gbs") if peak else (6800.0, "fallback (no MEASURED_PEAKS.json)")
    if pipe == "tensor":
        peak = peaks.get("bf16_tflops_sustained") or peaks.get("bf16_tflops")
        if peak:
            return peak, "MEASURED_PEAKS.json bf16_tflops_sustained (kernel timed inside a long step)"
        return 1700.0, "fallback (no MEASURED_PEAKS.json)"
    return fma_peak(lib, pipe == "fp64")  # SIMT fp64, or fp32 for the fp32 and double-float phases


def roofline_for(phases, work, lib, steps, name=None, alg=None):
    """Roofline object of phase `name`, or of the phase with the largest
    device time (composite phases that enclose timed sub-phases are not
    candidates).  work[] is (executed work, pipe) per logical call over all
    walkers, alg[] the algorithmic work of the same call (algorithmic_work);
    phases that launch once per walker chunk make several launches per
    call, so achieved = algorithmic work x calls per block / device time per
    block.  For the split-operand tensor phases the executed rate and
    fraction are reported beside it.  The double-float phases (overlap,
    Green's function, QR of the mixed forms) are measured against the fp32
    SIMT pipe they run on."""
    leaf = {k: v for k, v in phases.items() if not (k == "energy" and "e_gemm" in phases)}
    cand = {k: v for k, v in leaf.items() if k in work}
    if not cand:
        return None
    dname = name or max(cand.items(), key=lambda kv: kv[1][1])[0]
    if dname not in work or dname not in phases:
        return None
    dcalls, dms = phases[dname]
    executed, pipe = work[dname]
    algo = (alg or {}).get(dname, executed)
    chunked = {"vbuild_gemm": STEPS_PER_BLOCK, "trotter": STEPS_PER_BLOCK, "e_gemm": 1, "e_exchange": 1,
               "e_green_rows": 1, "energy": 1}
    mult = chunked.get(dname, dcalls / steps)
    ms_block = dms / steps
    common = {"kernel": dname, "traffic": None, "avg_launch_ms": round(dms / dcalls, 4),
              "launches_per_step": round(dcalls / steps, 2),
              "share_of_step": round(dms / sum(v[1] for v in leaf.values()), 4)}
    ppipe = "fp32" if pipe == "df32" else pipe
    peak, src = _peak_for(ppipe, lib)
    if pipe == "hbm":
        achieved = algo * mult / (ms_block / 1000.0) / 1e9
        return {**common, "bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": src, "work": "algorithmic bytes"}
    achieved = algo * mult / (ms_block / 1000.0) / 1e12
    out = {**common, "bound": ppipe, "achieved": round(achieved, 4), "peak": peak, "unit": "TFLOP/s",
           "frac": round(achieved / peak, 4) if peak else None, "peak_source": src,
           "work": "algorithmic flops (the reference's formulas, FP64-counted)"}
    if pipe == "df32" and dname in ("overlap", "green"):
        out["executed"] = ("m = C^T W as exact bf16 digit products on the tensor cores; LU (double-float) "
                           "and inverse, G_half (fp32) on the fp32 pipe")
    elif pipe == "df32":
        out["executed"] = "double-float (fp32 pairs) arithmetic on the fp32 pipe, ~10 instructions per flop"
    elif executed != algo:
        ex = executed * mult / (ms_block / 1000.0) / 1e12
        out.update(executed_achieved=round(ex, 4), executed_frac=round(ex / peak, 4) if peak else None,
                   executed="bf16 split-operand products the tensor cores execute (%.2fx the algorithmic flops)"
                            % (executed / algo))
    return out


# ------------------------------------------------------------ our engine ---
def make_engine_state(wl, W, precision):
    import torch
    from ad_afqmc_prototype_gb300 import synth
    from ad_afqmc_prototype_gb300.core.system import system
    from ad_afqmc_prototype_gb300.ham.chol import ham_chol
    from ad_afqmc_prototype_gb300.meas.rhf import make_rhf_meas_ops
    from ad_afqmc_prototype_gb300.prop.afqmc import engine_problem, init_prop_state
    from ad_afqmc_prototype_gb300.prop.chol_afqmc_ops import make_chol_afqmc_ops
    from ad_afqmc_prototype_gb300.prop.types import afqmc_params
    from ad_afqmc_prototype_gb300.trial.rhf import get_rdm1, make_rhf_trial_ops, rhf_trial

    H = synth.make_workload(wl)
    n, o = wl.nbasis, wl.nocc
    sys_ = system(norb=n, nelec=(o, o), walker_kind="restricted")
    ham = ham_chol(h0=H["h0"], h1=H["h1"], chol=H["chol"])
    trial = rhf_trial(H["mo_coeff"])
    t_ops, m_ops = make_rhf_trial_ops(sys_), make_rhf_meas_ops(sys_)
    p_ops = make_chol_afqmc_ops(ham, "restricted")
    params = afqmc_params(dt=0.005, n_prop_steps=STEPS_PER_BLOCK, qr_every=QR_EVERY, n_walkers=W, seed=2024,
                          precision=precision)
    pctx = p_ops.build_prop_ctx(get_rdm1(trial), params.dt)
    mctx = m_ops.build_meas_ctx(ham, trial)
    state = init_prop_state(sys=sys_, n_walkers=W, seed=params.seed, ham_data=ham, trial_ops_=t_ops,
                            trial_data=trial, meas_ops=m_ops,
                            initial_walkers=synth.trial_walkers(H["mo_coeff"], W))
    kw = dict(params=params, ham_data=ham, trial_data=trial, meas_ops=m_ops, prop_ops=p_ops, prop_ctx=pctx,
              meas_ctx=mctx)
    prob = engine_problem(n_walkers=W, need_energy=True, **kw)
    torch.cuda.synchronize()
    return dict(H=H, sys=sys_, kw=kw, prob=prob, state=state, params=params)


def run_ours(args, rank, world):
    import torch
    import torch.distributed as dist
    from ad_afqmc_prototype_gb300 import _lib, engine, synth
    from ad_afqmc_prototype_gb300.prop.afqmc import device_state
    from ad_afqmc_prototype_gb300.prop.blocks import afqmc_block

    wl = synth.WORKLOADS[args.workload]
    W = args.walkers or wl.n_walkers
    n, o, G = wl.nbasis, wl.nocc, wl.nchol
    env = make_engine_state(wl, W, args.precision)
    prob, params = env["prob"], env["params"]
    st = device_state(env["state"], inplace=True)
    lib = _lib.load()
    seed = 1000 + rank
    ctr = 0

    def one_block():
        nonlocal ctr
        engine.block(prob, params, st, seed, ctr)
        ctr += STEPS_PER_BLOCK + 1

    for _ in range(args.warmup):
        one_block()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(torch.cuda.current_device())
    clocks.start()
    lib.afq_timing_reset()
    lib.afq_timing_enable(1)
    launches0 = lib.afq_launch_count()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        one_block()
    e1.record(stream)
    torch.cuda.synchronize()
    launches = lib.afq_launch_count() - launches0
    lib.afq_timing_enable(0)
    phases = _lib.timing_report()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    if world > 1:
        t = torch.tensor([ms], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        dist.barrier()
    value = world * W * STEPS_PER_BLOCK / (ms / 1000.0)

    # dominant kernel and its roofline
    work = phase_work(n, o, G, W, trial_real=prob.trial_is_real, precision=args.precision)
    alg = algorithmic_work(n, o, G, W, trial_real=prob.trial_is_real)
    roof = roofline_for(phases, work, lib, args.steps, alg=alg)
    leaf = {k: v for k, v in phases.items() if not (k == "energy" and "e_gemm" in phases)}
    top = max(leaf.items(), key=lambda kv: kv[1][1])[0]
    dominant = {"phase": top, "share_of_step": round(leaf[top][1] / sum(v[1] for v in leaf.values()), 4),
                "pipe": work[top][1] if top in work else None}
    if roof is not None:
        t = MEASURED_TRAFFIC.get((args.workload, args.precision, W, roof["kernel"]))
        if t is not None:
            roof["traffic"] = t
            roof["traffic_source"] = "ncu dram__bytes_read.sum + dram__bytes_write.sum, one full-size launch"
            if roof["kernel"] == "vbuild_gemm" and args.precision in SPLIT_SECTIONS:
                ks = SPLIT_SECTIONS[args.precision]
                # split x~ and chol^T rows (bf16) read, V written (bf16 hi + mid, or fp32): 8 W n^2 bytes
                roof["traffic_algorithmic"] = int(2 * (2 * W) * _r64(ks * G) + 2 * n * n * _r64(ks * G)
                                                  + 8 * W * n * n)
            if roof["kernel"] == "trotter":
                # V hi + mid of every walker read once (2 planes x n^2 x 2 pieces x 2 bytes), walkers read
                # and written in binary64 (16 n o bytes each way)
                roof["traffic_algorithmic"] = int(W * (8 * n * n + 32 * n * o))
    tc = {k: roofline_for(phases, work, lib, args.steps, name=k, alg=alg) for k in phases
          if k in work and k != roof["kernel"]} if roof else {}
    for k, r in tc.items():
        t = MEASURED_TRAFFIC.get((args.workload, args.precision, W, k))
        if r is not None and t is not None:
            r["traffic"] = t

    compare = oracle_cmp = None
    if args.precision in SPLIT_SECTIONS and not args.no_fp64:
        compare = compare_with_fp64(env, st, W)
        oracle_cmp = compare_with_oracle(wl, args.precision, st)

    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, env, afqmc_block, W)

    cvline = None
    if args.precision in SPLIT_SECTIONS and not args.no_cv:
        cvline = run_cv(args, env, st, W, world, seed, ctr)

    out = {"metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else
           ("bf16x3" if args.precision == "mixed" else "bf16x2") + "/f32+f64",
           "data": "synthetic (seeded Cholesky Hamiltonian, see ad_afqmc_prototype_gb300/synth.py)",
           "config": {"workload": args.workload, "norb": n, "nocc": o, "nchol": G, "n_walkers_per_gpu": W,
                      "precision": args.precision, "parallelism": f"replicas{world}",
                      "step": "one block: 10 propagation steps, QR after step 5, QR + energy + comb at the end",
                      "l2": "inputs larger than L2 (walkers %d MB, V %d MB per step)"
                            % (W * n * o * 16 >> 20, W * n * n * 16 >> 20),
                      "synthetic": {"seed": wl.seed, "chol_scale": env["H"]["scale"], "chol_decay": env["H"]["decay"],
                                    "rule": "h1 = diag(linspace(-2, 0.5)) + sym(N(0, 0.1)) off-diagonal; "
                                            "L_g = sym(N(0, 1)) * chol_scale * exp(-g / chol_decay), "
                                            "chol_scale = 0.3 * 12 / norb, chol_decay = nchol / 4; trial = "
                                            "lowest nocc eigenvectors of h1"}},
           "roofline": roof, "dominant_phase": dominant, "other_kernels": tc,
           "phases_ms": {k: round(v[1] / args.steps, 3) for k, v in phases.items()},
           "gpu_launches": int(launches), "clocks": clk, "e2e": e2e}
    if cvline:
        out["control_variate"] = cvline
    if rank == 0 and not args.no_grad:
        out["differentiation"] = run_grad(n_blocks=args.grad_blocks)
        # the 200-orbital benchmark Hamiltonian: 256 walkers, 4 blocks (40 steps), binary64
        out["differentiation_c4"] = run_grad("c4_n200_o30_g1000_w4096", n_blocks=4, n_walkers=256)
    if rank == 0 and not args.no_large and args.workload != "c5_n400_o50_g2000_w1024":
        out["large_workload"] = run_large(args.precision)
    if compare:
        out["plain_fp64"] = compare
        out["ratio_vs_plain_fp64"] = round(value / compare["value"], 2)
    if oracle_cmp:
        out["vs_fp64_oracle"] = oracle_cmp
    if rank == 0 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(wl, args.cpu_seconds)
    return out


def run_grad(workload="c3_n60_o10_g300_w1024", n_blocks=20, checkpoint_every=20, eps=1e-4, n_walkers=None):
    """The differentiated energy: E = sum_b W_b e_b / sum_b W_b over n_blocks
    blocks (QR every 5 steps, checkpoints every 20 steps) with h1 + lam D at
    lam = 0; dE/dlam by the adjoint kernels against central differences at
    lam = +-eps on the same fields, the comb held at the unperturbed run's
    indices (and, for information, left free).  Default: the 60-orbital
    workload, 20 blocks (200 steps); n_walkers overrides its walker count."""
    import torch
    from ad_afqmc_prototype_gb300 import synth
    from ad_afqmc_prototype_gb300.core.system import system
    from ad_afqmc_prototype_gb300.grad import block_energies, mixed_energy
    from ad_afqmc_prototype_gb300.ham.chol import ham_chol
    from ad_afqmc_prototype_gb300.meas.rhf import make_rhf_meas_ops
    from ad_afqmc_prototype_gb300.prop.afqmc import init_prop_state
    from ad_afqmc_prototype_gb300.prop.types import afqmc_params
    from ad_afqmc_prototype_gb300.trial.rhf import make_rhf_trial_ops, rhf_trial
    wl = synth.WORKLOADS[workload]
    if n_walkers:
        wl = dataclasses.replace(wl, n_walkers=int(n_walkers))
    H = synth.make_workload(wl)
    sys_ = system(norb=wl.nbasis, nelec=(wl.nocc, wl.nocc), walker_kind="restricted")
    ham = ham_chol(h0=H["h0"], h1=H["h1"], chol=H["chol"])
    trial = rhf_trial(H["mo_coeff"])
    params = afqmc_params(dt=0.005, n_walkers=wl.n_walkers, seed=wl.seed, n_prop_steps=STEPS_PER_BLOCK,
                          qr_every=QR_EVERY)
    st0 = init_prop_state(sys=sys_, n_walkers=wl.n_walkers, seed=wl.seed, ham_data=ham,
                          trial_ops_=make_rhf_trial_ops(sys_), trial_data=trial, meas_ops=make_rhf_meas_ops(sys_),
                          initial_walkers=synth.trial_walkers(H["mo_coeff"], wl.n_walkers))
    D = torch.as_tensor(H["D"], device="cuda")
    kw = dict(ham_data=ham, trial_data=trial, params=params, state=st0, n_blocks=n_blocks, seed=17, counter=0,
              checkpoint_every=checkpoint_every)
    stream = torch.cuda.current_stream()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    # warm-up: one differentiated block, forward and backward (library handles, workspace, first launches)
    hw = ham.h1.clone().requires_grad_(True)
    ew, ww = block_energies(hw, **{**kw, "n_blocks": 1})
    mixed_energy(ew, ww).backward()
    torch.cuda.synchronize()
    h1 = ham.h1.clone().requires_grad_(True)
    runs = []
    ev[0].record(stream)
    e, w = block_energies(h1, run_out=runs, **kw)
    E = mixed_energy(e, w)
    ev[1].record(stream)
    E.backward()
    ev[2].record(stream)
    torch.cuda.synchronize()
    fwd_ms, bwd_ms = ev[0].elapsed_time(ev[1]), ev[1].elapsed_time(ev[2])
    e_val = float(E.detach())
    adj = float((h1.grad * D).sum())
    idx = runs[0].sr_idx

    def central(sr):
        vals, moved = [], 0
        with torch.no_grad():
            for s in (1.0, -1.0):
                r = []
                ee, ww = block_energies(ham.h1 + s * eps * D, sr_fixed=sr, run_out=r, **kw)
                vals.append(float(mixed_energy(ee, ww)))
                moved += int((r[0].sr_idx != idx).sum())
        return (vals[0] - vals[1]) / (2 * eps), moved

    fd, _ = central(idx)
    free, moved = central(None)
    return {"workload": workload, "n_walkers": wl.n_walkers, "n_blocks": n_blocks, "steps": n_blocks * STEPS_PER_BLOCK,
            "checkpoint_every_steps": checkpoint_every, "precision": "fp64",
            "energy": round(e_val, 10), "dE_dlambda_adjoint": adj, "dE_dlambda_fd_fixed_comb": fd,
            "rel_diff": abs(adj - fd) / abs(fd), "fd_eps": eps,
            "dE_dlambda_fd_free_comb": free, "free_comb_indices_moved": moved,
            "forward_ms": round(fwd_ms, 2), "backward_ms": round(bwd_ms, 2),
            "backward_over_forward": round(bwd_ms / fwd_ms, 2),
            "walker_steps_per_s_forward_backward": round(wl.n_walkers * n_blocks * STEPS_PER_BLOCK
                                                        / ((fwd_ms + bwd_ms) / 1000.0), 1)}


def run_large(precision, workload="c5_n400_o50_g2000_w1024", blocks=2):
    """The 400-orbital workload (nocc 50, nchol 2000, 1024 walkers) in the
    chosen form: one warm-up and `blocks` timed blocks with per-phase device
    times and each phase's roofline (algorithmic work), the device memory the
    run holds, the control-variate form timed on the same state (network
    trained on 3 recorded blocks), then one block of the binary64 form from
    the same state and fields for the ratio and |dE|."""
    import ctypes

    import torch
    from ad_afqmc_prototype_gb300 import _lib, engine, synth
    from ad_afqmc_prototype_gb300.prop.afqmc import device_state
    from ad_afqmc_prototype_gb300.prop.cv import ExchangeControlVariate
    wl = synth.WORKLOADS[workload]
    W, n, o, G = wl.n_walkers, wl.nbasis, wl.nocc, wl.nchol
    env = make_engine_state(wl, W, precision)
    st = device_state(env["state"], inplace=True)
    prob, params = env["prob"], env["params"]
    lib = _lib.load()
    ctr = 0
    engine.block(prob, params, st, 11, ctr)
    ctr += STEPS_PER_BLOCK + 1
    torch.cuda.synchronize()
    lib.afq_timing_reset()
    lib.afq_timing_enable(1)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(blocks):
        engine.block(prob, params, st, 11, ctr)
        ctr += STEPS_PER_BLOCK + 1
    e1.record()
    torch.cuda.synchronize()
    lib.afq_timing_enable(0)
    phases = _lib.timing_report()
    ms = e0.elapsed_time(e1) / blocks
    value = W * STEPS_PER_BLOCK / (ms / 1000.0)
    work = phase_work(n, o, G, W, trial_real=prob.trial_is_real, precision=precision)
    alg = algorithmic_work(n, o, G, W, trial_real=prob.trial_is_real)
    roofs = {k: roofline_for(phases, work, lib, blocks, name=k, alg=alg) for k in phases if k in work}
    d = engine.make_dims(W, n, o, G, True, prob.precision)
    mib = 1 << 20
    footprint = {"chol_f64_mib": round(G * n * n * 8 / mib, 1),
                 "rot_chol_f64_mib": round(G * o * n * 8 / mib, 1),
                 "lowp_split_operands_mib": round(int(lib.afq_lowp_bytes(ctypes.byref(d))) / mib, 1),
                 "walkers_c128_mib": round(W * n * o * 16 / mib, 1),
                 "block_workspace_mib": round(int(lib.afq_block_workspace(ctypes.byref(d), int(params.n_chunks))) / mib, 1),
                 "torch_peak_allocated_mib": round(torch.cuda.max_memory_allocated() / mib, 1)}
    # control variate: 3 recorded blocks train the network, then timed estimate blocks
    cv = ExchangeControlVariate(hidden=256, sample_fraction=1 / 8, seed=5)
    cv.mode = "record"
    for _ in range(3):
        engine.block(prob, params, st, 11, ctr, cv=cv.block_args(W))
        cv.after_block()
        ctr += STEPS_PER_BLOCK + 1
    cv.fit(epochs=20, batch=1024, lr=1e-3)
    cv.mode = "estimate"
    engine.block(prob, params, st, 11, ctr, cv=cv.block_args(W))
    cv.after_block()
    ctr += STEPS_PER_BLOCK + 1
    torch.cuda.synchronize()
    e0.record()
    for _ in range(blocks):
        engine.block(prob, params, st, 11, ctr, cv=cv.block_args(W))
        cv.after_block()
        ctr += STEPS_PER_BLOCK + 1
    e1.record()
    torch.cuda.synchronize()
    ms_cv = e0.elapsed_time(e1) / blocks
    cmp = compare_with_fp64(env, st, W, timed_blocks=1)
    return {"workload": workload, "precision": precision, "value": round(value, 3), "unit": UNIT,
            "ms_per_step": round(ms, 2), "phases_ms": {k: round(v[1] / blocks, 3) for k, v in phases.items()},
            "kernels": {k: {kk: r[kk] for kk in ("achieved", "frac", "bound", "unit", "executed_frac")
                            if kk in r} for k, r in roofs.items() if r},
            "hbm_footprint": footprint,
            "control_variate": {"value": round(W * STEPS_PER_BLOCK / (ms_cv / 1000.0), 3), "unit": UNIT,
                                "ms_per_step": round(ms_cv, 2), "exact_exchange_fraction": 1 / 8,
                                "training_blocks": 3},
            "plain_fp64": cmp, "ratio_vs_plain_fp64": round(value / cmp["value"], 2),
            "note": "norb 400 > 256: the Taylor series runs on the fp32 SIMT kernel; the QRs in global memory"}


def run_cv(args, env, st, W, world, seed, ctr, chain_blocks=40, run_steps=400):
    """The mixed + control-variate form against the exact measurement.

    Five recorded blocks (the first 50 steps) train the exchange network
    with the engine's kernels (timed).  Then two chains of `chain_blocks`
    blocks run from the same state on the same random stream: the exact
    measurement, and the control variate with exact exchange on 1/8 of the
    walkers.  Each chain's block energies give the standard error of its
    mean (blocking analysis, stat_utils.blocking_analysis_ratio), and

      efficiency = (se_exact^2 t_exact) / (se_cv^2 t_cv)

    per block, with the training time spread over a `run_steps`-step run
    (the learned-control-variate workload's 400 steps): > 1 means the control
    variate reaches a given error bar sooner.  The noise the sampling adds to
    one block's estimate is also measured on a fixed state (zero-step
    blocks, different samples)."""
    import torch
    from ad_afqmc_prototype_gb300 import engine
    from ad_afqmc_prototype_gb300.prop.cv import ExchangeControlVariate
    from ad_afqmc_prototype_gb300.stat_utils import blocking_analysis_ratio

    prob, params = env["prob"], env["params"]
    cv = ExchangeControlVariate(hidden=256, sample_fraction=1 / 8, seed=seed)
    cv.mode = "record"
    for _ in range(5):
        engine.block(prob, params, st, seed, ctr, cv=cv.block_args(W))
        cv.after_block()
        ctr += STEPS_PER_BLOCK + 1
    # one throwaway epoch on a second network first: the torch operations the
    # training uses (randperm on the device, gathers) are compiled for this GPU
    # on first use, a one-time cost that is not part of the training
    warm = ExchangeControlVariate(hidden=256, sample_fraction=1 / 8, seed=seed + 1)
    warm.data_x, warm.data_y = cv.data_x, cv.data_y
    warm.fit(epochs=1, batch=1024, lr=1e-3)
    torch.cuda.synchronize()
    t0 = time.time()
    losses = cv.fit(epochs=20, batch=1024, lr=1e-3)
    torch.cuda.synchronize()
    fit_s = time.time() - t0
    n_steps_fit = cv.adam_step

    def clone():
        return engine.DeviceState(*[t.clone() for t in (st.walkers, st.weights, st.overlaps, st.pop_shift,
                                                          st.e_estimate)])
    stream = torch.cuda.current_stream()

    def chain(use_cv):
        s0 = clone()
        cv.mode = "estimate" if use_cv else "off"
        engine.block(prob, params, clone(), seed, ctr, cv=cv.block_args(W))  # warm-up on a copy
        cv.after_block()
        es, ws = [], []
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        c = ctr
        for _ in range(chain_blocks):
            e, w = engine.block(prob, params, s0, seed, c, cv=cv.block_args(W))
            cv.after_block()
            es.append(e)
            ws.append(w)
            c += STEPS_PER_BLOCK + 1
        e1.record(stream)
        torch.cuda.synchronize()
        E = torch.cat(es).double().cpu().numpy()
        Wt = torch.cat(ws).double().cpu().numpy()
        r = blocking_analysis_ratio(E, Wt, print_q=False)
        return e0.elapsed_time(e1) / chain_blocks, float(r["mu"]), float(r["se_star"]), E

    ms_x, mu_x, se_x, _ = chain(False)
    ms_cv, mu_cv, se_cv, _ = chain(True)
    fit_ms_per_block = 1000.0 * fit_s / (run_steps / STEPS_PER_BLOCK)
    eff = (se_x ** 2 * ms_x) / (se_cv ** 2 * (ms_cv + fit_ms_per_block)) if se_cv > 0 else None

    # noise of one block's estimate on a fixed state (zero-step blocks)
    cv.mode = "estimate"
    z = dataclasses.replace(params, n_prop_steps=0)
    exact = float(engine.block(prob, z, clone(), seed, 0, zeta=0.5)[0])

    def draws(shift, scale, k=16):
        out = []
        for j in range(k):
            a = cv.block_args(W)
            a.y_shift, a.y_scale = shift, scale
            out.append(float(engine.block(prob, z, clone(), seed + 7919 * (j + 1), 0, zeta=0.5, cv=a)[0]))
            cv.after_block()
        return np.array(out)
    net, alone = draws(cv.y_shift, cv.y_scale), draws(0.0, 0.0)
    return {"value": round(world * W * STEPS_PER_BLOCK / (ms_cv / 1000.0), 3), "unit": UNIT,
            "ms_per_step": round(ms_cv, 3), "exact_exchange_fraction": 1 / 8,
            "network": "64-256-256-1 GELU, bf16 weights, mma.sync bf16 products (two-piece activations)",
            "training": {"blocks": 5, "samples": 5 * W, "epochs": 20, "adam_steps": n_steps_fit,
                         "seconds": round(fit_s, 3), "ms_per_adam_step": round(1000.0 * fit_s / max(n_steps_fit, 1), 3),
                         "loss_first": round(losses[0], 5), "loss_last": round(losses[-1], 5)},
            "chains": {"blocks": chain_blocks, "exact_ms_per_block": round(ms_x, 3),
                       "cv_ms_per_block": round(ms_cv, 3), "training_ms_per_block": round(fit_ms_per_block, 3),
                       "exact_mean_ha": mu_x, "exact_se_ha": se_x, "cv_mean_ha": mu_cv, "cv_se_ha": se_cv},
            "efficiency_vs_exact": round(eff, 4) if eff is not None else None,
            "noise_std_ha": float(net.std(ddof=1)), "noise_std_sample_alone_ha": float(alone.std(ddof=1)),
            "variance_ratio": float(net.var(ddof=1) / max(alone.var(ddof=1), 1e-300)),
            "mean_minus_exact_ha": float(net.mean() - exact),
            "measured": "chains: %d blocks each from one state on the same random stream; noise: 16 estimates of "
                        "one block-end state's energy (zero-step blocks, different samples)" % chain_blocks}


def compare_with_fp64(env, st_mixed, W, timed_blocks=3):
    """The metric's denominator and accuracy check, on the same workload:
    one block of the plain binary64 form and one of the mixed form from the
    same state with the same fields and comb uniform (|E_mixed - E_fp64|);
    the binary64 block also warms its form up, then `timed_blocks` more
    binary64 blocks are timed for the walker-steps/s."""
    import dataclasses

    import torch
    from ad_afqmc_prototype_gb300 import engine
    from ad_afqmc_prototype_gb300.prop.afqmc import engine_problem

    kw = dict(env["kw"])
    kw["params"] = dataclasses.replace(env["params"], precision="fp64")
    prob64 = engine_problem(n_walkers=W, need_energy=True, **kw)

    def clone(s):
        return engine.DeviceState(*[t.clone() for t in (s.walkers, s.weights, s.overlaps, s.pop_shift,
                                                          s.e_estimate)])
    a, b = clone(st_mixed), clone(st_mixed)
    ea, _ = engine.block(prob64, kw["params"], a, 77, 0, zeta=0.5)
    eb, _ = engine.block(env["prob"], env["params"], b, 77, 0, zeta=0.5)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for k in range(timed_blocks):
        engine.block(prob64, kw["params"], a, 77, (k + 1) * (STEPS_PER_BLOCK + 1))
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / timed_blocks
    return {"value": round(W * STEPS_PER_BLOCK / (ms / 1000.0), 3), "unit": UNIT, "ms_per_step": round(ms, 1),
            "measured": "binary64 blocks on the same workload: one untimed (the accuracy block), then %d timed"
                        % timed_blocks,
            "energy_error_per_block_ha": float(abs(float(ea) - float(eb))),
            "energy_fp64_ha": float(ea), "energy_mixed_ha": float(eb)}


def compare_with_oracle(wl, precision, st, n_sub=16, seed=5):
    """|dE| of the chosen form against the FP64 oracle itself: the first
    n_sub walkers of the benchmark's state (off the trial after the warm-up
    and timed blocks) with their weights, overlaps and shifts, one block of
    the engine in the chosen form and one of the oracle (oracle/afqmc_oracle.py)
    on the same fields and comb uniform; the binary64 engine beside it."""
    import dataclasses

    import torch
    from oracle import afqmc_oracle as O
    from ad_afqmc_prototype_gb300 import engine
    sub = make_engine_state(wl, n_sub, precision)
    H = sub["H"]
    walkers = st.walkers[:n_sub].clone()
    weights = st.weights[:n_sub].clone()
    overlaps = st.overlaps[:n_sub].clone()
    shift, e_est = float(st.pop_shift.reshape(-1)[0]), float(st.e_estimate.reshape(-1)[0])
    rng = np.random.default_rng(seed)
    fields = rng.standard_normal((STEPS_PER_BLOCK, n_sub, wl.nchol))
    zeta = float(rng.random())
    prob = O.make_problem(H["h0"], H["h1"], H["chol"], H["mo_coeff"], 0.005)
    P = O.Params(dt=0.005, n_prop_steps=STEPS_PER_BLOCK, qr_every=QR_EVERY)
    ost = O.State(walkers=walkers.cpu().numpy(), weights=weights.cpu().numpy(), overlaps=overlaps.cpu().numpy(),
                  pop_control_ene_shift=shift, e_estimate=e_est)
    ost, oobs, _ = O.afqmc_block(prob, P, ost, fields, zeta)
    out = {"walkers": n_sub, "energy_oracle_ha": oobs["energy"]}
    for form in (precision, "fp64"):
        env = sub if form == precision else make_engine_state(wl, n_sub, "fp64")
        dev = lambda t: t.to(device="cuda", copy=True)  # noqa: E731
        ds = engine.DeviceState(dev(walkers), dev(weights), dev(overlaps),
                                torch.tensor([shift], dtype=torch.float64, device="cuda"),
                                torch.tensor([e_est], dtype=torch.float64, device="cuda"))
        e, _ = engine.block(env["prob"], env["params"], ds, 0, 0, fields=fields, zeta=zeta)
        out["energy_error_ha" if form == precision else "fp64_engine_error_ha"] = abs(float(e) - oobs["energy"])
    out["measured"] = ("one block (10 steps, QR after step 5) of %d walkers of the benchmark state, engine vs the "
                       "NumPy FP64 oracle on the same fields" % n_sub)
    return out


_FMA_PEAK = {}


def fma_peak(lib, fp64: bool):
    """SIMT FMA throughput of this GPU (binary64 or binary32), measured once
    in-process: the pool's MEASURED_PEAKS.json has HBM and bf16 peaks only."""
    if fp64 not in _FMA_PEAK:
        import ctypes
        v = ctypes.c_double(0.0)
        rc = lib.afq_probe_fma_peak(1 if fp64 else 0, ctypes.byref(v))
        _FMA_PEAK[fp64] = ((round(v.value, 4), "measured in-process (%s FMA chains)" % ("fp64" if fp64 else "fp32"))
                           if rc == 0 else (None, None))
    return _FMA_PEAK[fp64]


def _parse_cpulist(text):
    cpus = set()
    for part in text.strip().split(","):
        if not part:
            continue
        a, _, b = part.partition("-")
        cpus.update(range(int(a), int(b or a) + 1))
    return cpus


def gpu_local_cpus(dev=0):
    """Host CPUs of the NUMA node the GPU is attached to (sysfs), or None."""
    try:
        import torch
        p = torch.cuda.get_device_properties(dev)
        addr = "%04x:%02x:%02x.0" % (p.pci_domain_id, p.pci_bus_id, p.pci_device_id)
        with open(f"/sys/bus/pci/devices/{addr}/numa_node") as f:
            node = int(f.read())
        if node < 0:
            return None
        with open(f"/sys/devices/system/node/node{node}/cpulist") as f:
            return _parse_cpulist(f.read()) or None
    except (AttributeError, OSError, ValueError, RuntimeError):
        return None


def run_e2e(args, env, afqmc_block, W):
    """The same metric through the public API with host buffers: each step
    copies walkers, weights and overlaps from pinned host memory, runs
    afqmc_block, and reads walkers, weights, overlaps and the block energy
    back to pinned host memory.  The process runs on the GPU's local NUMA
    node meanwhile (when sysfs names one), so that the pinned buffers are
    placed in the memory next to the GPU; the affinity is restored after."""
    old = os.sched_getaffinity(0)
    local = gpu_local_cpus() if args.e2e_numa else None
    use = (local & old) if local else None
    if use:
        os.sched_setaffinity(0, use)
    try:
        out = _run_e2e(args, env, afqmc_block, W)
    finally:
        if use:
            os.sched_setaffinity(0, old)
    out["host_numa_local"] = bool(use)
    return out


def _run_e2e(args, env, afqmc_block, W):
    import torch
    st0 = env["state"]
    hw = torch.empty(st0.walkers.shape, dtype=torch.complex128, pin_memory=True)
    hwt = torch.empty(st0.weights.shape, dtype=torch.float64, pin_memory=True)
    hov = torch.empty(st0.overlaps.shape, dtype=torch.complex128, pin_memory=True)
    he = torch.empty((), dtype=torch.float64, pin_memory=True)
    hw.copy_(st0.walkers)
    hwt.copy_(st0.weights)
    hov.copy_(st0.overlaps)
    dw, dwt, dov = torch.empty_like(st0.walkers), torch.empty_like(st0.weights), torch.empty_like(st0.overlaps)
    state = st0

    def one(state):
        dw.copy_(hw, non_blocking=True)
        dwt.copy_(hwt, non_blocking=True)
        dov.copy_(hov, non_blocking=True)
        s_in = state._replace(walkers=dw, weights=dwt, overlaps=dov)
        s_out, obs = afqmc_block(s_in, sys=env["sys"], inplace=True, **env["kw"])
        hw.copy_(s_out.walkers, non_blocking=True)
        hwt.copy_(s_out.weights, non_blocking=True)
        hov.copy_(s_out.overlaps, non_blocking=True)
        he.copy_(obs.scalars["energy"], non_blocking=True)
        return s_out

    for _ in range(max(1, min(args.warmup, 2))):
        state = one(state)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        state = one(state)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    bi = hw.numel() * 16 + hwt.numel() * 8 + hov.numel() * 16
    return {"value": round(W * STEPS_PER_BLOCK / (ms / 1000.0), 3), "unit": UNIT, "h2d_bytes_per_step": bi,
            "d2h_bytes_per_step": bi + 8, "ms_per_step": round(ms, 3), "api": "prop.blocks.afqmc_block"}


# --------------------------------------------------------- CPU baselines ---
def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_block_rate(wl, budget_s, warm=False):
    """Times the CPU oracle on a bounded sample of the workload: blocks of
    10 steps (QR after step 5) on a few walkers until `budget_s` is spent.
    Returns (walker-steps/s, sample description)."""
    from oracle import afqmc_oracle as O
    from ad_afqmc_prototype_gb300 import synth
    H = synth.make_workload(wl)
    prob = O.make_problem(H["h0"], H["h1"], H["chol"], H["mo_coeff"], 0.005)
    P = O.Params(dt=0.005, n_prop_steps=STEPS_PER_BLOCK, qr_every=QR_EVERY)
    ws = min(wl.n_walkers, 32 if wl.nbasis >= 120 else 256)
    st = O.init_prop_state(prob, ws, synth.trial_walkers(H["mo_coeff"], ws))
    rng = np.random.default_rng(0)
    if warm:
        st, _, _ = O.afqmc_block(prob, P, st, rng.standard_normal((STEPS_PER_BLOCK, ws, wl.nchol)), 0.5)
    t0 = time.perf_counter()
    nblk = 0
    while True:
        f = rng.standard_normal((STEPS_PER_BLOCK, ws, wl.nchol))
        st, _, _ = O.afqmc_block(prob, P, st, f, float(rng.random()))
        nblk += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    return ws * STEPS_PER_BLOCK * nblk / dt, f"{nblk} block(s) of 10 steps on {ws} walkers, {dt:.1f} s"


def cpu_baseline(wl, budget_s):
    rate, sample = cpu_block_rate(wl, budget_s)
    return {"value": round(rate, 3), "unit": UNIT, "cores": cpu_cores(), "kind": "port", "sample": sample,
            "what": "NumPy FP64 restatement of the reference algorithm (oracle/afqmc_oracle.py), BLAS threads = all"}


def run_reference(args, rank, world):
    from ad_afqmc_prototype_gb300 import synth
    wl = synth.WORKLOADS[args.workload]
    for _ in range(args.warmup):
        cpu_block_rate(wl, 0.0)
    rates = []
    sample = ""
    for _ in range(args.steps):
        r, sample = cpu_block_rate(wl, 0.0)
        rates.append(r)
    value = float(np.mean(rates))
    ms = 1000.0 * STEPS_PER_BLOCK * (32 if wl.nbasis >= 120 else 256) / value
    return {"impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "precision": "fp64",
                       "step": "one block: 10 propagation steps, QR after step 5, QR + energy + comb at the end"},
            "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": cpu_cores(), "kind": "port",
                             "sample": sample + " per step",
                             "what": "the JAX reference cannot be installed (no jax wheel); its algorithm "
                                     "restated in NumPy FP64 (oracle/afqmc_oracle.py)"},
            "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    args = parse()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(run_reference(args, rank, world)), flush=True)
        return
    import torch
    local = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import __graft_entry__ as g
    g.build()
    if args.grad_only:
        if rank == 0:
            print(json.dumps({"differentiation": run_grad(n_blocks=args.grad_blocks)}), flush=True)
        return
    out = run_ours(args, rank, world)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
