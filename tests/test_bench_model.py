"""CPU checks of bench.py's work model and roofline selection (no GPU):
the tensor-core Taylor products run on the tensor pipe, the roofline counts
algorithmic work (the executed split-operand work beside it), the mixed
forms' double-float phases are measured against the fp32 pipe, and the
roofline's numbers follow from the phase times."""
import math

import pytest

bench = pytest.importorskip("bench")


def test_phase_work_pipes_per_precision():
    fp64 = bench.phase_work(200, 30, 1000, 4096, precision="fp64")
    assert {p for _, p in fp64.values()} == {"fp64"}
    fast = bench.phase_work(200, 30, 1000, 4096, precision="mixed_fast")
    assert fast["trotter"][1] == "tensor"
    # three bf16 sections of 6 V products (2n x 2o x 2n) and 2 E - I products (2n x 2o x n) per walker
    # 128 x 208 x 16 MMAs, two a K step: 6 V products of 26 K steps, 2 E - I products of 13
    assert fast["trotter"][0] == pytest.approx((6 * 26 + 2 * 13) * 2 * (2 * 128 * 208 * 16) * 4096)
    for k in ("overlap", "green", "qr"):
        assert fast[k][1] == "df32"
    for k in ("vbuild_gemm", "fb_gemm", "e_gemm"):
        assert fast[k][1] == "tensor"
    # no tensor-core Taylor kernel past norb 256 or nocc 32
    assert bench.phase_work(400, 50, 2000, 1024, precision="mixed_fast")["trotter"][1] == "fp32"
    assert bench.phase_work(200, 30, 1000, 4096, precision="mixed")["trotter"][1] == "fp32"


def test_roofline_is_algorithmic_with_executed_beside(monkeypatch):
    monkeypatch.setitem(bench._FMA_PEAK, False, (70.0, "given"))  # fp32 SIMT peak (the probe needs a GPU)
    work = bench.phase_work(200, 30, 1000, 4096, precision="mixed_fast")
    alg = bench.algorithmic_work(200, 30, 1000, 4096)
    # (calls, device ms) over 2 blocks
    phases = {"overlap": (20, 30.0), "trotter": (20, 49.0), "vbuild_gemm": (20, 44.0), "e_gemm": (2, 20.0),
              "energy": (2, 22.0), "qr": (4, 17.0)}
    r = bench.roofline_for(phases, work, None, 2, alg=alg)
    assert r["kernel"] == "trotter" and r["bound"] == "tensor" and r["unit"] == "TFLOP/s"
    # achieved counts the reference's flops (8 n_terms + 8) n^2 o per walker, not the three bf16 sections
    flops_block = (8 * 6 + 8) * 200 ** 2 * 30 * 4096 * bench.STEPS_PER_BLOCK
    assert r["achieved"] == pytest.approx(flops_block / (49.0 / 2 / 1000.0) / 1e12, rel=1e-4)
    assert math.isclose(r["frac"], r["achieved"] / r["peak"], rel_tol=1e-3)
    # executed: the Taylor kernel's MMAs (128 rows, N = 208, hi and mid pieces of V)
    assert r["executed_achieved"] == pytest.approx(r["achieved"] * work["trotter"][0] / alg["trotter"], rel=1e-3)
    assert work["trotter"][0] / alg["trotter"] == pytest.approx(7168 * 208 ** 2 / (56 * 200 ** 2 * 30), rel=1e-9)
    # the share excludes the composite energy phase that encloses e_gemm
    assert r["share_of_step"] == pytest.approx(49.0 / (30 + 49 + 44 + 20 + 17), rel=1e-3)
    # the double-float phases are measured against the fp32 pipe they run on
    ov = bench.roofline_for(phases, work, None, 2, name="overlap", alg=alg)
    assert ov["bound"] == "fp32" and ov["peak"] == 70.0 and "executed_achieved" not in ov
    assert ov["achieved"] == pytest.approx(alg["overlap"] * 10 / (30.0 / 2 / 1000.0) / 1e12, rel=1e-4)


def test_roofline_binary64_form_keeps_fp64_phases(monkeypatch):
    monkeypatch.setitem(bench._FMA_PEAK, True, (1.25, "given"))  # the in-process probe needs a GPU
    work = bench.phase_work(200, 30, 1000, 4096, precision="fp64")
    phases = {"vbuild_gemm": (20, 100.0), "overlap": (20, 10.0)}
    r = bench.roofline_for(phases, work, None, 2)
    assert r["kernel"] == "vbuild_gemm" and r["bound"] == "fp64" and r["peak"] == 1.25
    r = bench.roofline_for(phases, work, None, 2, name="overlap")
    assert r["kernel"] == "overlap" and r["bound"] == "fp64"


def test_host_numa_helpers():
    """The end-to-end line's NUMA helper parses sysfs cpulists and gives up
    quietly where no GPU (or no sysfs entry) is found."""
    assert bench._parse_cpulist("0-3,8,10-11\n") == {0, 1, 2, 3, 8, 10, 11}
    assert bench._parse_cpulist("5") == {5}
    assert bench._parse_cpulist("") == set()
    got = bench.gpu_local_cpus()
    assert got is None or (isinstance(got, set) and got)
