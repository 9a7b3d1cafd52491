"""The benchmark line's derived fields, on the CPU: the roofline entry's keys
and arithmetic, and the default batch (one wave of the tensor-core GPR)."""
import json
import os
import sys
import types

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_roofline_entry_keys_and_arithmetic():
    stages = [0.22, 0.35, 0.24, 0.52]  # ms: neighbours, descriptors, gpr, chain rule
    N, D = 38912, 64
    roof = bench.roofline(stages, N, D, "tc")
    peaks, _ = bench.load_peaks()
    assert roof["kernel"] == "chain_rule" and roof["bound"] == "hbm" and roof["unit"] == "GB/s"
    bpa = bench.stage_bytes_per_atom(D)["chain_rule"]
    assert np.isclose(roof["achieved"], bpa * N / (0.52e-3) / 1e9)
    assert roof["peak"] == peaks["hbm_gbs"]
    assert np.isclose(roof["frac"], roof["achieved"] / roof["peak"])
    inputs = json.load(open(os.path.join(ROOT, "profiles", "roofline_inputs.txt")))
    assert np.isclose(roof["traffic"], inputs["dram_bytes_per_atom"]["chain_rule"] * N)
    t = roof["gpr_tensor"]
    assert t["bound"] == "tensor" and t["unit"] == "TFLOP/s"
    assert np.isclose(t["frac"], t["achieved"] / t["peak"])
    assert set(roof["stage_ms"]) == set(bench.STAGES)
    # forms without a tensor-core GPR report no tensor entry; TF32 has its own
    assert "gpr_tensor" not in bench.roofline(stages, N, D, "fp32")
    t32 = bench.roofline(stages, N, D, "tf32")["gpr_tensor"]
    assert np.isclose(t32["peak"], 0.5 * peaks["bf16_tflops"])
    assert np.isclose(t32["achieved"], 4.0 * N * 4032 * 64 / 0.24e-3 / 1e12)
    # a measured TF32 rate replaces the nominal ratio
    t32m = bench.roofline(stages, N, D, "tf32", tf32_tflops=900.0)["gpr_tensor"]
    assert t32m["peak"] == 900.0 and "measured" in t32m["peak_source"]


def test_roofline_population_counts_and_no_alloy_traffic():
    stages = [0.5, 1.0, 0.8, 1.2]
    N, D, P, T = 100000, 64, 40.0, 300.0
    roof = bench.roofline(stages, N, D, "tf32", P=P, T=T, traffic_file=False)
    assert roof["traffic"] is None
    assert np.isclose(roof["algorithmic_bytes_per_atom"],
                      bench.stage_bytes_per_atom(D, P, T)["chain_rule"])
    assert np.isclose(roof["chain_rule_fp32"]["flops_per_atom"], 150.0 * T + 15.0 * P * 20)


def test_population_cpu_baseline_on_two_cells():
    import gapgb.synth as S
    pop = S.population(3, seed=5)
    ty, al, rc, ze = S.sf_table()
    zt = np.array([3, 8, 14, 26], np.int32)
    D = 2 * len(ty)
    rng = np.random.default_rng(0)
    arrays = (zt, zt.astype(np.float64), ty, al, rc, ze, np.ones(D), rng.normal(size=(4, D)),
              rng.normal(size=4) * 1e-3)
    cb = bench.population_cpu_baseline(arrays, pop, 2)
    assert cb["kind"] == "port" and cb["value"] > 0 and cb["unit"] == bench.UNIT
    assert "%d atoms" % int(pop[0][2]) in cb["sample"]


def test_roofline_uses_measured_simt_peaks_and_plain_stages():
    stages = [0.22, 0.35, 0.24, 0.52]
    plain = [0.9, 60.0, 75.0, 35.0]
    N, D = 38912, 64
    simt = {"fp32_tflops": 70.0, "fp64_tflops": 1.2, "ex2_per_s_1e12": 4.5}
    roof = bench.roofline(stages, N, D, "tc", simt=simt, plain_stages=plain)
    c = roof["chain_rule_fp32"]
    assert c["peak_tflops"] == 70.0 and np.isclose(c["frac"], c["achieved_tflops"] / 70.0)
    assert np.isclose(roof["gpr_exp"]["peak_per_s"], 4.5e12)
    pl = roof["plain_fp64"]
    assert pl["peak_tflops"] == 1.2
    # the plain GPR: 4 M D flops per atom over its stage time
    assert np.isclose(pl["gpr"]["achieved_tflops"], 4.0 * bench.M_SPARSE * D * N / 75e-3 / 1e12)
    assert np.isclose(pl["gpr"]["frac"], pl["gpr"]["achieved_tflops"] / 1.2)


def test_default_batch_is_one_gpr_wave(monkeypatch):
    import torch
    monkeypatch.setattr(torch.cuda, "get_device_properties",
                        lambda dev: types.SimpleNamespace(multi_processor_count=152))
    args = types.SimpleNamespace(batch=None)
    assert bench.default_batch(args, 0) == 76  # 152 SMs x 2 CTAs x 128 atoms / 512
    args = types.SimpleNamespace(batch=64)
    assert bench.default_batch(args, 0) == 64  # an explicit --batch wins


def test_step_kernel_counts():
    # prep x2, neighbour build x2 (wide and other cells), structure sums x2,
    # and 4 per pipeline
    assert bench.step_kernels("tc", 38912) == 14        # two pipelines
    assert bench.step_kernels("tc", 38912, pipelines=1) == 10
    assert bench.step_kernels("tc", 8192) == 10         # below the split threshold
    assert bench.step_kernels("fp32", 38912) == 10      # SIMT forms run one pipeline
    assert bench.step_kernels("tf32", 10 ** 6, generic=True) == 13
