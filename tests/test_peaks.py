"""The measured arithmetic peaks (gapgb_measure_peaks) that the benchmark's
roofline entries divide by: finite, ordered as the hardware's pipes are, and
consistent with the clock the kernels report."""
import pytest

pytestmark = pytest.mark.gpu


def test_measured_peaks_are_plausible(gapgb_mod):
    import torch
    p = gapgb_mod.measure_peaks()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    for k in ("fp32_mhz", "fp64_mhz", "ex2_mhz"):
        assert 300.0 < p[k] < 3500.0, p
    # FP32: at most 128 lanes x 2 flops per SM per clock
    cap32 = sms * 128 * 2 * p["fp32_mhz"] * 1e6 / 1e12
    assert 0.3 * cap32 < p["fp32_tflops"] <= 1.05 * cap32, (p, cap32)
    # FP64 and MUFU run well below the FP32 FMA rate
    assert 0.0 < p["fp64_tflops"] < p["fp32_tflops"]
    assert 0.0 < p["ex2_per_s_1e12"] * 2 < p["fp32_tflops"]
