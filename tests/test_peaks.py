"""The measured arithmetic peaks (gapgb_measure_peaks) that the benchmark's
roofline entries divide by: finite, ordered as the hardware's pipes are, and
below what 128 FP32 lanes per SM can do at the GB300's 2070 MHz maximum."""
import pytest

pytestmark = pytest.mark.gpu


def test_measured_peaks_are_plausible(gapgb_mod):
    import torch
    p = gapgb_mod.measure_peaks()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    # FP32: at most 128 lanes x 2 flops per SM per clock (2070 MHz maximum)
    cap32 = sms * 128 * 2 * 2070e6 / 1e12
    assert 0.3 * cap32 < p["fp32_tflops"] <= 1.05 * cap32, (p, cap32)
    # FP64 and MUFU run well below the FP32 FMA rate
    assert 0.0 < p["fp64_tflops"] < p["fp32_tflops"]
    assert 0.0 < p["ex2_per_s_1e12"] * 2 < p["fp32_tflops"]
