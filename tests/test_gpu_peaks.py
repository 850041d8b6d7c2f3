"""chgpu_measure_peaks: the FMA and copy rates the benchmark reports the
kernels against are measured, and plausible for a GB300 (FP64 far below
FP32; copy in the TB/s range)."""
import pytest

pytestmark = pytest.mark.gpu


def test_measured_peaks_plausible(gpu_lib):
    from channel_gb300.lib import measure_peaks

    pk = measure_peaks()
    assert 0.2 < pk["fp64_tflops"] < 100.0, pk
    assert 10.0 < pk["fp32_tflops"] < 300.0, pk
    assert pk["fp32_tflops"] > 4 * pk["fp64_tflops"], pk
    assert 500.0 < pk["copy_gbs"] < 20000.0, pk
