"""risa_gb_measure_peak, the micro-benchmarks behind the backprojection's
roofline denominators: the shared-memory read rate and the FP32 FMA rate per
SM and clock must lie just under the hardware's issue limits (128 bytes and
256 FLOP per SM per clock), the SM clock they report must be a real clock of
the device, and bad arguments are refused without a launch."""
import pytest

import risa_gb300 as rg

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def test_shared_memory_read_peak():
    m = rg.measure_peak(rg.PEAK_SMEM_READ, reps=3)
    props = torch.cuda.get_device_properties(0)
    assert m["sms"] == props.multi_processor_count
    assert 100.0 < m["per_sm_per_clk"] <= 128.5, m  # 128 B/clk/SM: four 8-lane phases of 16 B per load
    assert 500.0 < m["sm_mhz"] < 3500.0, m
    assert m["value"] == pytest.approx(m["per_sm_per_clk"] * m["sm_mhz"] * 1e6 * m["sms"] / 1e9, rel=1e-6)


def test_fp32_fma_peak():
    m = rg.measure_peak(rg.PEAK_FP32_FMA, reps=3)
    assert 200.0 < m["per_sm_per_clk"] <= 256.5, m  # 128 FMA lanes x 2 FLOP per SM and clock
    assert m["value"] == pytest.approx(m["per_sm_per_clk"] * m["sm_mhz"] * 1e6 * m["sms"] / 1e12, rel=1e-6)


def test_bad_arguments_are_refused():
    with pytest.raises(rg.RisaError):
        rg.measure_peak(7)
    with pytest.raises(rg.RisaError):
        rg.measure_peak(rg.PEAK_SMEM_READ, reps=0)
