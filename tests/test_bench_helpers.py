"""Host-side helpers of bench.py (no GPU): the clock record's parsing (median
SM clock under load, the throttle reasons seen), the figures the bench line
takes from the committed ncu summaries, and the peak it divides by."""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


class _Done:
    """Stands in for the finished nvidia-smi process."""

    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def _sampler(tmp_path, monkeypatch, lines):
    monkeypatch.setenv("ELX_CLOCKS_DIR", str(tmp_path))
    s = bench.ClockSampler(0)
    with open(s.path, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    s.fh = open(os.devnull, "w")
    s.proc = _Done()
    return s


def test_clock_record_median_under_load_and_reasons(tmp_path, monkeypatch):
    na, act = "Not Active", "Active"
    lines = [
        f"0, 345, 2070, 95.1, 0x1, {na}, {na}, {na}, {na}",        # idle, before the load
        f"0, 2070, 2070, 900.2, 0x0, {na}, {na}, {na}, {na}",
        f"0, 2055, 2070, 1301.0, 0x4, {na}, {na}, {na}, {act}",    # power cap
        f"0, 2070, 2070, 1100.7, 0x0, {na}, {na}, {na}, {na}",
        "garbage line",
        f"0, [N/A], 2070, 0, 0x0, {na}, {na}, {na}, {na}",
    ]
    clk = _sampler(tmp_path, monkeypatch, lines).stop()
    assert clk["sm_max_mhz"] == 2070.0
    assert clk["sm_mhz"] == 2070.0        # the idle sample is not under load
    assert clk["reasons"] == ["sw_power_cap"]
    assert clk["samples"] == 4


def test_clock_record_flags_slowdowns(tmp_path, monkeypatch):
    na, act = "Not Active", "Active"
    lines = [f"0, 1500, 2070, 700.0, 0x8, {act}, {na}, {act}, {na}"] * 3
    clk = _sampler(tmp_path, monkeypatch, lines).stop()
    assert clk["reasons"] == ["hw_slowdown", "sw_thermal_slowdown"]
    assert clk["sm_mhz"] == 1500.0


def test_no_clock_record(tmp_path, monkeypatch):
    assert _sampler(tmp_path, monkeypatch, []).stop() is None
    s = bench.ClockSampler(0)
    assert s.stop() is None  # never started (no nvidia-smi)


def test_profiled_figures_come_from_the_committed_summary():
    traffic = bench.profiled("traffic_bytes_per_launch")
    pipe = bench.profiled("fp64_pipe_frac")
    assert traffic is not None and 4.0e8 < traffic < 1.0e9  # DRAM bytes of one FP64 product
    assert pipe is not None and 0.0 < pipe <= 1.0
    assert bench.profiled("traffic_bytes_per_launch", "sell_spmm_fp32_w16_hexa8_plate96.md") > 0
    assert bench.profiled("no_such_key") is None
    assert bench.profiled("traffic_bytes_per_launch", "no_such_file.md") is None


def test_measured_peak():
    peak, kind = bench.measured_peak()
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            assert (peak, kind) == (float(json.load(fh)["hbm_gbs"]), "measured")
    else:
        assert kind == "fallback" and peak > 0
