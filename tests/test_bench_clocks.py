"""Clock and throttle sampling of bench.py (CPU, a stand-in nvidia-smi on PATH): the median SM
clock under load, the highest clock and the throttle reasons seen, which decide whether a timed
run is kept; and the measured HBM peak the roofline divides by."""
import json
import os
import stat
import sys
import time

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402

IDLE = "Not Active"


def _row(sm, mx, hw=IDLE, thermal=IDLE, sw_thermal=IDLE, power=IDLE):
    return f"0, {sm}, {mx}, 850.25, 0x0000000000000000, {hw}, {thermal}, {sw_thermal}, {power}"


def _fake_smi(tmp_path, rows):
    """An nvidia-smi that prints `rows` as its query output, then waits to be stopped."""
    d = tmp_path / "bin"
    d.mkdir()
    (tmp_path / "rows.txt").write_text("\n".join(rows) + "\n")
    exe = d / "nvidia-smi"
    exe.write_text("#!%s\nimport sys, time\nsys.stdout.write(open(%r).read())\nsys.stdout.flush()\ntime.sleep(60)\n"
                   % (sys.executable, str(tmp_path / "rows.txt")))
    exe.chmod(exe.stat().st_mode | stat.S_IXUSR)
    return str(d)


def _sample(monkeypatch, path):
    monkeypatch.setenv("PATH", path)
    s = bench.ClockSampler(0)
    s.start()
    time.sleep(1.0)  # the stand-in has printed everything by then
    return s.stop()


def test_clean_run(tmp_path, monkeypatch):
    rows = [_row(2070, 2070), _row(2055, 2070), _row(2070, 2070), _row("[N/A]", 2070)]
    got = _sample(monkeypatch, _fake_smi(tmp_path, rows))
    assert got == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": [], "samples": 4}


@pytest.mark.parametrize("column,name", [("hw", "hw_slowdown"), ("thermal", "hw_thermal_slowdown"),
                                         ("sw_thermal", "sw_thermal_slowdown"), ("power", "sw_power_cap")])
def test_throttle_reasons_are_reported(tmp_path, monkeypatch, column, name):
    rows = [_row(2070, 2070), _row(1800, 2070, **{column: "Active"}), _row(1900, 2070)]
    got = _sample(monkeypatch, _fake_smi(tmp_path, rows))
    assert got["reasons"] == [name]
    assert got["sm_mhz"] == 1900.0 and got["sm_max_mhz"] == 2070.0 and got["samples"] == 3


def test_clock_held_below_maximum_is_visible(tmp_path, monkeypatch):
    # a leftover clock lock: no reason active, the clock far below its maximum
    rows = [_row(1200, 2070)] * 5
    got = _sample(monkeypatch, _fake_smi(tmp_path, rows))
    assert got["reasons"] == [] and got["sm_mhz"] == 1200.0 and got["sm_max_mhz"] == 2070.0


def test_without_nvidia_smi(tmp_path, monkeypatch):
    empty = tmp_path / "empty"
    empty.mkdir()
    got = _sample(monkeypatch, str(empty))
    assert got["sm_mhz"] is None and got["reasons"] == ["nvidia-smi unavailable"]


def test_measured_hbm_peak_comes_from_the_measured_file():
    peak, source = bench.measured_hbm_peak()
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            assert (peak, source) == (float(json.load(f)["hbm_gbs"]), "measured")
    else:
        assert (peak, source) == (6800.0, "fallback")
