"""bench.py's clock record on CPU: the nvidia-smi sampler run against a fake
nvidia-smi that prints fixed samples.  The summary gives the median SM clock
under load, the maximum clock, and every throttle reason seen Active in any
sample (a run with hw_slowdown, hw_thermal_slowdown or sw_thermal_slowdown is
rejected; sw_power_cap is kept and noted)."""
import importlib.util
import os
import stat
import time
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _load_bench():
    spec = importlib.util.spec_from_file_location("bench_clocks_under_test", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _fake_smi(tmp_path, rows):
    body = "\n".join(rows)
    script = tmp_path / "nvidia-smi"
    script.write_text(f"#!/bin/sh\ncat <<'EOF'\n{body}\nEOF\nexec sleep 30\n")
    script.chmod(script.stat().st_mode | stat.S_IXUSR)
    return tmp_path


def _sample(monkeypatch, bench, bindir):
    monkeypatch.setenv("PATH", f"{bindir}{os.pathsep}{os.environ.get('PATH', '')}")
    with bench.ClockSampler(0) as cs:
        t0 = time.time()
        while time.time() - t0 < 10 and (cs.file is None or Path(cs.file.name).stat().st_size == 0):
            time.sleep(0.05)
        time.sleep(0.2)
    return cs.summary()


NA = "Not Active"


@pytest.fixture(scope="module")
def bench():
    return _load_bench()


def test_clean_run(bench, tmp_path, monkeypatch):
    rows = [f"0, {mhz}, 2070, 1100.0, 0x0000000000000000, {NA}, {NA}, {NA}, {NA}" for mhz in (2070, 2055, 2070)]
    s = _sample(monkeypatch, bench, _fake_smi(tmp_path, rows))
    assert s == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": [], "samples": 3}


def test_reasons_seen_in_any_sample(bench, tmp_path, monkeypatch):
    rows = [
        f"0, 2070, 2070, 1390.0, 0x0000000000000004, {NA}, {NA}, {NA}, Active",
        f"0, 1500, 2070, 1000.0, 0x0000000000000008, Active, {NA}, {NA}, {NA}",
        f"0, 2070, 2070, 1200.0, 0x0000000000000000, {NA}, {NA}, {NA}, {NA}",
    ]
    s = _sample(monkeypatch, bench, _fake_smi(tmp_path, rows))
    assert s["reasons"] == ["hw_slowdown", "sw_power_cap"]
    assert s["sm_mhz"] == 2070.0 and s["samples"] == 3


def test_malformed_and_unavailable_rows_are_skipped(bench, tmp_path, monkeypatch):
    rows = [
        "0, [N/A], 2070, [N/A], [N/A], [N/A], [N/A], [N/A], [N/A]",
        "garbage",
        f"0, 1900, 2070, 1100.0, 0x0000000000000000, {NA}, {NA}, Active, {NA}",
    ]
    s = _sample(monkeypatch, bench, _fake_smi(tmp_path, rows))
    assert s == {"sm_mhz": 1900.0, "sm_max_mhz": 2070.0, "reasons": ["sw_thermal_slowdown"], "samples": 1}


def test_no_nvidia_smi_gives_no_record(bench, tmp_path, monkeypatch):
    monkeypatch.setenv("PATH", str(tmp_path))  # an empty directory: nvidia-smi is not found
    with bench.ClockSampler(0) as cs:
        pass
    assert cs.summary() is None
