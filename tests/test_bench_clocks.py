"""The bench's clock record (CPU, with a stand-in for nvidia-smi): only
samples taken inside the timed regions count, throttle reasons seen there are
reported, and a region too short for any sample falls back to the samples
right after it."""
import os
import sys
import time

import pytest

import bench

FAKE = """#!{python}
import datetime, sys, time
ctl = {ctl!r}
while True:
    now = datetime.datetime.now()
    try:
        sm, cap = open(ctl).read().split()
    except (OSError, ValueError):
        continue
    stamp = now.strftime("%Y/%m/%d %H:%M:%S.%f")[:-3]
    print(f"{{stamp}}, 0, {{sm}}, 2070, 900.00, 0x0, Not Active, Not Active, Not Active, {{cap}}", flush=True)
    time.sleep(0.02)
"""


@pytest.fixture
def fake_smi(tmp_path):
    ctl = tmp_path / "state"
    ctl.write_text("1005 Not_Active")
    exe = tmp_path / "fake-smi"
    exe.write_text(FAKE.format(python=sys.executable, ctl=str(ctl)))
    exe.chmod(0o755)

    def state(sm, cap="Not_Active"):
        tmp = tmp_path / "state.tmp"
        tmp.write_text(f"{sm} {cap}")
        os.replace(tmp, ctl)
    return str(exe), state


def _norm(clk):
    return clk["sm_mhz"], clk["sm_max_mhz"], clk["reasons"]


def test_only_samples_inside_the_timed_regions_count(fake_smi):
    exe, state = fake_smi
    c = bench.ClockSampler(0, exe=exe)
    c.start()
    time.sleep(0.15)             # idle before the region: 1005 MHz
    state(2070)
    c.begin()
    time.sleep(0.25)
    c.end()
    time.sleep(0.03)
    state(1005)
    time.sleep(0.15)             # idle between regions
    state(1980, "Active")        # power cap inside the second region
    c.begin()
    time.sleep(0.25)
    c.end()
    time.sleep(0.03)
    state(1005)
    time.sleep(0.1)
    clk = c.stop()
    assert clk["regions"] == 2 and clk["samples"] >= 4  # about 25 expected
    assert clk["span"] == "samples inside the timed regions"
    assert clk["sm_mhz"] in (1980.0, 2070.0, 2025.0) and clk["sm_max_mhz"] == 2070.0
    assert clk["reasons"] == ["sw_power_cap"]


def test_short_region_takes_the_next_sample(fake_smi):
    exe, state = fake_smi
    state(2070)
    c = bench.ClockSampler(0, exe=exe)
    c.start()
    time.sleep(0.03)
    c.begin()
    c.end()                      # far shorter than the sampling interval
    time.sleep(0.2)
    clk = c.stop()
    assert clk["samples"] >= 1 and clk["sm_mhz"] == 2070.0
    # (a sample stamped to the millisecond can still land inside the region)
    assert clk["span"].startswith("no sample inside") or clk["samples"] == 1


def test_missing_tool_is_reported():
    c = bench.ClockSampler(0, exe="/nonexistent/nvidia-smi")
    c.start()
    c.begin()
    c.end()
    assert c.stop()["reasons"] == ["nvidia-smi unavailable"]
