"""The benchmark's clock record: the samples nvidia-smi wrote inside the timed
region are kept (by their own timestamps) and the throttle reasons read from
them; no GPU or nvidia-smi is needed to check the parsing."""
import datetime
import importlib
import sys

from .conftest import ROOT


def _bench():
    sys.path.insert(0, str(ROOT))
    return importlib.import_module("bench")


def _row(t, sm, reasons=("Not Active",) * 4):
    ts = datetime.datetime.fromtimestamp(t).strftime("%Y/%m/%d %H:%M:%S.%f")[:-3]
    return f"{ts}, 0, {sm}, 2070, 900.5, 0x0, " + ", ".join(reasons)


def test_clock_summary_keeps_the_timed_region(tmp_path):
    bench = _bench()
    c = bench.ClockSampler(0)
    t0 = 1_900_000_000.0
    rows = [_row(t0 - 1.0, 345),  # idle, before the region
            _row(t0 + 0.01, 2070), _row(t0 + 0.035, 2070),
            _row(t0 + 0.06, 2055, ("Not Active", "Not Active", "Not Active", "Active")),
            _row(t0 + 2.0, 400)]  # after
    with open(c.tmp.name, "w") as f:
        f.write("\n".join(rows) + "\n")
    c.t0, c.t1 = t0, t0 + 0.08
    s = c.summary()
    assert s["samples"] == 3 and s["window"] == "timed region"
    assert s["sm_mhz"] == 2070 and s["sm_max_mhz"] == 2070
    assert s["reasons"] == ["sw_power_cap"]


def test_clock_summary_without_samples_in_the_region(tmp_path):
    bench = _bench()
    c = bench.ClockSampler(0)
    t0 = 1_900_000_000.0
    with open(c.tmp.name, "w") as f:
        f.write(_row(t0 - 5.0, 2070) + "\n")
    c.t0, c.t1 = t0, t0 + 0.05
    s = c.summary()
    assert s["samples"] == 1 and s["window"] == "around the timed region"
    c2 = bench.ClockSampler(0)
    assert c2.summary()["samples"] == 0
