"""The benchmark's bookkeeping, checked without a GPU or nvidia-smi: the clock
record (the samples nvidia-smi wrote inside the timed region are kept, by their
own timestamps, and the throttle reasons read from them) and the roofline's
algorithmic bytes and DRAM traffic."""
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


def test_roofline_of_the_learned_step_counts_its_queue_rows():
    """The dominant kernel's algorithmic bytes: the plain G2P's per-item state, plus,
    for the learned step, each queued row's queue entry instead of its F_E and
    plastic scalar; the DRAM traffic per item comes from the committed ncu table."""
    bench = _bench()
    counts = {"particles": 1000, "verts": 10, "elems": 20, "nodes": 300}
    plain = bench.algorithmic_bytes("g2p", counts)
    assert plain == 152 * 1010 + 24 * 300
    learned = bench.algorithmic_bytes("g2p_learned", dict(counts, rows=400))
    assert learned == plain + 400 * (84 + 8 - 40)
    arm = {"kernel_ms": {"p2g": 1.0, "force": 1.5, "g2p": 2.0, "mlp": 0.4}, "mlp_rows_last_step": 400,
           "workload": "sand_cloth", "profiled_ms_per_step": 5.0}
    r = bench.roofline_of(arm, counts)
    assert r["kernel"] == "g2p_learned"
    assert abs(r["achieved"] - learned / 2e-3 / 1e9) < 1e-9
    assert r["traffic"] is not None and r["traffic"] > 0
    arm_plain = dict(arm, mlp_rows_last_step=0)
    assert bench.roofline_of(arm_plain, counts)["kernel"] == "g2p"
