"""Benchmark of the GB300 MPM step: particle-steps/s on the sand-column collapse
(524,288 Drucker-Prager particles, 128^3 grid, dt = 5e-5), one GPU per rank.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`value` is device throughput with the particle state resident in HBM; `e2e` is
the same metric through the C-ABI with host buffers (pinned), the host->device
upload and the device->host readback of the particle state inside every timed
step.  The reference arm (`--impl reference`) runs the FP64 CPU restatement of
the reference step (oracle/) on all host cores, because the reference itself
(an MSVC application on Eigen + libigl) cannot be built here.  Multi-GPU runs
are independent replicas (the step has no data exchange between GPUs).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "particle-steps/s, learned vs plain return map, 1 GB300, at <=1e-3 stress error"
UNIT = "particle-steps/s"
L2_FLUSH_BYTES = 512 << 20  # > 129 MB L2


def algorithmic_bytes(phase: str, n_p: int, n_nodes: int) -> float:
    """Algorithmic bytes per launch (FP32 state, per-particle and per-node terms)."""
    per = {"p2g": (64, 32), "force": (56, 36), "g2p": (152, 24), "normalize": (0, 44), "grid": (0, 68)}
    a, b = per[phase]
    return a * n_p + b * n_nodes


def measured_peak_gbs():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.tmp, stderr=subprocess.DEVNULL)
        except (OSError, ValueError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        self.tmp.flush()

    def summary(self):
        try:
            rows = [r.split(",") for r in Path(self.tmp.name).read_text().strip().splitlines() if r.strip()]
        except OSError:
            rows = []
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if len(r) > 5 + i and "Active" in r[5 + i]
                          and "Not" not in r[5 + i]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def dist_env():
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    return rank, world, local


def make_scene(args):
    from anisotropicelastoplasticity_gb300 import scenes

    return scenes.sand_column(n=args.particles, res=args.res, seed=1)


def cpu_baseline(args, steps: int):
    """The oracle (FP64 restatement of the reference step) on all host cores, a bounded sample."""
    from oracle.oracle import Oracle

    sc = make_scene(args)
    orc = Oracle(sc.grid, sc.params, threads=os.cpu_count() or 1)
    orc.set_particle_system(sc.particles)
    orc.set_level_set(sc.levelset)
    orc.init(volumes=True)
    orc.step(sc.dt)  # warm-up
    t0 = time.perf_counter()
    for _ in range(steps):
        orc.step(sc.dt)
    dt = time.perf_counter() - t0
    return {"value": len(sc.particles) * steps / dt, "unit": UNIT, "cores": orc.threads, "kind": "port",
            "sample": f"{steps} full steps of the {len(sc.particles)}-particle sand column (128^3 grid), FP64, "
                      f"{orc.threads} OpenMP threads, after 1 warm-up step"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return None
    from oracle.oracle import Oracle

    sc = make_scene(args)
    orc = Oracle(sc.grid, sc.params, threads=os.cpu_count() or 1)
    orc.set_particle_system(sc.particles)
    orc.set_level_set(sc.levelset)
    orc.init(volumes=True)
    for _ in range(args.warmup):
        orc.step(sc.dt)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        orc.step(sc.dt)
    el = time.perf_counter() - t0
    v = len(sc.particles) * args.steps / el
    return {
        "metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded sand column)",
        "config": {"workload": "sand_column", "particles": len(sc.particles), "grid": [args.res] * 3,
                   "dt": sc.dt, "material": "drucker_prager_sand"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": orc.threads, "kind": "port",
                         "sample": f"{args.steps} full steps after {args.warmup} warm-up steps"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference (MSVC + Eigen + libigl) cannot be built here; this arm times oracle/, the FP64 "
                "C++ restatement of its step with the same sparse-matrix dataflow",
    }


def run_ours(args):
    import torch

    from anisotropicelastoplasticity_gb300 import HybridSolver
    from anisotropicelastoplasticity_gb300.solver import mats_to_ref, rows_to_ref, vec_to_ref  # noqa: F401

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    sc = make_scene(args)
    n_p = len(sc.particles)
    solver = HybridSolver(sc.particles, sc.grid, sc.params)
    solver.set_level_set(sc.levelset)
    stream = torch.cuda.Stream()
    solver.set_stream(stream.cuda_stream)
    solver.init_volumes()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        solver.step(sc.dt)
    solver.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()
        torch.cuda.synchronize()

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    solver.set_profiling(True)
    barrier()
    with ClockSampler(local) as clk:
        wall0 = time.perf_counter()
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                flush.zero_()  # L2 flush between timed steps (outside the events)
                starts[k].record(stream)
                solver.step(sc.dt)
                ends[k].record(stream)
        solver.synchronize()
        barrier()
        wall = time.perf_counter() - wall0
    ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    phase_ms, timed = solver.phase_times()
    solver.set_profiling(False)
    st = solver.stats()
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * n_p * args.steps / (ms * 1e-3)

    # roofline of the dominant kernel (CUDA events on the launching stream)
    per_launch = {k: v / max(timed, 1) for k, v in phase_ms.items()}
    dom = max(("p2g", "force", "g2p"), key=lambda k: per_launch[k])
    peak, peak_kind = measured_peak_gbs()
    nodes = int(st["active_nodes"])
    ach = algorithmic_bytes(dom, n_p, nodes) / (per_launch[dom] * 1e-3) / 1e9
    traffic = None
    tp = ROOT / "profiles" / "traffic.json"
    if tp.exists():
        try:
            t = json.loads(tp.read_text()).get(dom)
            if t:
                traffic = t["bytes_per_particle"] * n_p + t.get("bytes_per_node", 0.0) * nodes
        except Exception:
            traffic = None
    roofline = {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                "traffic": traffic, "peak_source": peak_kind,
                "kernels": {k: {"ms_per_launch": per_launch[k],
                                "algorithmic_GBps": (algorithmic_bytes(k, n_p, nodes) / (per_launch[k] * 1e-3) / 1e9)
                                if k in ("p2g", "force", "g2p", "normalize", "grid") else None}
                            for k in per_launch}}

    # end to end through the C-ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, solver, sc, stream)

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded sand column)",
        "config": {"workload": "sand_column", "particles": n_p, "grid": [args.res] * 3, "dt": sc.dt,
                   "material": "drucker_prager_sand", "return_map": "plain", "parallelism": f"replicas{world}",
                   "l2": "flushed between timed steps (512 MB write)", "active_nodes": nodes,
                   "active_blocks": int(st["active_blocks"])},
        "roofline": roofline,
        "gpu_launches": 5 * args.steps,
        "library_launches_note": "plus the CUB radix-sort kernels of each step's particle ordering",
        "fp64_fallbacks_last_step": int(st["fp64_fallbacks"]),
        "wall_s": wall,
    }
    out["clocks"] = clk.summary()
    if e2e is not None:
        out["e2e"] = e2e
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args, args.cpu_steps)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return out if rank == 0 else None


def run_e2e(args, solver, sc, stream):
    import torch

    n = len(sc.particles)
    ps = solver.sync()  # current state in the reference layout on the host

    def pinned(a):
        t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True)
        t.numpy()[...] = a
        return t.numpy()

    host = {
        "positions": pinned(ps.positions), "velocities": pinned(ps.velocities),
        "affine_momenta": pinned(ps.affine_momenta),
        "elastic_deformation_gradients": pinned(ps.elastic_deformation_gradients),
        "masses": pinned(ps.masses), "volumes": pinned(ps.volumes), "plastic_amount": pinned(ps.plastic_amount),
    }
    steps = max(1, min(args.steps, 10))
    import ctypes as C

    lib = solver._lib
    h = solver._h
    from anisotropicelastoplasticity_gb300.solver import mats_to_ref, rows_to_ref, vec_to_ref

    bufs = {
        "x": pinned(vec_to_ref(host["positions"])), "v": pinned(vec_to_ref(host["velocities"])),
        "B": pinned(rows_to_ref(host["affine_momenta"])), "F": pinned(mats_to_ref(host["elastic_deformation_gradients"])),
        "m": host["masses"], "vol": host["volumes"], "q": pinned(np.asarray(ps.plastic_amount, float)),
    }
    mat = np.ascontiguousarray(ps.material, np.uint8)
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    h2d = 8 * (3 + 3 + 9 + 9 + 1 + 1 + 1) * n + n
    d2h = 8 * (3 + 3 + 9 + 9 + 1 + 1) * n
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        st = lib.aep_set_particles(h, n, dp(bufs["x"]), dp(bufs["v"]), dp(bufs["B"]), dp(bufs["F"]), None,
                                   dp(bufs["m"]), dp(bufs["vol"]), dp(bufs["q"]),
                                   mat.ctypes.data_as(C.POINTER(C.c_uint8)))
        assert st == 0, st
        assert lib.aep_step(h, sc.dt) == 0
        st = lib.aep_get_particles(h, n, dp(bufs["x"]), dp(bufs["v"]), dp(bufs["B"]), dp(bufs["F"]), None,
                                   dp(bufs["vol"]), dp(bufs["q"]))
        assert st == 0, st
    el = time.perf_counter() - t0
    return {"value": n * steps / el, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "steps": steps, "path": "aep_set_particles + aep_step + aep_get_particles, pinned FP64 host arrays "
                                    "in the reference layouts"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--particles", type=int, default=524288)
    ap.add_argument("--res", type=int, default=128)
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    if args.impl == "reference":
        out = run_reference(args)
    else:
        out = run_ours(args)
    if out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
