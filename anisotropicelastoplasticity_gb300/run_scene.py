"""Run one of the seeded scenes for a number of steps and print one JSON line with
the step time and the per-kernel CUDA-event times:

    python -m anisotropicelastoplasticity_gb300.run_scene cloth_drape --steps 20
    python -m anisotropicelastoplasticity_gb300.run_scene sand_cloth --arg res=256 --arg nside=256 --arg n_sand=950000

Scenes: snow_block (32,768 particles, 64^3), sand_column (524,288, 128^3),
cloth_drape (65,536 vertices + 130,050 elements, 128^3), snow_sand_collision
(2,097,152, 256^3), sand_cloth (8,388,608 items, 512^3).  The steps are timed
twice: once with a start and an end event each, then again with the library's
events between its kernels (which add a few microseconds per step) for the
per-kernel times.  `--arg name=value` passes a size argument to the scene's
factory (scenes.py), for a smaller case of the same scene.  `--learned STEPS`
runs the learned return map instead of the exact one: the network is trained for
STEPS Adam steps on the exact mappings of 20 plain steps of the same scene (a
separate run, harvested first) and checked with the strict bound (1e-4 of the
predicted strain)."""
import argparse
import json
import sys

from . import HybridSolver, scenes

SCENES = {
    "snow_block": scenes.snow_block,
    "sand_column": scenes.sand_column,
    "cloth_drape": scenes.cloth_drape,
    "snow_sand_collision": scenes.snow_sand_collision,
    "sand_cloth": scenes.sand_cloth,
}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("scene", choices=sorted(SCENES))
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--arg", action="append", default=[], metavar="NAME=VALUE",
                    help="integer size argument of the scene factory (n, res, nside, n_sand, seed)")
    ap.add_argument("--learned", type=int, default=None, metavar="STEPS",
                    help="learned return map, trained for STEPS steps on the scene's own exact mappings")
    args = ap.parse_args(argv)
    kw = {}
    for a in args.arg:
        name, _, value = a.partition("=")
        if name not in ("n", "res", "nside", "n_sand", "seed") or not value.lstrip("-").isdigit():
            ap.error(f"bad --arg {a!r}")
        kw[name] = int(value)
    import torch

    mlp = None
    if args.learned is not None:
        from .learned import ReturnMapMLP, harvest_records

        recs = harvest_records(SCENES[args.scene](**kw), steps=20, capacity=2000000, stride=1)
        mlp = ReturnMapMLP(seed=0)
        if args.learned > 0 and len(recs) > 0:  # a scene at rest may have no plastic state yet
            mlp.train(recs.data_ptr(), len(recs), steps=args.learned, batch=8192, lr=2e-3, lr_final=2e-5)
        del recs
        torch.cuda.empty_cache()
    sc = SCENES[args.scene](**kw)
    s = HybridSolver(sc.particles, sc.grid, sc.params)
    if mlp is not None:
        s.set_return_map(mlp, 1e-4)
    if sc.mesh is not None:
        s.set_lagrangian_mesh(sc.mesh)
    s.set_level_set(sc.levelset)
    stream = torch.cuda.Stream()
    s.set_stream(stream.cuda_stream)
    s.init_volumes()
    for _ in range(args.warmup):
        s.step(sc.dt)
    s.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with torch.cuda.stream(stream):
        for a, b in ev:
            a.record(stream)
            s.step(sc.dt)
            b.record(stream)
    s.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in ev) / max(args.steps, 1)
    s.set_profiling(True)
    for _ in range(args.steps):
        s.step(sc.dt)
    s.synchronize()
    phases, k = s.phase_times()
    s.set_profiling(False)
    st = s.stats()
    s.close()
    items = sc.num_items()
    print(json.dumps({
        "scene": args.scene, "items": items, "grid": [int(r) for r in sc.grid.resolution], "dt": sc.dt,
        "steps": args.steps, "ms_per_step": ms, "item_steps_per_s": items / (ms * 1e-3),
        "phases_ms_per_step": {p: v / max(k, 1) for p, v in phases.items()},
        "active_nodes": st["active_nodes"], "fp64_fallbacks_last_step": st["fp64_fallbacks"],
        "total_mass": st["total_mass"],
        "return_map": "exact" if mlp is None else "learned",
        "learned_accepted_last_step": st["learned_accepted"], "learned_fallbacks_last_step": st["learned_fallbacks"],
    }))
    if mlp is not None:
        mlp.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
