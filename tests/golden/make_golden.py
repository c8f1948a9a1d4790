"""Generate the golden fixtures of tests/test_golden.py.

The reference ships no golden vectors and cannot be built here (Eigen/libigl are
absent), so these fixtures are outputs of the FP64 oracle (oracle/aep_oracle.cpp)
on small seeded scenes.  They pin the oracle against regressions and give the GPU
a fixed target that needs no oracle build.  Inputs are stored with the outputs.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from anisotropicelastoplasticity_gb300 import scenes  # noqa: E402
from anisotropicelastoplasticity_gb300.solver import LevelSet  # noqa: E402
from oracle.oracle import Oracle  # noqa: E402

HERE = Path(__file__).resolve().parent
STEPS = 3


def cases():
    rng = np.random.default_rng(1234)
    out = {}
    sc = scenes.snow_block(n=512, res=16, seed=5)
    ps = sc.particles
    ps.elastic_deformation_gradients = np.eye(3) + 0.02 * rng.standard_normal((len(ps), 3, 3))
    out["snow_block_512"] = sc
    sc = scenes.sand_column(n=768, res=16, seed=6)
    sc.particles.velocities = 0.3 * rng.standard_normal((len(sc.particles), 3))
    out["sand_column_768"] = sc
    sc = scenes.snow_sand_collision(n=768, res=16, seed=7)
    sc.levelset = LevelSet.ground(0.05) | LevelSet.sphere([0.5, 0.5, 0.0], 0.2)
    out["snow_sand_768"] = sc
    return out


def level_set_array(ls):
    arr = np.zeros((len(ls.shapes), 7))
    for i, (t, p) in enumerate(ls.shapes):
        arr[i, 0] = t
        arr[i, 1:] = p
    return arr


def main():
    for name, sc in cases().items():
        ps = sc.particles
        o = Oracle(sc.grid, sc.params, threads=1)
        o.set_particle_system(ps)
        o.set_level_set(sc.levelset)
        o.init(volumes=True)
        vol0 = o.get_particles()["volumes"]
        for _ in range(STEPS):
            o.step(sc.dt)
        r = o.get_particles()
        g = o.get_grid()
        np.savez_compressed(
            HERE / f"{name}.npz",
            grid_min=sc.grid.min_bound, grid_max=sc.grid.max_bound, grid_res=sc.grid.resolution,
            dt=sc.dt, steps=STEPS, friction=sc.params.friction, levelset=level_set_array(sc.levelset),
            x0=ps.positions, v0=ps.velocities, B0=ps.affine_momenta, F0=ps.elastic_deformation_gradients,
            Fp0=ps.plastic_deformation_gradients, m=ps.masses, q0=ps.plastic_amount, mat=ps.material,
            vol_init=vol0, x=r["positions"], v=r["velocities"], B=r["affine_momenta"],
            F=r["elastic_deformation_gradients"], plastic=r["plastic"], grid_mass=g["masses"])
        print(name, len(ps))


if __name__ == "__main__":
    main()
