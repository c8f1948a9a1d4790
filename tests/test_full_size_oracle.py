"""The benchmark configurations at their own full sizes, GPU step against the FP64
oracle on identical seeded inputs (HybridSolver.cpp:867-989):

* the grid after the first step's P2G and after its grid update + collision;
* the particle (and cloth) state after 1 and after 10 steps;

on the 524,288-particle sand column (128^3), the 65,536-vertex cloth drape
(195,586 items, 128^3) and the 2,097,152-particle snow + sand collision (256^3).
The bounds are those of the res-32 parity suite (tests/test_parity_gpu.py,
tests/test_cloth_gpu.py) unless stated at the assertion; every measured
difference is printed.  The whole-run comparisons (mass, momentum and centre of
mass every 10 steps) are in tests/test_snow_block_full_run.py.
"""
import numpy as np
import pytest

from anisotropicelastoplasticity_gb300 import HybridSolver, capi, scenes

from oracle.oracle import Oracle

from .parity_util import mass_weighted_rel, max_rel

pytestmark = pytest.mark.gpu

CONFIGS = {"sand_column": scenes.sand_column, "cloth_drape": scenes.cloth_drape,
           "snow_sand_collision": scenes.snow_sand_collision}
SIZES = {"sand_column": 524288, "cloth_drape": 195586, "snow_sand_collision": 2097152}


def _pair(sc):
    gpu = HybridSolver(sc.particles, sc.grid, sc.params)
    orc = Oracle(sc.grid, sc.params)
    if sc.mesh is not None:
        gpu.set_lagrangian_mesh(sc.mesh)
        orc.set_lagrangian_mesh(sc.mesh)
    if sc.particles is not None:
        orc.set_particle_system(sc.particles)
    gpu.set_level_set(sc.levelset)
    orc.set_level_set(sc.levelset)
    return gpu, orc


def _vel_errors(vg, vo):
    """Velocity differences relative to the largest velocity: the largest, the 99th
    percentile and the mean (the mean is the mass-weighted one for equal masses)."""
    d = np.abs(vg - vo).max(axis=1) / max(np.abs(vo).max(), 1e-30)
    return float(d.max()), float(np.percentile(d, 99)), float(d.mean())


def _particle_errors(gp, op, h):
    bscale = max(np.abs(op["affine_momenta"]).max(), np.abs(op["velocities"]).max() * h)
    vmax, v99, vmean = _vel_errors(gp["velocities"], op["velocities"])
    dB = np.abs(gp["affine_momenta"] - op["affine_momenta"]).max(axis=(1, 2)) / bscale
    return {"x": float(np.abs(gp["positions"] - op["positions"]).max()), "v_max": vmax, "v_p99": v99,
            "v_mean": vmean,
            "F": float(np.abs(gp["elastic_deformation_gradients"] - op["elastic_deformation_gradients"]).max()),
            "B_max": float(dB.max()), "B_p99": float(np.percentile(dB, 99)),
            "q": float(np.abs(gp["plastic"] - op["plastic"]).max())}


def _mesh_errors(gm, om):
    vs = np.abs(om["vertex_velocities"]).max() / 32
    vmax, v99, vmean = _vel_errors(np.concatenate([gm["vertex_velocities"], gm["element_velocities"]]),
                                   np.concatenate([om["vertex_velocities"], om["element_velocities"]]))
    return {"x": float(max(np.abs(gm["vertex_positions"] - om["vertex_positions"]).max(),
                           np.abs(gm["element_positions"] - om["element_positions"]).max())),
            "v_max": vmax, "v_p99": v99, "v_mean": vmean,
            "d": float(np.abs(gm["element_directions"] - om["element_directions"]).max()),
            "B": float(max(np.abs(gm["vertex_affine_momenta"] - om["vertex_affine_momenta"]).max(),
                           np.abs(gm["element_affine_momenta"] - om["element_affine_momenta"]).max()) / vs)}


@pytest.mark.parametrize("name", sorted(CONFIGS))
def test_first_step_grid_matches_oracle_at_full_size(name):
    sc = CONFIGS[name]()
    assert sc.num_items() == SIZES[name]
    for stage in (capi.AEP_STAGE_P2G, capi.AEP_STAGE_GRID):
        gpu, orc = _pair(sc)
        gpu.step_stage(sc.dt, stage)
        orc.init(volumes=False)
        if stage != capi.AEP_STAGE_P2G:
            orc.step(sc.dt, stage=stage)
        g, o = gpu.get_grid(), orc.get_grid()
        gpu.close()
        orc.close()
        dm = max_rel(g["masses"], o["masses"])
        dv = mass_weighted_rel(g["velocities"], o["velocities"], o["masses"])
        msg = f"{name} stage {stage}: mass {dm:.3g}, velocity {dv:.3g}"
        dvb = 0.0
        if stage == capi.AEP_STAGE_GRID:
            dvb = mass_weighted_rel(g["velocities_before_friction"], o["velocities_before_friction"], o["masses"])
            msg += f", before friction {dvb:.3g}"
        print(msg)
        # node masses to FP32 summation (a run of particles sharing a base node sums its
        # weights in FP32 before the fixed-point flush: up to ~40 terms at 256^3,
        # measured 2.5e-6 on the collision); mass-weighted velocities as in the res-32 suite
        assert dm < 5e-6, msg
        assert dv < (2e-5 if stage == capi.AEP_STAGE_P2G else 1e-4), msg
        assert dvb < 1e-4, msg


@pytest.mark.parametrize("name", sorted(CONFIGS))
def test_one_and_ten_steps_match_oracle_at_full_size(name):
    sc = CONFIGS[name]()
    gpu, orc = _pair(sc)
    gpu.init_volumes()
    orc.init(volumes=True)
    h = float(sc.grid.h.min())
    found = {}
    for k in range(1, 11):
        gpu.step(sc.dt)
        orc.step(sc.dt)
        if k not in (1, 10):
            continue
        if sc.particles is not None:
            e = _particle_errors(gpu.get_particles(), orc.get_particles(), h)
            found[(k, "particles")] = e
            print(f"{name} step {k} particles: " + ", ".join(f"{a} {b:.3g}" for a, b in e.items()))
        if sc.mesh is not None:
            e = _mesh_errors(gpu.get_mesh(), orc.get_mesh())
            found[(k, "cloth")] = e
            print(f"{name} step {k} cloth: " + ", ".join(f"{a} {b:.3g}" for a, b in e.items()))
    # bounds: positions, deformation and plastic state as in the res-32 parity suite;
    # velocities by their mean and 99th percentile relative to the largest velocity
    # (a scene at rest moves at g dt per step, and a grid node at the ground whose
    # normal velocity is ~0 takes the collision branch in one precision and not the
    # other, so the largest single difference is not a measure of the step)
    for (k, part), e in found.items():
        if part == "particles":
            tol = {"x": 5e-7, "F": 2e-6, "q": 2e-6, "v_mean": 1e-4, "v_p99": 1e-3, "B_p99": 1e-3} if k == 1 else \
                {"x": 1e-6, "F": 1e-5, "q": 1e-5, "v_mean": 2e-4, "v_p99": 2e-3, "B_p99": 2e-3}
        else:
            # element directions: measured 2.8e-5 at step 1 and the same at step 10 on the
            # 130,050-element drape (a few elements of the jittered sheet; the res-32
            # sheets stay below 5e-6)
            tol = {"x": 5e-7, "d": 1e-4, "v_mean": 1e-4, "v_p99": 1e-3} if k == 1 else \
                {"x": 2e-6, "d": 1e-4, "v_mean": 2e-4, "v_p99": 2e-3}
        for key, bound in tol.items():
            assert e[key] < bound, (name, k, part, key, e)
    assert gpu.stats()["overflow"] == 0
    gpu.close()
    orc.close()
