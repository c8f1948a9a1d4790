"""Precision of the sand return mapping near the Drucker-Prager apex
(HybridSolver.cpp:632-674) and the per-particle stress error of the step
against the FP64 oracle.

The step computes the return mapping in the stretch form (the trial stretch
F_tr^T F_tr - I resolved below FP32's spacing near 1, ln s = log1p(lam)/2 and
F_E = F + a small correction, rounded once).  These tests place sand states on
both sides of the switch between the cone and the apex (tr ln s = 0) and inside
the elastic region, and compare one step with the oracle, with the FP32 mapping
and with the option that redoes mappings near the apex in FP64
(aep_params.fp64_apex).  The stress measure is |P_gpu - P_fp64| per particle
relative to max(|P_fp64|, 1% of the rms stress), the measure of the benchmark.
"""
import numpy as np
import pytest

from anisotropicelastoplasticity_gb300 import HybridSolver, make_params, scenes

from oracle.oracle import Oracle
from oracle.stress import rel_stats, stress

from .parity_util import perturbed, small_scene

pytestmark = pytest.mark.gpu


def _rotations(rng, n):
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    return np.stack([np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
                     np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
                     np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1)], 1)


# tr ln s = c |dev ln s|: the cone projects when |dev| + k alpha tr > 0 (k alpha ~ 1.25 at
# q = 0), the apex takes tr > 0; c = -2 is elastic, -0.5 on the cone, +-1e-4 at the switch
SWITCH_SIDES = [-2.0, -0.5, -1e-4, 1e-4, 0.5]


def _fp32_inputs(ps):
    """Round the state to FP32 values, so that the GPU and the oracle start from
    identical numbers (the GPU stores FP32)."""
    for k in ("positions", "velocities", "affine_momenta", "elastic_deformation_gradients", "masses",
              "plastic_amount"):
        setattr(ps, k, getattr(ps, k).astype(np.float32).astype(np.float64))
    return ps


def _floor(o, mat, prm):
    """The oracle's state rounded to FP32: the error any FP32 state carries."""
    f = np.float32
    return stress(o["elastic_deformation_gradients"].astype(f), o["plastic"].astype(f), mat, prm,
                  o["volumes"].astype(f))


def _switch_scene(seed):
    sc = small_scene("sand", seed=seed)
    ps = sc.particles.copy()
    n = len(ps)
    rng = np.random.default_rng(seed)
    c = np.array(SWITCH_SIDES)[rng.integers(0, len(SWITCH_SIDES), n)]
    dev = rng.standard_normal((n, 3))
    dev -= dev.mean(axis=1, keepdims=True)
    dev /= np.linalg.norm(dev, axis=1, keepdims=True)
    mag = 10.0 ** rng.uniform(-4, -2, n)
    ln = mag[:, None] * dev + (c * mag / 3.0)[:, None]
    R1, R2 = _rotations(rng, n), _rotations(rng, n)
    ps.elastic_deformation_gradients = R1 @ (np.exp(ln)[:, :, None] * R2)
    ps.plastic_amount = 0.1 * rng.random(n)
    sc.particles = _fp32_inputs(ps)
    return sc, c


@pytest.mark.parametrize("fp64_apex", [0, 1])
def test_states_on_both_sides_of_the_apex_switch_match_oracle(fp64_apex):
    sc, c = _switch_scene(seed=5)
    prm = make_params(friction=0.5, fp64_apex=fp64_apex)
    gpu = HybridSolver(sc.particles, sc.grid, prm)
    gpu.set_level_set(sc.levelset)
    orc = Oracle(sc.grid, prm)
    orc.set_particle_system(sc.particles)
    orc.set_level_set(sc.levelset)
    gpu.init_volumes()
    orc.init(volumes=True)
    gpu.step(sc.dt)
    orc.step(sc.dt)
    st = gpu.stats()
    g, o = gpu.get_particles(), orc.get_particles()
    if fp64_apex:
        assert st["fp64_apex"] > 0
    else:
        assert st["fp64_apex"] == 0
    # F_E within a few units of FP32's spacing of the oracle's, on every side of the switch
    dF = np.abs(g["elastic_deformation_gradients"] - o["elastic_deformation_gradients"]).max(axis=(1, 2))
    for side in SWITCH_SIDES:
        sel = c == side
        assert dF[sel].max() < 6e-7, (side, dF[sel].max())
    # the plastic amount (its increment is continuous across the switch)
    assert np.abs(g["plastic"] - o["plastic"]).max() < 2e-6
    mat = sc.particles.material
    ref = stress(o["elastic_deformation_gradients"], o["plastic"], mat, prm, o["volumes"])
    err = rel_stats(stress(g["elastic_deformation_gradients"], g["plastic"], mat, prm, g["volumes"]), ref)
    floor = rel_stats(_floor(o, mat, prm), ref)
    print(f"fp64_apex={fp64_apex}: stress error p99 {err['p99']:.3e} max {err['max']:.3e}; "
          f"FP32-state floor p99 {floor['p99']:.3e}; max |dF| {dF.max():.3e}")
    # This scene's strains span 1e-4..1e-2, so its smallest stresses sit at the 1%-of-rms
    # floor of the measure and merely storing the oracle's state in FP32 costs ~2e-3 at
    # p99 (measured 2.34e-3; the GPU's error measured 2.34e-3 as well): the bound is
    # the floor itself, with 20% room.
    assert err["p99"] < 1.2 * floor["p99"] and err["median"] < 1.2 * floor["median"], (err, floor)


def test_stress_error_of_strained_snow_and_sand_after_five_steps():
    """The benchmark's error sample at test size: snow and sand with +-1% random
    elastic strain (every particle stressed, both return mappings active), five
    steps, per-particle stress error at p99 against the FP64 oracle, per material."""
    sc = scenes.snow_sand_collision(n=16384, res=64, seed=3)
    rng = np.random.default_rng(11)
    ps = sc.particles
    ps.elastic_deformation_gradients = np.eye(3) + 0.01 * rng.standard_normal((len(ps), 3, 3))
    _fp32_inputs(ps)
    gpu = HybridSolver(ps, sc.grid, sc.params)
    gpu.set_level_set(sc.levelset)
    orc = Oracle(sc.grid, sc.params)
    orc.set_particle_system(ps)
    orc.set_level_set(sc.levelset)
    gpu.init_volumes()
    orc.init(volumes=True)
    for _ in range(5):
        gpu.step(sc.dt)
        orc.step(sc.dt)
    g, o = gpu.get_particles(), orc.get_particles()
    mat = ps.material
    pg = stress(g["elastic_deformation_gradients"], g["plastic"], mat, sc.params, g["volumes"])
    po = stress(o["elastic_deformation_gradients"], o["plastic"], mat, sc.params, o["volumes"])
    pf = _floor(o, mat, sc.params)
    for m in (0, 1):
        e = rel_stats(pg[mat == m], po[mat == m])
        f = rel_stats(pf[mat == m], po[mat == m])
        print(f"material {m}: step-5 stress error p99 {e['p99']:.3e} max {e['max']:.3e}; "
              f"FP32-state floor p99 {f['p99']:.3e}")
        assert e["p99"] < 1e-3, (m, e, f)


def test_fp64_apex_option_changes_only_near_apex_states():
    """With the option, states far from the apex take the same FP32 mapping bit for bit."""
    sc = perturbed(small_scene("mixed"), seed=23)
    outs = []
    for flag in (0, 1):
        prm = make_params(friction=0.5, fp64_apex=flag)
        gpu = HybridSolver(sc.particles, sc.grid, prm)
        gpu.set_level_set(sc.levelset)
        gpu.step(sc.dt)
        outs.append(gpu.get_particles())
    snow = sc.particles.material == 0
    for k in ("elastic_deformation_gradients", "plastic", "positions"):
        assert np.array_equal(outs[0][k][snow], outs[1][k][snow]), k
