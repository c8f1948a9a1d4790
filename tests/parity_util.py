"""Shared helpers for the GPU-vs-oracle parity tests: small seeded scenes with
non-trivial deformation, and error measures."""
from __future__ import annotations

import numpy as np

from anisotropicelastoplasticity_gb300 import HybridSolver, scenes
from anisotropicelastoplasticity_gb300.solver import LevelSet

from oracle.oracle import Oracle


def perturbed(scene, seed: int, fscale=0.03, vscale=0.5, bscale=None, fpscale=0.01, qmax=0.2):
    """Give a scene random elastic/plastic deformation, velocities and APIC momenta
    so that every term of the step is exercised."""
    rng = np.random.default_rng(seed)
    ps = scene.particles.copy()
    n = len(ps)
    h = float(scene.grid.h.min())
    if bscale is None:
        bscale = vscale * h / 3.0
    ps.elastic_deformation_gradients = np.eye(3) + fscale * rng.standard_normal((n, 3, 3))
    ps.plastic_deformation_gradients = np.eye(3) + fpscale * rng.standard_normal((n, 3, 3))
    ps.velocities = ps.velocities + vscale * rng.standard_normal((n, 3))
    ps.affine_momenta = bscale * rng.standard_normal((n, 3, 3))
    ps.plastic_amount = qmax * rng.random(n)
    scene.particles = ps
    return scene


def small_scene(kind: str, seed: int = 7):
    if kind == "snow":
        sc = scenes.snow_block(n=6000, res=32, seed=seed)
    elif kind == "sand":
        sc = scenes.sand_column(n=12000, res=32, seed=seed)
    elif kind == "mixed":
        sc = scenes.snow_sand_collision(n=12000, res=32, seed=seed)
    elif kind == "boundary":
        # a slab hugging the low-x wall and the ground: stencils cut by the grid boundary
        sc = scenes.sand_column(n=4000, res=32, seed=seed)
        rng = np.random.default_rng(seed)
        x = sc.particles.positions
        x[:, 0] = 0.003 + 0.06 * rng.random(len(x))
        x[:, 2] = 0.004 + 0.1 * rng.random(len(x))
        sc.levelset = LevelSet.ground(0.04) | LevelSet.sphere([0.3, 0.5, 0.0], 0.12)
    else:
        raise ValueError(kind)
    return sc


def make_pair(scene, threads: int = 0):
    gpu = HybridSolver(scene.particles, scene.grid, scene.params)
    gpu.set_level_set(scene.levelset)
    orc = Oracle(scene.grid, scene.params, threads=threads)
    orc.set_particle_system(scene.particles)
    orc.set_level_set(scene.levelset)
    return gpu, orc


def max_rel(a, b, floor=1e-30):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), floor))


def mass_weighted_rel(v_gpu, v_orc, m):
    m = np.asarray(m)[:, None]
    return float((m * np.abs(v_gpu - v_orc)).sum() / max((m * np.abs(v_orc)).sum(), 1e-30))
