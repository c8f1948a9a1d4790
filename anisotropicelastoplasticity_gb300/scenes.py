"""Seeded synthetic scenes for the benchmark configurations.

The reference builds its scenes with unseeded rand()/time(0) generators
(ParticleSystem.cpp:119-401); these generators are new and seeded (numpy PCG64).
All scenes use the reference's frame: gravity along -z and the ground level
set on x[2] (HybridSolver.cpp:457, LevelSet.cpp:8-16).  A configuration stated
with y up is rotated to z up (the solids are isotropic and gravity and the
ground plane rotate together, so the dynamics are the same).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import capi
from .solver import LagrangianMesh, LevelSet, ParticleSystem, RegularGrid, make_params


@dataclass
class Scene:
    name: str
    grid: RegularGrid
    particles: ParticleSystem | None
    levelset: LevelSet
    params: capi.aep_params
    dt: float
    steps: int
    note: str = ""
    mesh: LagrangianMesh | None = None

    def num_items(self) -> int:
        n = len(self.particles) if self.particles is not None else 0
        if self.mesh is not None:
            n += len(self.mesh.vertex_positions) + len(self.mesh.faces)
        return n


def _block(rng, n, lo, hi):
    lo, hi = np.asarray(lo, float), np.asarray(hi, float)
    return lo + rng.random((n, 3)) * (hi - lo)


def _particles(x, v, m, vol, mat):
    n = len(x)
    return ParticleSystem(positions=x, velocities=v, masses=m, volumes=vol,
                          elastic_deformation_gradients=np.tile(np.eye(3), (n, 1, 1)),
                          plastic_deformation_gradients=np.tile(np.eye(3), (n, 1, 1)),
                          affine_momenta=np.zeros((n, 3, 3)), plastic_amount=np.zeros(n),
                          material=np.full(n, mat, dtype=np.uint8) if np.isscalar(mat) else mat)


def snow_block(n: int = 32768, res: int = 64, seed: int = 0, track_plastic_F: bool = False) -> Scene:
    """Plain snow block drop: 32,768 particles in [0.375, 0.625]^3 of a 64^3 grid over
    [0,1]^3, 8 per cell, velocity 1 m/s towards the ground, snow E=1.4e5, nu=0.2,
    theta_c=2.5e-2, theta_s=7.5e-3, xi=10, density 400, ground at 0.05 with mu=0.2,
    dt=1e-4, 200 steps."""
    rng = np.random.default_rng(seed)
    x = _block(rng, n, [0.375] * 3, [0.625] * 3)
    side = 0.25
    m = np.full(n, 400.0 * side ** 3 / n)
    v = np.tile([0.0, 0.0, -1.0], (n, 1))
    ps = _particles(x, v, m, m / 400.0, capi.AEP_SNOW)
    prm = make_params(friction=0.2, track_plastic_F=int(track_plastic_F))
    return Scene("snow_block", RegularGrid([0, 0, 0], [1, 1, 1], [res] * 3), ps, LevelSet.ground(0.05), prm,
                 1e-4, 200, "quadratic stencil in the configuration text; the reference is cubic (interpolation.cpp:9-33)")


def sand_column(n: int = 524288, res: int = 128, seed: int = 1) -> Scene:
    """Sand column collapse: 524,288 particles in a cylinder r=0.1, height 0.4 on the
    ground at 0.05, axis at x=y=0.5, grid 128^3, Drucker-Prager sand E=3.537e5,
    nu=0.3, friction angle 35 deg (h0), density 2200, ground mu=0.5, dt=5e-5, 1000 steps."""
    rng = np.random.default_rng(seed)
    r = 0.1 * np.sqrt(rng.random(n))
    th = 2.0 * np.pi * rng.random(n)
    z = 0.05 + 0.4 * rng.random(n)
    x = np.stack([0.5 + r * np.cos(th), 0.5 + r * np.sin(th), z], axis=1)
    vol_total = np.pi * 0.1 ** 2 * 0.4
    m = np.full(n, 2200.0 * vol_total / n)
    ps = _particles(x, np.zeros((n, 3)), m, m / 2200.0, capi.AEP_SAND)
    prm = make_params(friction=0.5, sand_h0=35.0)
    return Scene("sand_column", RegularGrid([0, 0, 0], [1, 1, 1], [res] * 3), ps, LevelSet.ground(0.05), prm,
                 5e-5, 1000, f"{n / (vol_total * res ** 3):.1f} particles per cell at this N")


def snow_sand_collision(n: int = 2097152, res: int = 256, seed: int = 3) -> Scene:
    """Mixed snow and sand at scale: half snow (snow-block material, density 400), half
    sand (sand-column material, density 2200) in two cubes of 8 particles per cell,
    colliding at relative speed 2; grid 256^3.  The cubes are placed face to face
    along x (the impact starts at the first step), each shifted at random (seed 3)
    by up to +-0.02 in y and z."""
    rng = np.random.default_rng(seed)
    nh = n // 2
    side = (nh / 8.0) ** (1.0 / 3.0) / res
    c_snow = np.array([0.5 - side / 2, 0.50, 0.30]) + 0.04 * (rng.random(3) - 0.5) * np.array([0, 1, 1])
    c_sand = np.array([0.5 + side / 2, 0.50, 0.30]) + 0.04 * (rng.random(3) - 0.5) * np.array([0, 1, 1])
    xs = _block(rng, nh, c_snow - side / 2, c_snow + side / 2)
    xd = _block(rng, n - nh, c_sand - side / 2, c_sand + side / 2)
    x = np.concatenate([xs, xd])
    v = np.concatenate([np.tile([1.0, 0, 0], (nh, 1)), np.tile([-1.0, 0, 0], (n - nh, 1))])
    m = np.concatenate([np.full(nh, 400.0 * side ** 3 / nh), np.full(n - nh, 2200.0 * side ** 3 / (n - nh))])
    vol = np.concatenate([np.full(nh, side ** 3 / nh), np.full(n - nh, side ** 3 / (n - nh))])
    mat = np.concatenate([np.full(nh, capi.AEP_SNOW, np.uint8), np.full(n - nh, capi.AEP_SAND, np.uint8)])
    ps = _particles(x, v, m, vol, mat)
    prm = make_params(friction=0.5)
    return Scene("snow_sand_collision", RegularGrid([0, 0, 0], [1, 1, 1], [res] * 3), ps, LevelSet.ground(0.05),
                 prm, 5e-5, 500)


def sheet(nside: int, side: float, center_xy, height: float, jitter: float, rng):
    """nside x nside vertex square sheet in the plane z = height, two triangles per quad."""
    t = np.linspace(-side / 2, side / 2, nside)
    X, Y = np.meshgrid(center_xy[0] + t, center_xy[1] + t, indexing="ij")
    V = np.stack([X.ravel(), Y.ravel(), np.full(X.size, height)], axis=1)
    V += rng.uniform(-jitter, jitter, V.shape)
    idx = np.arange(nside * nside).reshape(nside, nside)
    a, b, c, d = idx[:-1, :-1].ravel(), idx[1:, :-1].ravel(), idx[1:, 1:].ravel(), idx[:-1, 1:].ravel()
    F = np.concatenate([np.stack([a, b, c], 1), np.stack([a, c, d], 1)]).astype(np.int32)
    return V, F


def cloth_drape(nside: int = 256, res: int = 128, seed: int = 2, shear_stiffness: float = 1e3) -> Scene:
    """Cloth drape: a 256x256-vertex square sheet (65,536 vertices, 130,050 triangles) of
    side 0.6, flat at height 0.7, vertex positions jittered +-1e-4 (seed 2); in-plane
    E=1e4, nu=0.3, normal stiffness 1e3, frictional cap 0.3, mass 0.2 per unit area;
    sphere r=0.2 at (0.5, 0.5, 0.4) plus the ground; grid 128^3, dt=2e-5, 2000 steps."""
    rng = np.random.default_rng(seed)
    V, F = sheet(nside, 0.6, (0.5, 0.5), 0.7, 1e-4, rng)
    thickness = 1.0 / res
    mesh = LagrangianMesh.from_triangles(V, F, density=0.2 / thickness, thickness=thickness, youngs_modulus=1e4,
                                         poisson_ratio=0.3, shear_stiffness=shear_stiffness, stiffness=1e3,
                                         friction_coeff=0.3)
    ls = LevelSet.sphere([0.5, 0.5, 0.4], 0.2) | LevelSet.ground(0.05)
    # The reference's in-plane vertex forces carry no element volume
    # (LagrangianMesh.cpp:452-458); with E = 1e4 on this mesh they would be ~1e6 times
    # too stiff for dt = 2e-5, so this scene weights them by the element volume.
    prm = make_params(cloth_volume_weighting=1)
    return Scene("cloth_drape", RegularGrid([0, 0, 0], [1, 1, 1], [res] * 3), None, ls, prm, 2e-5, 2000,
                 f"thickness {thickness:g} (density x thickness = 0.2 per area); shear stiffness "
                 f"{shear_stiffness:g} (not given by the configuration); in-plane forces weighted by the "
                 f"element volume", mesh)


def sand_cloth(nside: int = 512, n_sand: int = 7604222, res: int = 512, seed: int = 4) -> Scene:
    """Sand and cloth at scale: 7,604,222 sand particles in a cylinder r=0.12, height
    0.16 on the ground at 0.05 (about 8 per cell at 512^3), under a 512x512-vertex
    sheet (262,144 vertices, 522,242 triangles) of side 0.6 at height 0.3 that falls
    onto the pile; sand as in the sand column, cloth as in the drape (in-plane E=1e4,
    volume-weighted in-plane forces); grid 512^3, dt=2e-5, 500 steps."""
    rng = np.random.default_rng(seed)
    r = 0.12 * np.sqrt(rng.random(n_sand))
    th = 2.0 * np.pi * rng.random(n_sand)
    z = 0.05 + 0.16 * rng.random(n_sand)
    x = np.stack([0.5 + r * np.cos(th), 0.5 + r * np.sin(th), z], axis=1)
    vol_total = np.pi * 0.12 ** 2 * 0.16
    m = np.full(n_sand, 2200.0 * vol_total / n_sand)
    ps = _particles(x, np.zeros((n_sand, 3)), m, m / 2200.0, capi.AEP_SAND)
    V, F = sheet(nside, 0.6, (0.5, 0.5), 0.3, 1e-4, rng)
    thickness = 1.0 / res
    mesh = LagrangianMesh.from_triangles(V, F, density=0.2 / thickness, thickness=thickness, youngs_modulus=1e4,
                                         poisson_ratio=0.3, shear_stiffness=1e3, stiffness=1e3, friction_coeff=0.3)
    prm = make_params(friction=0.5, cloth_volume_weighting=1)
    return Scene("sand_cloth", RegularGrid([0, 0, 0], [1, 1, 1], [res] * 3), ps, LevelSet.ground(0.05), prm, 2e-5,
                 500, f"{n_sand / (vol_total * res ** 3):.1f} sand particles per cell; cloth as in the drape", mesh)


# --- the reference's particle factories (ParticleSystem.cpp:119-401), seeded ---------
# Rejection sampling of the unit ball / disk, the total mass spread evenly, volumes 1
# (the first P2G of solve recomputes them), F_E = F_P = I.  The C++ facade
# (include/aep/hybrid_solver.hpp) has the same factories on std::mt19937_64.

def _unit_ball(rng, n, dim):
    out = np.empty((0, dim))
    while len(out) < n:
        c = rng.uniform(-1.0, 1.0, (2 * (n - len(out)) + 16, dim))
        out = np.concatenate([out, c[np.linalg.norm(c, axis=1) <= 1.0]])
    return out[:n]


def snow_ball(center, radius: float, n: int, seed: int = 0) -> ParticleSystem:
    """SnowBall (ParticleSystem.cpp:119-183): total mass 100 * 3.14 r^3, snow."""
    x = np.asarray(center, float) + radius * _unit_ball(np.random.default_rng(seed), n, 3)
    return _particles(x, np.zeros((n, 3)), np.full(n, 100.0 * 3.14 * radius ** 3 / n), np.ones(n), capi.AEP_SNOW)


def sand_ball(center, radius: float, n: int, seed: int = 0) -> ParticleSystem:
    """SandBall (ParticleSystem.cpp:185-247): total mass 1300 * 3.14 r^3, sand."""
    x = np.asarray(center, float) + radius * _unit_ball(np.random.default_rng(seed), n, 3)
    return _particles(x, np.zeros((n, 3)), np.full(n, 1300.0 * 3.14 * radius ** 3 / n), np.ones(n), capi.AEP_SAND)


def sand_block(bmin, bmax, hole_radius: float, n: int, seed: int = 0) -> ParticleSystem:
    """SandBlock (ParticleSystem.cpp:249-329): uniform in the box minus the ball of
    hole_radius at (bmin.x, bmin.y, mid z); total mass 1300 (box volume - pi R^3 / 4)."""
    lo, hi = np.asarray(bmin, float), np.asarray(bmax, float)
    if hole_radius * 2.0 >= hi[2] - lo[2]:
        raise ValueError("SandBlock: the hole is too big")
    hc = np.array([lo[0], lo[1], 0.5 * (lo[2] + hi[2])])
    rng = np.random.default_rng(seed)
    x = np.empty((0, 3))
    while len(x) < n:
        c = _block(rng, 2 * (n - len(x)) + 16, lo, hi)
        x = np.concatenate([x, c[np.linalg.norm(c - hc, axis=1) >= hole_radius]])
    total = 1300.0 * (np.prod(hi - lo) - 0.25 * np.pi * hole_radius ** 3)
    return _particles(x[:n], np.zeros((n, 3)), np.full(n, total / n), np.ones(n), capi.AEP_SAND)


def sand_cylinder(base_center, radius: float, height: float, n: int, seed: int = 0) -> ParticleSystem:
    """SandCylinder (ParticleSystem.cpp:331-401): disk x [0, height) above base_center,
    velocity (0, 0, -1), total mass 1300 pi r^2 h, sand."""
    rng = np.random.default_rng(seed)
    d = radius * _unit_ball(rng, n, 2)
    z = rng.uniform(0.0, height, n)
    x = np.asarray(base_center, float) + np.stack([d[:, 0], d[:, 1], z], axis=1)
    v = np.zeros((n, 3))
    v[:, 2] = -1.0
    return _particles(x, v, np.full(n, 1300.0 * np.pi * radius ** 2 * height / n), np.ones(n), capi.AEP_SAND)


CONFIGS = {0: snow_block, 1: sand_column, 2: cloth_drape, 3: snow_sand_collision, 4: sand_cloth}
