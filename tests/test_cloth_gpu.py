"""Cloth (LagrangianMesh) on the GPU against the FP64 oracle: grid forces with the
in-plane vertex forces and element normal stress (LagrangianMesh.cpp:382-460,
HybridSolver.cpp:370-455), grid after update + collision, and the mesh state after
1 and 10 steps (vertex G2P with damped APIC, element directions, cloth QR return
mapping, HybridSolver.cpp:684-722); a sheet alone and a sheet over sand."""
import numpy as np
import pytest

from anisotropicelastoplasticity_gb300 import HybridSolver, LagrangianMesh, LevelSet, capi, make_params, scenes
from anisotropicelastoplasticity_gb300.solver import RegularGrid

from oracle.oracle import Oracle

from .parity_util import mass_weighted_rel, max_rel

pytestmark = pytest.mark.gpu


def small_cloth(with_sand: bool, seed: int = 4, E: float = 5.0, weighting: int = 0):
    """A 20x20 sheet; with the reference's unweighted in-plane forces a soft in-plane
    modulus keeps the dynamics tame at dt = 2e-5."""
    rng = np.random.default_rng(seed)
    V, F = scenes.sheet(20, 0.6, (0.5, 0.5), 0.45, 1e-4, rng)
    mesh = LagrangianMesh.from_triangles(V, F, density=0.2 * 32, thickness=1 / 32, youngs_modulus=E,
                                         poisson_ratio=0.3, shear_stiffness=1e3, stiffness=1e3, friction_coeff=0.3)
    # deform: stretch/shear the sheet in plane and tilt / compress the normal direction
    mesh.vertex_positions = V @ np.array([[1.03, 0.02, 0.0], [0.0, 0.98, 0.0], [0.0, 0.0, 1.0]]).T
    mesh.vertex_positions[:, 2] += 0.01 * rng.standard_normal(len(V))
    Vp = mesh.vertex_positions
    D = mesh.element_directions.copy()
    D[:, :, 0] = Vp[F[:, 1]] - Vp[F[:, 0]]
    D[:, :, 1] = Vp[F[:, 2]] - Vp[F[:, 0]]
    D[:, :, 2] = 0.97 * D[:, :, 2] + 0.05 * rng.standard_normal((len(F), 3))
    mesh.element_directions = D
    mesh.vertex_velocities = 0.3 * rng.standard_normal((len(V), 3))
    mesh.element_velocities = mesh.vertex_velocities[F].mean(axis=1)
    grid = RegularGrid([0, 0, 0], [1, 1, 1], [32, 32, 32])
    ps = None
    if with_sand:
        sc = scenes.sand_column(n=6000, res=32, seed=seed)
        ps = sc.particles
        ps.positions[:, 2] = 0.1 + 0.3 * rng.random(len(ps))
        ps.velocities = 0.2 * rng.standard_normal((len(ps), 3))
    ls = LevelSet.sphere([0.5, 0.5, 0.3], 0.12) | LevelSet.ground(0.05)
    return grid, ps, mesh, ls, make_params(friction=0.3, cloth_volume_weighting=weighting)


def pair(grid, ps, mesh, ls, prm):
    gpu = HybridSolver(None, grid, prm)
    if ps is not None:
        gpu.set_particle_system(ps)
    gpu.set_lagrangian_mesh(mesh)
    gpu.set_level_set(ls)
    orc = Oracle(grid, prm)
    if ps is not None:
        orc.set_particle_system(ps)
    orc.set_lagrangian_mesh(mesh)
    orc.set_level_set(ls)
    return gpu, orc


@pytest.mark.parametrize("with_sand,E,weighting", [(False, 5.0, 0), (True, 5.0, 0), (False, 1e4, 1), (True, 1e4, 0)])
def test_cloth_forces_match_oracle(with_sand, E, weighting):
    grid, ps, mesh, ls, prm = small_cloth(with_sand, E=E, weighting=weighting)
    gpu, orc = pair(grid, ps, mesh, ls, prm)
    dt = 2e-5
    gpu.step_stage(dt, capi.AEP_STAGE_FORCES)
    g = gpu.get_grid()
    orc.init(volumes=False)
    orc.step(dt, stage=capi.AEP_STAGE_FORCES)
    o = orc.get_grid()
    f_orc = o["forces"] - o["masses"][:, None] * np.array(list(prm.gravity))
    assert max_rel(g["masses"], o["masses"]) < 2e-6
    assert max_rel(g["forces"], f_orc) < 5e-4


@pytest.mark.parametrize("with_sand", [False, True])
def test_cloth_grid_update_matches_oracle(with_sand):
    grid, ps, mesh, ls, prm = small_cloth(with_sand)
    gpu, orc = pair(grid, ps, mesh, ls, prm)
    dt = 2e-5
    gpu.step_stage(dt, capi.AEP_STAGE_GRID)
    g = gpu.get_grid()
    orc.init(volumes=False)
    orc.step(dt, stage=capi.AEP_STAGE_GRID)
    o = orc.get_grid()
    assert mass_weighted_rel(g["velocities"], o["velocities"], o["masses"]) < 1e-4
    assert mass_weighted_rel(g["velocities_before_friction"], o["velocities_before_friction"], o["masses"]) < 1e-4


def _compare_mesh(gm, om, pos_tol, vel_tol, dir_tol, B_tol):
    assert np.abs(gm["vertex_positions"] - om["vertex_positions"]).max() < pos_tol
    assert np.abs(gm["element_positions"] - om["element_positions"]).max() < pos_tol
    assert max_rel(gm["vertex_velocities"], om["vertex_velocities"]) < vel_tol
    assert max_rel(gm["element_velocities"], om["element_velocities"]) < vel_tol
    assert np.abs(gm["element_directions"] - om["element_directions"]).max() < dir_tol
    vs = np.abs(om["vertex_velocities"]).max() / 32
    assert np.abs(gm["vertex_affine_momenta"] - om["vertex_affine_momenta"]).max() / vs < B_tol
    assert np.abs(gm["element_affine_momenta"] - om["element_affine_momenta"]).max() / vs < B_tol


@pytest.mark.parametrize("with_sand", [False, True])
def test_cloth_one_step_matches_oracle(with_sand):
    grid, ps, mesh, ls, prm = small_cloth(with_sand)
    gpu, orc = pair(grid, ps, mesh, ls, prm)
    gpu.step(2e-5)
    orc.init(volumes=False)
    orc.step(2e-5)
    _compare_mesh(gpu.get_mesh(), orc.get_mesh(), 5e-7, 2e-4, 5e-6, 2e-3)
    if with_sand:
        gp, op = gpu.get_particles(), orc.get_particles()
        assert np.abs(gp["positions"] - op["positions"]).max() < 5e-7
        assert max_rel(gp["velocities"], op["velocities"]) < 2e-4


@pytest.mark.parametrize("E,weighting", [(5.0, 0), (1e4, 1)])
def test_cloth_ten_steps_match_oracle(E, weighting):
    grid, ps, mesh, ls, prm = small_cloth(True, seed=9, E=E, weighting=weighting)
    gpu, orc = pair(grid, ps, mesh, ls, prm)
    gpu.init_volumes()
    orc.init(volumes=True)
    for _ in range(10):
        gpu.step(2e-5)
        orc.step(2e-5)
    _compare_mesh(gpu.get_mesh(), orc.get_mesh(), 2e-6, 1e-3, 2e-5, 5e-3)


def test_cloth_mass_conserved_exactly():
    grid, ps, mesh, ls, prm = small_cloth(False)
    gpu = HybridSolver(None, grid, prm)
    gpu.set_lagrangian_mesh(mesh)
    gpu.set_level_set(ls)
    m0 = None
    for _ in range(10):
        gpu.step(2e-5)
        s = gpu.stats()
        m0 = s["total_mass"] if m0 is None else m0
        assert s["total_mass"] == m0
    total = mesh.vertex_masses.sum() + mesh.element_masses.sum()
    assert abs(m0 - total) / total < 1e-6


def _edge_fixed(mesh, nside=20):
    """vertexIsFixed for the x-min edge of the sheet, its first nside vertices
    (LagrangianMesh::bindConstraints)."""
    f = np.zeros(len(mesh.vertex_positions))
    f[:nside] = 1.0
    return f


@pytest.mark.parametrize("with_sand", [False, True])
def test_fixed_vertices_grid_matches_oracle(with_sand):
    grid, ps, mesh, ls, prm = small_cloth(with_sand)
    fixed = _edge_fixed(mesh)
    assert 10 <= fixed.sum() <= 40
    gpu, orc = pair(grid, ps, mesh, ls, prm)
    gpu.bind_constraints(fixed)
    orc.set_fixed_vertices(fixed)
    dt = 2e-5
    gpu.step_stage(dt, capi.AEP_STAGE_GRID)
    g = gpu.get_grid()
    orc.init(volumes=False)
    orc.step(dt, stage=capi.AEP_STAGE_GRID)
    o = orc.get_grid()
    # nodes the constraint zeroed: v and v_bf both zero (a sticking collision
    # zeroes v alone and keeps the tangential v_bf)
    zeroed = ((np.abs(o["velocities"]).max(axis=1) == 0) & (np.abs(o["velocities_before_friction"]).max(axis=1) == 0)
              & (o["masses"] > 0))
    assert zeroed.sum() > 100  # a band of nodes with mass
    assert np.all(g["velocities"][zeroed] == 0) and np.all(g["velocities_before_friction"][zeroed] == 0)
    assert mass_weighted_rel(g["velocities"], o["velocities"], o["masses"]) < 1e-4


def test_fixed_vertices_ten_steps_match_oracle_and_stay():
    grid, ps, mesh, ls, prm = small_cloth(True, seed=9)
    fixed = _edge_fixed(mesh)
    gpu, orc = pair(grid, ps, mesh, ls, prm)
    gpu.bind_constraints(fixed)
    orc.set_fixed_vertices(fixed)
    gpu.init_volumes()
    orc.init(volumes=True)
    for _ in range(10):
        gpu.step(2e-5)
        orc.step(2e-5)
    gm, om = gpu.get_mesh(), orc.get_mesh()
    _compare_mesh(gm, om, 2e-6, 1e-3, 2e-5, 5e-3)
    f = fixed > 0
    assert np.abs(gm["vertex_positions"][f] - mesh.vertex_positions[f]).max() < 1e-6
    assert np.abs(gm["vertex_velocities"][f]).max() == 0.0


def test_fixed_vertices_argument_checks():
    grid, ps, mesh, ls, prm = small_cloth(False)
    gpu = HybridSolver(None, grid, prm)
    gpu.set_lagrangian_mesh(mesh)
    with pytest.raises(capi.AepError):
        gpu.bind_constraints(np.ones(3))
    gpu.bind_constraints(None)
