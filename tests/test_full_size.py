"""The benchmark configurations at their full sizes, through properties that do
not depend on the size: the fixed-point grid mass is exactly the same every step,
no accumulator overflows, the state stays finite and inside the grid, the
collision conserves its horizontal momentum (no wall or ground in reach during
the steps: internal forces and the transfers conserve it), and a run repeats bit
for bit.  The sizes: the 524,288-particle sand column (128^3), the 65,536-vertex
cloth drape (128^3), the 2,097,152-particle snow+sand collision (256^3) and the
8,388,608-item sand + cloth scene (512^3)."""
import numpy as np
import pytest

from anisotropicelastoplasticity_gb300 import HybridSolver, scenes


def _solver(sc):
    s = HybridSolver(sc.particles, sc.grid, sc.params)
    if sc.mesh is not None:
        s.set_lagrangian_mesh(sc.mesh)
    s.set_level_set(sc.levelset)
    s.init_volumes()
    return s


def _run(sc, steps, each=None):
    s = _solver(sc)
    masses = []
    for k in range(steps):
        s.step(sc.dt)
        st = s.stats()
        assert st["overflow"] == 0
        masses.append(st["total_mass"])
        if each is not None:
            each(k, st)
    return s, masses


def _finite_inside(s, sc):
    p = s.get_particles()
    for key in ("positions", "velocities", "affine_momenta", "elastic_deformation_gradients", "plastic"):
        assert np.all(np.isfinite(p[key])), key
    lo, hi = np.asarray(sc.grid.min_bound), np.asarray(sc.grid.max_bound)
    assert np.all(p["positions"] >= lo) and np.all(p["positions"] <= hi)
    return p


@pytest.mark.gpu
def test_sand_column_full_size_repeats_and_conserves_mass():
    sc = scenes.sand_column()
    assert len(sc.particles) == 524288
    s1, m1 = _run(sc, 20)
    assert len(set(m1)) == 1  # the exact fixed-point mass, every step
    a = _finite_inside(s1, sc)
    s1.close()
    s2, m2 = _run(sc, 20)
    b = s2.get_particles()
    s2.close()
    assert m1 == m2
    for key in ("positions", "velocities", "elastic_deformation_gradients", "plastic"):
        assert np.array_equal(a[key], b[key]), key


@pytest.mark.gpu
def test_cloth_drape_full_size():
    sc = scenes.cloth_drape()
    assert len(sc.mesh.vertex_positions) == 65536 and len(sc.mesh.faces) == 130050
    s, masses = _run(sc, 20)
    assert len(set(masses)) == 1
    mesh = s.get_mesh()
    for key in ("vertex_positions", "vertex_velocities", "element_directions"):
        assert np.all(np.isfinite(mesh[key])), key
    s.close()


@pytest.mark.gpu
def test_collision_full_size_conserves_horizontal_momentum():
    sc = scenes.snow_sand_collision()
    ps = sc.particles
    assert len(ps) == 2097152
    # sum m |v_x| of the initial state: the scale of the x-momentum
    scale = float(np.sum(ps.masses * np.abs(ps.velocities[:, 0])))
    moms = []
    s, masses = _run(sc, 10, each=lambda k, st: moms.append(list(st["total_momentum"])))
    assert len(set(masses)) == 1
    moms = np.array(moms)
    assert np.abs(moms[:, 0] - moms[0, 0]).max() < 1e-5 * scale
    assert np.abs(moms[:, 1] - moms[0, 1]).max() < 1e-5 * scale
    # gravity alone changes the z-momentum: by M g dt per step
    dz = np.diff(moms[:, 2])
    total = float(np.sum(ps.masses))
    assert np.allclose(dz, -9.8 * total * sc.dt, rtol=1e-3)
    _finite_inside(s, sc)
    s.close()


@pytest.mark.gpu
def test_sand_cloth_full_size():
    sc = scenes.sand_cloth()
    assert sc.num_items() == 8388608
    s, masses = _run(sc, 4)
    assert len(set(masses)) == 1
    _finite_inside(s, sc)
    mesh = s.get_mesh()
    assert np.all(np.isfinite(mesh["element_directions"]))
    s.close()
