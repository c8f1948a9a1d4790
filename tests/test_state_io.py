"""Full-state checkpoint (bit-exact resume) and the interpolation-weight query
(one row of HybridSolver::evaluateInterpolationWeights_, HybridSolver.cpp:18-97)
against the oracle's weights."""
import numpy as np
import pytest

from anisotropicelastoplasticity_gb300 import HybridSolver, capi, scenes
from oracle.oracle import particle_weights

from .parity_util import perturbed

pytestmark = pytest.mark.gpu


def _solver(sc):
    s = HybridSolver(sc.particles, sc.grid, sc.params)
    s.set_level_set(sc.levelset)
    s.init_volumes()
    return s


def _state(s):
    st = s.get_particles()
    return np.concatenate([st[k].ravel() for k in sorted(st)])


def test_checkpoint_resume_is_bit_exact():
    sc = perturbed(scenes.snow_sand_collision(n=12000, res=32, seed=2), seed=3)
    a = _solver(sc)
    for _ in range(5):
        a.step(sc.dt)
    blob = a.checkpoint()
    for _ in range(5):
        a.step(sc.dt)
    ref = _state(a)
    b = HybridSolver(None, sc.grid, capi.default_params())  # parameters come from the checkpoint
    b.load_checkpoint(blob)
    for _ in range(5):
        b.step(sc.dt)
    got = _state(b)
    assert np.array_equal(got, ref)
    assert a.stats()["total_mass"] == b.stats()["total_mass"]


def test_checkpoint_with_mesh_and_fixed_vertices(tmp_path):
    from .test_cloth_gpu import _edge_fixed, small_cloth

    grid, ps, mesh, ls, prm = small_cloth(True, seed=9)
    a = HybridSolver(None, grid, prm)
    a.set_particle_system(ps)
    a.set_lagrangian_mesh(mesh)
    a.set_level_set(ls)
    a.bind_constraints(_edge_fixed(mesh))
    a.init_volumes()
    for _ in range(3):
        a.step(2e-5)
    path = tmp_path / "state.aep"
    a.save_checkpoint_file(path)
    for _ in range(4):
        a.step(2e-5)
    ref = a.get_mesh()
    b = HybridSolver(None, grid, prm)
    b.mesh = mesh
    b.load_checkpoint_file(path)
    for _ in range(4):
        b.step(2e-5)
    got = b.get_mesh()
    for k in ref:
        assert np.array_equal(got[k], ref[k]), k


def test_checkpoint_rejects_other_grid_and_garbage():
    sc = scenes.snow_block(n=2000, res=32, seed=1)
    a = _solver(sc)
    blob = a.checkpoint()
    other = scenes.snow_block(n=2000, res=16, seed=1)
    b = HybridSolver(None, other.grid, other.params)
    with pytest.raises(capi.AepError):
        b.load_checkpoint(blob)
    with pytest.raises(capi.AepError):
        a.load_checkpoint(b"not a checkpoint" * 40)
    with pytest.raises(capi.AepError):
        a.load_checkpoint(blob[:-4])


def test_weights_match_oracle_rows():
    sc = scenes.sand_column(n=4000, res=32, seed=5)
    s = _solver(sc)
    ids = np.array([0, 17, 1234, 3999])
    nodes, w, g = s.weights(ids)
    pos = s.get_particles()["positions"]
    for r, pid in enumerate(ids):
        on, ow, og = particle_weights(sc.grid, sc.params, pos[pid])
        order = np.argsort(on)  # the row of the column-sorted sparse matrix
        on, ow, og = on[order], ow[order], og[order]
        keep = nodes[r] >= 0
        assert np.array_equal(nodes[r][keep], on)
        assert np.abs(w[r][keep] - ow).max() < 1e-6
        assert np.abs(g[r][keep] - og).max() < 1e-6 * 32 * 4
        assert abs(w[r].sum() - 1.0) < 1e-5
