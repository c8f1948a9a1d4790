"""Full-state checkpoint (bit-exact resume) and the interpolation-weight query
(one row of HybridSolver::evaluateInterpolationWeights_, HybridSolver.cpp:18-97)
against the oracle's weights."""
import ctypes
import struct

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


def test_checkpoint_load_rejects_corrupted_contents():
    """A blob whose header and size are consistent but whose contents break what the
    kernels index with (a face index, a fixed vertex, a material tag, an id, the
    fixed-point bits of the parameters) is refused before anything reaches the GPU,
    and the handle keeps working afterwards."""
    from .test_cloth_gpu import _edge_fixed, small_cloth

    grid, ps, mesh, ls, prm = small_cloth(True, seed=4)
    a = HybridSolver(None, grid, prm)
    a.set_particle_system(ps)
    a.set_lagrangian_mesh(mesh)
    a.set_level_set(ls)
    a.bind_constraints(_edge_fixed(mesh))
    a.init_volumes()
    a.step(2e-5)
    blob = a.checkpoint()
    n = len(ps) + len(mesh.vertex_positions) + len(mesh.faces)
    nv, nf = len(mesh.vertex_positions), len(mesh.faces)
    nfixed = int((_edge_fixed(mesh) != 0).sum())
    nfa = 27  # x, v, B, F, m, vol, plastic (no F_P)
    body = n * (4 * nfa + 1 + 4 + 4) + nf * (12 + 24) + 4 * nfixed
    hdr = len(blob) - body
    assert hdr > 0
    mat_off = hdr + 4 * nfa * n
    ids_off = mat_off + n
    faces_off = ids_off + 8 * n
    fixed_off = faces_off + nf * (12 + 24)
    prm_off = 8 + 8 + 40 + ctypes.sizeof(capi.aep_grid_desc)  # magic, version + float arrays, 5 int64, grid
    mass_bits_off = prm_off + capi.aep_params.mass_bits.offset
    assert struct.unpack_from("<i", blob, mass_bits_off)[0] == prm.mass_bits

    def corrupt(off, fmt, value):
        b = bytearray(blob)
        struct.pack_into(fmt, b, off, value)
        return bytes(b)

    bad = {"face index": corrupt(faces_off + 4 * 7, "<i", nv + 3),
           "negative face index": corrupt(faces_off, "<i", -1),
           "fixed vertex": corrupt(fixed_off, "<i", nv),
           "material tag": corrupt(mat_off + 5, "<B", 7),
           "id": corrupt(ids_off + 4 * 2, "<i", n + 100),
           "mass bits": corrupt(mass_bits_off, "<i", 99)}
    b = HybridSolver(None, grid, prm)
    for what, blob_bad in bad.items():
        with pytest.raises(capi.AepError) as e:
            b.load_checkpoint(blob_bad)
        assert e.value.status == capi.AEP_INVALID_ARG, what
    b.mesh = mesh
    b.load_checkpoint(blob)  # the intact blob still loads and steps
    b.step(2e-5)
    a.step(2e-5)
    for k, v in a.get_mesh().items():
        assert np.array_equal(b.get_mesh()[k], v), k


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


def test_host_round_trip_of_particles_and_mesh_state_is_exact():
    """The end-to-end form of a step (the caller's arrays are the state: upload,
    step, read back) equals stepping on the device: re-uploading the same number of
    particles keeps the attached mesh and the device order, and aep_set_mesh_state
    writes the mesh members aep_get_mesh reads."""
    from .test_cloth_gpu import small_cloth

    grid, ps, mesh, ls, prm = small_cloth(True, seed=6)
    runs = []
    for round_trip in (False, True):
        s = HybridSolver(None, grid, prm)
        s.set_particle_system(ps)
        s.set_lagrangian_mesh(mesh)
        s.set_level_set(ls)
        s.init_volumes()
        for k in range(6):
            s.step(2e-5)
            if round_trip and k % 2 == 0:
                p = s.get_particles()
                lib, h, n = s._lib, s._h, len(ps)
                from anisotropicelastoplasticity_gb300.solver import mats_to_ref, rows_to_ref, vec_to_ref

                arrs = [vec_to_ref(p["positions"]), vec_to_ref(p["velocities"]), rows_to_ref(p["affine_momenta"]),
                        mats_to_ref(p["elastic_deformation_gradients"]), None, np.ascontiguousarray(ps.masses),
                        p["volumes"], p["plastic"]]
                mat = np.ascontiguousarray(ps.material, np.uint8)
                dp = lambda a: None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
                assert lib.aep_set_particles(h, n, *[dp(a) for a in arrs],
                                             mat.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))) == capi.AEP_OK
                s.set_mesh_state(s.get_mesh())
        runs.append((s.get_particles(), s.get_mesh()))
    for k in runs[0][0]:
        assert np.array_equal(runs[0][0][k], runs[1][0][k]), k
    for k in runs[0][1]:
        assert np.array_equal(runs[0][1][k], runs[1][1][k]), k
