"""ctypes wrapper of liboracle.so (FP64 restatement of the reference step).

TEST INFRASTRUCTURE ONLY (the checker): used by tests/, __graft_entry__.smoke()
and bench.py's CPU-baseline leg.  Parity unpinned (see aep_oracle.cpp).

Arrays use the same (N, 3) / (N, 3, 3) numpy conventions as
anisotropicelastoplasticity_gb300.solver, converted to the reference layouts
at the call.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from anisotropicelastoplasticity_gb300 import capi
from anisotropicelastoplasticity_gb300.solver import (dirs_from_ref, dirs_to_ref, mats_from_ref, mats_to_ref,
                                                      rows_from_ref, rows_to_ref, vec_from_ref, vec_to_ref)

from . import build as _build

_dp = C.POINTER(C.c_double)
_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        lib = C.CDLL(str(_build.build()))
        vp = C.c_void_p
        lib.orc_create.restype = vp
        lib.orc_create.argtypes = [C.POINTER(capi.aep_grid_desc), C.POINTER(capi.aep_params)]
        lib.orc_destroy.argtypes = [vp]
        lib.orc_num_threads.argtypes = [C.c_int]
        lib.orc_num_threads.restype = C.c_int
        lib.orc_set_particles.argtypes = [vp, C.c_int64] + [_dp] * 8 + [C.POINTER(C.c_uint8)]
        lib.orc_set_mesh.argtypes = [vp, C.c_int64, C.c_int64, _dp, C.POINTER(C.c_int32)] + [_dp] * 8 + [C.c_double] * 5
        lib.orc_set_levelset.argtypes = [vp, C.POINTER(capi.aep_sdf), C.c_int32]
        lib.orc_init.argtypes = [vp, C.c_int]
        lib.orc_step.argtypes = [vp, C.c_double, C.c_double, C.c_int]
        lib.orc_solve.restype = C.c_int64
        lib.orc_solve.argtypes = [vp, C.c_double, C.c_double, C.c_int64, _dp, C.POINTER(C.c_int), _dp, C.c_int, _dp,
                                  C.c_int64]
        lib.orc_set_fixed_vertices.restype = C.c_int
        lib.orc_set_fixed_vertices.argtypes = [vp, C.c_int64, _dp]
        lib.orc_get_particles.argtypes = [vp, C.c_int64] + [_dp] * 7
        lib.orc_get_mesh.argtypes = [vp] + [_dp] * 7
        lib.orc_get_grid.argtypes = [vp] + [_dp] * 4
        lib.orc_get_stress.argtypes = [vp, C.c_int64, _dp]
        lib.orc_svd3.argtypes = [_dp, _dp, _dp, _dp]
        lib.orc_return_map.argtypes = [C.POINTER(capi.aep_params), C.c_int, _dp, _dp]
        lib.orc_cubic.restype = C.c_double
        lib.orc_cubic.argtypes = [C.c_double]
        lib.orc_dcubic.restype = C.c_double
        lib.orc_dcubic.argtypes = [C.c_double]
        lib.orc_gram_schmidt.argtypes = [_dp, _dp, _dp]
        lib.orc_particle_weights.restype = C.c_int
        lib.orc_particle_weights.argtypes = [vp, _dp, C.POINTER(C.c_int64), _dp, _dp]
        _lib = lib
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(_dp)


class Oracle:
    """FP64 restatement of HybridSolver on one scene (same call shape as HybridSolver)."""

    def __init__(self, grid, params, threads: int = 0):
        self.lib = load()
        self.grid = grid
        self.params = params
        self.h = C.c_void_p(self.lib.orc_create(C.byref(grid.desc()), C.byref(params)))
        self.threads = self.lib.orc_num_threads(int(threads))
        self.n = 0

    def close(self):
        if self.h:
            self.lib.orc_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_particle_system(self, ps):
        self.n = n = len(ps)
        arrs = [vec_to_ref(ps.positions), vec_to_ref(ps.velocities), rows_to_ref(ps.affine_momenta),
                mats_to_ref(ps.elastic_deformation_gradients), mats_to_ref(ps.plastic_deformation_gradients),
                np.ascontiguousarray(ps.masses, float), np.ascontiguousarray(ps.volumes, float),
                np.ascontiguousarray(ps.plastic_amount, float)]
        mat = np.ascontiguousarray(ps.material, np.uint8)
        self._keep = (arrs, mat)
        self.lib.orc_set_particles(self.h, n, *[_p(a) for a in arrs], mat.ctypes.data_as(C.POINTER(C.c_uint8)))

    def set_level_set(self, ls):
        arr, n = ls.to_c()
        self.lib.orc_set_levelset(self.h, arr, n)

    def set_lagrangian_mesh(self, mesh):
        self.mesh = mesh
        nv, nf = len(mesh.vertex_positions), len(mesh.faces)
        arrs = [vec_to_ref(mesh.vertex_positions), np.ascontiguousarray(mesh.faces.T, np.int32),
                vec_to_ref(mesh.vertex_velocities), vec_to_ref(mesh.element_velocities),
                np.ascontiguousarray(mesh.vertex_masses, float), np.ascontiguousarray(mesh.vertex_volumes, float),
                np.ascontiguousarray(mesh.element_masses, float), np.ascontiguousarray(mesh.element_volumes, float),
                dirs_to_ref(mesh.element_directions), dirs_to_ref(mesh.element_rest_directions)]
        self._keep_mesh = arrs
        self.lib.orc_set_mesh(self.h, nv, nf, _p(arrs[0]), arrs[1].ctypes.data_as(C.POINTER(C.c_int32)),
                              *[_p(a) for a in arrs[2:]], mesh.mu, mesh.lambda_, mesh.shear_stiffness,
                              mesh.stiffness, mesh.friction_coeff)

    def get_mesh(self) -> dict:
        nv, nf = len(self.mesh.vertex_positions), len(self.mesh.faces)
        xv, vv, xe, ve = np.empty(3 * nv), np.empty(3 * nv), np.empty(3 * nf), np.empty(3 * nf)
        Bv, Be, d = np.empty(9 * nv), np.empty(9 * nf), np.empty(9 * nf)
        self.lib.orc_get_mesh(self.h, _p(xv), _p(vv), _p(Bv), _p(xe), _p(ve), _p(Be), _p(d))
        return dict(vertex_positions=vec_from_ref(xv, nv), vertex_velocities=vec_from_ref(vv, nv),
                    vertex_affine_momenta=rows_from_ref(Bv, nv), element_positions=vec_from_ref(xe, nf),
                    element_velocities=vec_from_ref(ve, nf), element_affine_momenta=rows_from_ref(Be, nf),
                    element_directions=dirs_from_ref(d, nf))

    def init(self, volumes: bool = True):
        """weights + first P2G of solve (HybridSolver.cpp:829-855)."""
        self.lib.orc_init(self.h, int(volumes))

    def step(self, dt: float, stage: int = capi.AEP_STAGE_FULL, dt_force: float | None = None):
        self.lib.orc_step(self.h, float(dt if dt_force is None else dt_force), float(dt), int(stage))

    def solve(self, cfl: float, maxt: float, max_steps: int = 0, max_frames: int = 64, trace: int = 0) -> dict:
        """HybridSolver::solve (HS:827-989) after init(): adaptive Dt with the frame
        clamp.  Returns steps, final t, frames, the t of each frame and the Dt trace."""
        t = C.c_double(0.0)
        frames = C.c_int(0)
        ft = np.zeros(max(1, max_frames))
        dts = np.zeros(max(1, trace))
        it = self.lib.orc_solve(self.h, float(cfl), float(maxt), int(max_steps), C.byref(t), C.byref(frames), _p(ft),
                                int(max_frames), _p(dts), int(trace))
        nf = min(frames.value, max_frames)
        return dict(steps=int(it), t=t.value, frames=frames.value, frame_t=ft[:nf], dt=dts[:min(it, trace)])

    def set_fixed_vertices(self, vertex_is_fixed):
        """LagrangianMesh::bindConstraints: one value per vertex, nonzero = fixed; None clears."""
        if vertex_is_fixed is None:
            self.lib.orc_set_fixed_vertices(self.h, 0, None)
            return
        a = np.ascontiguousarray(vertex_is_fixed, float)
        if self.lib.orc_set_fixed_vertices(self.h, len(a), _p(a)) != 0:
            raise ValueError("vertex_is_fixed must have one entry per mesh vertex")

    def get_particles(self) -> dict:
        n = self.n
        x, v, B, Fe, Fp = (np.empty(k * n) for k in (3, 3, 9, 9, 9))
        vol, q = np.empty(n), np.empty(n)
        self.lib.orc_get_particles(self.h, n, _p(x), _p(v), _p(B), _p(Fe), _p(Fp), _p(vol), _p(q))
        return dict(positions=vec_from_ref(x, n), velocities=vec_from_ref(v, n), affine_momenta=rows_from_ref(B, n),
                    elastic_deformation_gradients=mats_from_ref(Fe, n),
                    plastic_deformation_gradients=mats_from_ref(Fp, n), volumes=vol, plastic=q)

    def get_grid(self) -> dict:
        ng = self.grid.grid_number()
        m, v, vbf, f = np.empty(ng), np.empty(3 * ng), np.empty(3 * ng), np.empty(3 * ng)
        self.lib.orc_get_grid(self.h, _p(m), _p(v), _p(vbf), _p(f))
        return dict(masses=m, velocities=vec_from_ref(v, ng), velocities_before_friction=vec_from_ref(vbf, ng),
                    forces=vec_from_ref(f, ng))

    def get_stress(self) -> np.ndarray:
        """per-particle 'cauchyStress' of the last force pass (HS:321-338), (N, 3, 3)."""
        st = np.empty(9 * self.n)
        if self.lib.orc_get_stress(self.h, self.n, _p(st)) != 0:
            raise RuntimeError("no stress available")
        return mats_from_ref(st, self.n)


def svd3(A: np.ndarray):
    lib = load()
    a = np.ascontiguousarray(np.asarray(A, float).T)
    U, s, V = np.empty(9), np.empty(3), np.empty(9)
    lib.orc_svd3(_p(a), _p(U), _p(s), _p(V))
    return U.reshape(3, 3).T, s, V.reshape(3, 3).T


def return_map(params, mat: int, s, q: float):
    """Singular-value return mapping of one particle (HybridSolver.cpp:626-674)."""
    sv = np.ascontiguousarray(np.asarray(s, float).copy())
    qq = C.c_double(q)
    load().orc_return_map(C.byref(params), int(mat), _p(sv), C.byref(qq))
    return sv, qq.value


def particle_weights(grid, params, pos):
    """Weights of one particle: (node ids, w, grad w) as built at HybridSolver.cpp:30-79."""
    orc = Oracle(grid, params)
    node = np.zeros(125, np.int64)
    w = np.zeros(125)
    g = np.zeros(375)
    p = np.ascontiguousarray(np.asarray(pos, float))
    c = orc.lib.orc_particle_weights(orc.h, _p(p), node.ctypes.data_as(C.POINTER(C.c_int64)), _p(w), _p(g))
    return node[:c], w[:c], g[:3 * c].reshape(c, 3)


def cubic(x: float) -> float:
    return load().orc_cubic(float(x))


def dcubic(x: float) -> float:
    return load().orc_dcubic(float(x))


def gram_schmidt(D: np.ndarray):
    lib = load()
    d = np.ascontiguousarray(np.asarray(D, float).T)
    Q, R = np.empty(9), np.empty(9)
    lib.orc_gram_schmidt(_p(d), _p(Q), _p(R))
    return Q.reshape(3, 3).T, R.reshape(3, 3).T
