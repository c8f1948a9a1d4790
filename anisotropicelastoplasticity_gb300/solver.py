"""Host-side mirror of the reference's C++ class surface over the C-ABI.

The reference's boundary is its classes with public Eigen members
(HybridSolver.h:27-94, ParticleSystem.h:20-57, RegularGrid.h:36-59,
LevelSet.h:5-12).  The classes here keep those names and meanings; arrays are
numpy with one row per particle: positions/velocities (N, 3), deformation
gradients and affine momenta (N, 3, 3) with [p, a, b] = M_p(a, b).  Layout
conversion to the reference's column-major memory happens at the C-ABI call.

Every compute call goes to libaep.so; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import capi
from .capi import AepError


def _dp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def vec_to_ref(a: np.ndarray) -> np.ndarray:
    """(N, 3) -> Eigen::MatrixX3d memory (all x, then y, then z)."""
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).T)


def vec_from_ref(buf: np.ndarray, n: int) -> np.ndarray:
    return buf.reshape(3, n).T.copy()


def mats_to_ref(F: np.ndarray) -> np.ndarray:
    """(N, 3, 3) -> std::vector<Matrix3d> memory (column-major per particle)."""
    return np.ascontiguousarray(np.asarray(F, dtype=np.float64).transpose(0, 2, 1))


def mats_from_ref(buf: np.ndarray, n: int) -> np.ndarray:
    return buf.reshape(n, 3, 3).transpose(0, 2, 1).copy()


def rows_to_ref(B: np.ndarray) -> np.ndarray:
    """(N, 3, 3) affine momenta -> affineMomenta_1|_2|_3 memory (aep.h)."""
    return np.ascontiguousarray(np.asarray(B, dtype=np.float64).transpose(1, 2, 0))


def rows_from_ref(buf: np.ndarray, n: int) -> np.ndarray:
    return buf.reshape(3, 3, n).transpose(2, 0, 1).copy()


class RegularGrid:
    """RegularGrid(minBound, maxBound, resolution) (RegularGrid.cpp:117-162)."""

    def __init__(self, min_bound, max_bound, resolution):
        self.min_bound = np.asarray(min_bound, dtype=np.float64).reshape(3)
        self.max_bound = np.asarray(max_bound, dtype=np.float64).reshape(3)
        self.resolution = np.asarray(resolution, dtype=np.int64).reshape(3)
        if np.any(self.max_bound <= self.min_bound) or np.any(self.resolution < 1):
            raise ValueError("maxBound must exceed minBound and resolution must be positive")
        self.h = (self.max_bound - self.min_bound) / self.resolution
        self.masses = np.zeros(self.grid_number())
        self.velocities = np.zeros((self.grid_number(), 3))

    def grid_number(self) -> int:
        return int(np.prod(self.resolution))

    def grid_volume(self) -> float:
        return float(np.prod(self.h))

    def to_index(self, i, j, k) -> int:  # RegularGrid.cpp:164-168
        rx, ry, _ = self.resolution
        return int(k * rx * ry + j * rx + i)

    def to_coordinate(self, index: int):  # RegularGrid.cpp:170-177
        rx, ry, _ = (int(r) for r in self.resolution)
        k = index // (rx * ry)
        j = (index % (rx * ry)) // rx
        return index - k * rx * ry - j * rx, j, k

    def positions(self) -> np.ndarray:
        rx, ry, rz = (int(r) for r in self.resolution)
        k, j, i = np.meshgrid(np.arange(rz), np.arange(ry), np.arange(rx), indexing="ij")
        idx = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1)
        return self.min_bound + idx * self.h

    def desc(self) -> capi.aep_grid_desc:
        d = capi.aep_grid_desc()
        for a in range(3):
            d.min[a] = float(self.min_bound[a])
            d.max[a] = float(self.max_bound[a])
            d.res[a] = int(self.resolution[a])
        return d


@dataclass
class ParticleSystem:
    """Public members of ParticleSystem (ParticleSystem.h:28-47); material per particle."""

    positions: np.ndarray
    velocities: np.ndarray
    masses: np.ndarray
    volumes: np.ndarray
    elastic_deformation_gradients: np.ndarray
    plastic_deformation_gradients: np.ndarray | None = None
    affine_momenta: np.ndarray | None = None  # (N, 3, 3): row a = affineMomenta_(a+1).row(p)
    plastic_amount: np.ndarray | None = None
    material: np.ndarray | None = None  # uint8, capi.AEP_SNOW / AEP_SAND

    def __post_init__(self):
        n = len(self.positions)
        self.positions = np.asarray(self.positions, dtype=np.float64).reshape(n, 3)
        self.velocities = np.asarray(self.velocities, dtype=np.float64).reshape(n, 3)
        self.masses = np.asarray(self.masses, dtype=np.float64).reshape(n)
        self.volumes = np.asarray(self.volumes, dtype=np.float64).reshape(n)
        self.elastic_deformation_gradients = np.asarray(self.elastic_deformation_gradients,
                                                        dtype=np.float64).reshape(n, 3, 3)
        if self.plastic_deformation_gradients is None:
            self.plastic_deformation_gradients = np.tile(np.eye(3), (n, 1, 1))
        if self.affine_momenta is None:
            self.affine_momenta = np.zeros((n, 3, 3))
        if self.plastic_amount is None:
            self.plastic_amount = np.zeros(n)
        if self.material is None:
            self.material = np.full(n, capi.AEP_SAND, dtype=np.uint8)
        self.material = np.asarray(self.material, dtype=np.uint8).reshape(n)

    def __len__(self) -> int:
        return len(self.positions)

    def copy(self) -> "ParticleSystem":
        return ParticleSystem(**{k: (None if v is None else np.array(v, copy=True))
                                 for k, v in self.__dict__.items()})


def dirs_to_ref(D: np.ndarray) -> np.ndarray:
    """(Nf, 3, 3) with columns d1 d2 d3 -> elementDirections_1 | _2 | _3 memory."""
    return np.ascontiguousarray(np.asarray(D, dtype=np.float64).transpose(2, 1, 0))


def dirs_from_ref(buf: np.ndarray, nf: int) -> np.ndarray:
    return buf.reshape(3, 3, nf).transpose(2, 1, 0).copy()


@dataclass
class LagrangianMesh:
    """Public members of LagrangianMesh (LagrangianMesh.h:37-73): one MPM particle per
    vertex and one per triangle; element directions as (Nf, 3, 3) with columns d1 d2 d3."""

    vertex_positions: np.ndarray
    faces: np.ndarray
    vertex_masses: np.ndarray
    vertex_volumes: np.ndarray
    element_masses: np.ndarray
    element_volumes: np.ndarray
    element_directions: np.ndarray
    element_rest_directions: np.ndarray
    mu: float
    lambda_: float
    shear_stiffness: float
    stiffness: float
    friction_coeff: float
    vertex_velocities: np.ndarray | None = None
    element_velocities: np.ndarray | None = None

    def __post_init__(self):
        nv, nf = len(self.vertex_positions), len(self.faces)
        self.vertex_positions = np.asarray(self.vertex_positions, np.float64).reshape(nv, 3)
        self.faces = np.asarray(self.faces, np.int32).reshape(nf, 3)
        if self.vertex_velocities is None:
            self.vertex_velocities = np.zeros((nv, 3))
        if self.element_velocities is None:
            self.element_velocities = np.zeros((nf, 3))

    @property
    def element_positions(self) -> np.ndarray:  # updateElementPositions (LagrangianMesh.cpp:371-380)
        return self.vertex_positions[self.faces].mean(axis=1)

    @staticmethod
    def from_triangles(V, F, density, thickness, youngs_modulus, poisson_ratio, shear_stiffness, stiffness,
                       friction_coeff) -> "LagrangianMesh":
        """Mass, volume and rest-direction rules of LagrangianMesh::ObjMesh
        (LagrangianMesh.cpp:306-351) for an in-memory triangle mesh with int32 indices;
        friction_coeff is the cap coefficient itself (ObjMesh takes tan of an angle)."""
        V = np.asarray(V, np.float64)
        F = np.asarray(F, np.int32)
        v1, v2, v3 = V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]
        a = np.linalg.norm(v2 - v1, axis=1)
        b = np.linalg.norm(v3 - v2, axis=1)
        c = np.linalg.norm(v1 - v3, axis=1)
        p = 0.5 * (a + b + c)
        area = np.sqrt(p * (p - a) * (p - b) * (p - c))  # triangleArea (geometry.cpp:13-23)
        evol = 0.25 * area * thickness
        vvol = np.zeros(len(V))
        for k in range(3):
            np.add.at(vvol, F[:, k], evol)
        nrm = np.cross(v2 - v1, v3 - v1)
        nrm /= np.linalg.norm(nrm, axis=1)[:, None]
        D = np.stack([v2 - v1, v3 - v1, nrm], axis=2)
        lam = youngs_modulus * poisson_ratio / (1 + poisson_ratio) / (1 - 2 * poisson_ratio)
        mu = youngs_modulus / 2 / (1 + poisson_ratio)
        return LagrangianMesh(V, F, density * vvol, vvol, density * evol, evol, D.copy(), D.copy(), mu, lam,
                              shear_stiffness, stiffness, friction_coeff)

    def copy(self) -> "LagrangianMesh":
        import copy as _c
        return _c.deepcopy(self)


@dataclass
class LevelSet:
    """Union of analytic level sets (LevelSet.cpp:8-42): phi = min over shapes."""

    shapes: list = field(default_factory=list)

    @staticmethod
    def plane(normal, offset) -> "LevelSet":
        n = np.asarray(normal, dtype=np.float64)
        n = n / np.linalg.norm(n)
        return LevelSet([(capi.AEP_SDF_PLANE, [*n, offset, 0.0, 0.0])])

    @staticmethod
    def ground(ground_z: float) -> "LevelSet":  # groundLevelSet / DgroundLevelSet
        return LevelSet.plane([0.0, 0.0, 1.0], ground_z)

    @staticmethod
    def sphere(center, radius) -> "LevelSet":
        return LevelSet([(capi.AEP_SDF_SPHERE, [*np.asarray(center, dtype=np.float64), radius, 0.0, 0.0])])

    @staticmethod
    def wall2ground(wall_x, wall_y, ground_z) -> "LevelSet":  # wall2groundLevelSet
        return LevelSet([(capi.AEP_SDF_WALL2GROUND, [wall_x, wall_y, ground_z, 0.0, 0.0, 0.0])])

    def __or__(self, other: "LevelSet") -> "LevelSet":
        return LevelSet(self.shapes + other.shapes)

    def to_c(self):
        arr = (capi.aep_sdf * max(1, len(self.shapes)))()
        for i, (t, p) in enumerate(self.shapes):
            arr[i].type = int(t)
            for k in range(6):
                arr[i].p[k] = float(p[k])
        return arr, len(self.shapes)


def make_params(**kw) -> capi.aep_params:
    """aep_params with the reference defaults, overridden by keyword (dotted for nested:
    snow_E, sand_h0, gravity, friction, ...)."""
    p = capi.default_params()
    for k, v in kw.items():
        if k.startswith("snow_"):
            setattr(p.snow, k[5:], float(v))
        elif k.startswith("sand_"):
            setattr(p.sand, k[5:], float(v))
        elif k == "gravity":
            for a in range(3):
                p.gravity[a] = float(v[a])
        else:
            cur = getattr(p, k)
            setattr(p, k, type(cur)(v))
    return p


class HybridSolver:
    """HybridSolver(ParticleSystem*, RegularGrid*) (HybridSolver.h:83-93) on one GPU.

    The reference runs `solve` on its own thread and exposes no step; here
    `step(dt)` is the loop body of HybridSolver::solve (HybridSolver.cpp:
    867-989) and state lives on the device until `sync()` copies it back into
    the ParticleSystem arrays.
    """

    def __init__(self, ps: ParticleSystem | None = None, rg: RegularGrid | None = None, params=None):
        self._lib = capi.load()
        self._h = C.c_void_p()
        self.ps = None
        self.mesh = None
        self.rg = rg
        self.params = params if params is not None else capi.default_params()
        if rg is not None:
            self._create()
        if ps is not None:
            self.set_particle_system(ps)

    # --- lifetime ---------------------------------------------------------------
    def _check(self, st: int):
        if st != capi.AEP_OK:
            msg = self._lib.aep_last_error(self._h).decode() if self._h else ""
            raise AepError(st, msg)

    def _create(self):
        st = self._lib.aep_solver_create(C.byref(self.rg.desc()), C.byref(self.params), C.byref(self._h))
        if st != capi.AEP_OK:
            raise AepError(st, "aep_solver_create")

    def close(self):
        if self._h:
            self._lib.aep_solver_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- reference setters (HybridSolver.h:86-89) ---------------------------------
    def set_regular_grid(self, rg: RegularGrid):
        self.close()
        self.rg = rg
        self._create()
        if self.ps is not None:
            self.set_particle_system(self.ps)

    def set_particle_system(self, ps: ParticleSystem):
        self.ps = ps
        self._np = None
        n = len(ps)
        x = vec_to_ref(ps.positions)
        v = vec_to_ref(ps.velocities)
        B = rows_to_ref(ps.affine_momenta)
        Fe = mats_to_ref(ps.elastic_deformation_gradients)
        Fp = mats_to_ref(ps.plastic_deformation_gradients)
        m = np.ascontiguousarray(ps.masses, dtype=np.float64)
        vol = np.ascontiguousarray(ps.volumes, dtype=np.float64)
        q = np.ascontiguousarray(ps.plastic_amount, dtype=np.float64)
        mat = np.ascontiguousarray(ps.material, dtype=np.uint8)
        self._check(self._lib.aep_set_particles(self._h, n, _dp(x), _dp(v), _dp(B), _dp(Fe), _dp(Fp), _dp(m),
                                                _dp(vol), _dp(q), mat.ctypes.data_as(C.POINTER(C.c_uint8))))

    def set_lagrangian_mesh(self, mesh: LagrangianMesh):
        """setLagrangianMesh (HybridSolver.h:88); call after set_particle_system, before stepping."""
        self.mesh = mesh
        nv, nf = len(mesh.vertex_positions), len(mesh.faces)
        xv = vec_to_ref(mesh.vertex_positions)
        faces = np.ascontiguousarray(mesh.faces.T, dtype=np.int32)
        vv, ve = vec_to_ref(mesh.vertex_velocities), vec_to_ref(mesh.element_velocities)
        mv, volv = (np.ascontiguousarray(a, np.float64) for a in (mesh.vertex_masses, mesh.vertex_volumes))
        me, vole = (np.ascontiguousarray(a, np.float64) for a in (mesh.element_masses, mesh.element_volumes))
        d, dr = dirs_to_ref(mesh.element_directions), dirs_to_ref(mesh.element_rest_directions)
        self._check(self._lib.aep_set_mesh(self._h, nv, nf, _dp(xv), faces.ctypes.data_as(C.POINTER(C.c_int32)),
                                           _dp(vv), _dp(ve), _dp(mv), _dp(volv), _dp(me), _dp(vole), _dp(d),
                                           _dp(dr), mesh.mu, mesh.lambda_, mesh.shear_stiffness, mesh.stiffness,
                                           mesh.friction_coeff))

    def get_mesh(self) -> dict:
        nv, nf = len(self.mesh.vertex_positions), len(self.mesh.faces)
        xv, vv, xe, ve = np.empty(3 * nv), np.empty(3 * nv), np.empty(3 * nf), np.empty(3 * nf)
        Bv, Be, d = np.empty(9 * nv), np.empty(9 * nf), np.empty(9 * nf)
        self._check(self._lib.aep_get_mesh(self._h, _dp(xv), _dp(vv), _dp(Bv), _dp(xe), _dp(ve), _dp(Be), _dp(d)))
        return dict(vertex_positions=vec_from_ref(xv, nv), vertex_velocities=vec_from_ref(vv, nv),
                    vertex_affine_momenta=rows_from_ref(Bv, nv), element_positions=vec_from_ref(xe, nf),
                    element_velocities=vec_from_ref(ve, nf), element_affine_momenta=rows_from_ref(Be, nf),
                    element_directions=dirs_from_ref(d, nf))

    def set_mesh_state(self, state: dict):
        """Write the mesh's per-step members (the keys of get_mesh; missing keys are
        kept) into the device state, keeping the device order (aep_set_mesh_state)."""
        nv, nf = len(self.mesh.vertex_positions), len(self.mesh.faces)
        conv = {"vertex_positions": vec_to_ref, "vertex_velocities": vec_to_ref, "vertex_affine_momenta": rows_to_ref,
                "element_positions": vec_to_ref, "element_velocities": vec_to_ref,
                "element_affine_momenta": rows_to_ref, "element_directions": dirs_to_ref}
        arrs = [conv[k](state[k]) if state.get(k) is not None else None for k in conv]
        self._check(self._lib.aep_set_mesh_state(self._h, nv, nf, *[_dp(a) for a in arrs]))

    def set_level_set(self, ls: LevelSet):
        arr, n = ls.to_c()
        self._check(self._lib.aep_set_levelset(self._h, arr, n))

    def bind_constraints(self, vertex_is_fixed):
        """LagrangianMesh::bindConstraints (LagrangianMesh.cpp:354-363) on the attached
        mesh: one value per vertex, nonzero = fixed; None removes the constraints."""
        if vertex_is_fixed is None:
            self._check(self._lib.aep_set_fixed_vertices(self._h, 0, None))
            return
        a = np.ascontiguousarray(vertex_is_fixed, np.float64)
        self._keep_fixed = a
        self._check(self._lib.aep_set_fixed_vertices(self._h, len(a), _dp(a)))

    # --- stepping ---------------------------------------------------------------
    def init_volumes(self):
        """First P2G of solve with evaluateVolumesAndDensities (HybridSolver.cpp:242-249)."""
        self._check(self._lib.aep_init_volumes(self._h))

    def step(self, dt: float, dt_force: float | None = None):
        """One loop body; dt_force (default dt) drives the force pass and grid update."""
        if dt_force is None:
            self._check(self._lib.aep_step(self._h, float(dt)))
        else:
            self._check(self._lib.aep_step_split(self._h, float(dt_force), float(dt)))

    def solve(self, cfl: float, maxt: float, alpha: float = 0.0, callback=None, max_steps: int = 0) -> dict:
        """HybridSolver::solve(CFL, maxt, alpha) (HybridSolver.cpp:827-989) with the
        adaptive Dt on the device.  callback(state: dict) runs after every step
        (state['frame_done'] marks a completed 1/60 s frame); returning True stops."""
        cb = None
        if callback is not None:
            def _cb(_h, st, _u):
                s_ = st.contents
                d = dict(t=s_.t, inner_t=s_.inner_t, dt=s_.dt, steps=s_.steps, frames=s_.frames,
                         frame_done=bool(s_.frame_done))
                try:
                    return 1 if callback(d) else 0
                except Exception:  # an exception cannot cross the C frame: stop the solve
                    self._cb_error = True
                    return 1
            cb = capi.SOLVE_FN(_cb)
        self._cb_error = False
        self._check(self._lib.aep_set_solve_callback(self._h, cb if cb is not None else capi.SOLVE_FN(), None))
        self._check(self._lib.aep_set_max_steps(self._h, int(max_steps)))
        try:
            self._check(self._lib.aep_solve(self._h, float(cfl), float(maxt), float(alpha)))
        finally:
            self._lib.aep_set_solve_callback(self._h, capi.SOLVE_FN(), None)
        if self._cb_error:
            raise RuntimeError("solve callback raised")
        return self.solve_state()

    def weights(self, ids) -> tuple:
        """Rows of evaluateInterpolationWeights_ (HybridSolver.cpp:18-97) for item ids at
        the current positions: (nodes (k, 64) with -1 for no node, w (k, 64), grad (k, 64, 3))."""
        ids = np.ascontiguousarray(np.atleast_1d(ids), np.int64)
        k = len(ids)
        nodes = np.empty((k, 64), np.int64)
        w = np.empty((k, 64))
        g = np.empty((k, 64, 3))
        p64 = C.POINTER(C.c_int64)
        self._check(self._lib.aep_get_weights(self._h, k, ids.ctypes.data_as(p64), nodes.ctypes.data_as(p64), _dp(w),
                                              _dp(g)))
        return nodes, w, g

    def checkpoint(self) -> bytes:
        """Full device state (current particle order, mesh, parameters, level set, fixed
        vertices); load_checkpoint of it resumes bit for bit."""
        n = C.c_int64()
        self._check(self._lib.aep_checkpoint_size(self._h, C.byref(n)))
        buf = C.create_string_buffer(n.value)
        self._check(self._lib.aep_checkpoint_save(self._h, buf, n.value))
        return buf.raw

    def load_checkpoint(self, blob: bytes):
        buf = C.create_string_buffer(bytes(blob), len(blob))
        self._check(self._lib.aep_checkpoint_load(self._h, buf, len(blob)))
        # header: magic[8], version, float_arrays (int32), n, np (int64), ...
        self._np = int(np.frombuffer(blob, np.int64, count=1, offset=24)[0])

    def save_checkpoint_file(self, path):
        with open(path, "wb") as f:
            f.write(self.checkpoint())

    def load_checkpoint_file(self, path):
        with open(path, "rb") as f:
            self.load_checkpoint(f.read())

    def solve_state(self) -> dict:
        st = capi.aep_solve_state()
        self._check(self._lib.aep_get_solve_state(self._h, C.byref(st)))
        return dict(t=st.t, inner_t=st.inner_t, dt=st.dt, steps=st.steps, frames=st.frames,
                    frame_done=bool(st.frame_done))

    def step_stage(self, dt: float, stage: int):
        self._check(self._lib.aep_step_stage(self._h, float(dt), int(stage)))

    def synchronize(self):
        self._check(self._lib.aep_synchronize(self._h))

    # --- readback -----------------------------------------------------------------
    def get_particles(self, want_fp: bool = False) -> dict:
        n = getattr(self, "_np", None)
        if n is None:
            n = len(self.ps) if self.ps is not None else 0
        x, v = np.empty(3 * n), np.empty(3 * n)
        B, Fe = np.empty(9 * n), np.empty(9 * n)
        Fp = np.empty(9 * n) if want_fp else None
        vol, q = np.empty(n), np.empty(n)
        self._check(self._lib.aep_get_particles(self._h, n, _dp(x), _dp(v), _dp(B), _dp(Fe), _dp(Fp), _dp(vol),
                                                _dp(q)))
        out = dict(positions=vec_from_ref(x, n), velocities=vec_from_ref(v, n), affine_momenta=rows_from_ref(B, n),
                   elastic_deformation_gradients=mats_from_ref(Fe, n), volumes=vol, plastic=q)
        if want_fp:
            out["plastic_deformation_gradients"] = mats_from_ref(Fp, n)
        return out

    def sync(self):
        """Copy the device state back into the bound ParticleSystem (reference members)."""
        st = self.get_particles(want_fp=bool(self.params.track_plastic_F))
        ps = self.ps
        ps.positions, ps.velocities = st["positions"], st["velocities"]
        ps.affine_momenta = st["affine_momenta"]
        ps.elastic_deformation_gradients = st["elastic_deformation_gradients"]
        ps.volumes = st["volumes"]
        sand = ps.material == capi.AEP_SAND
        ps.plastic_amount = np.where(sand, st["plastic"], 0.0)
        if "plastic_deformation_gradients" in st:
            ps.plastic_deformation_gradients = st["plastic_deformation_gradients"]
        return ps

    def get_grid(self) -> dict:
        ng = self.rg.grid_number()
        m, v, vbf, f = np.empty(ng), np.empty(3 * ng), np.empty(3 * ng), np.empty(3 * ng)
        self._check(self._lib.aep_get_grid(self._h, _dp(m), _dp(v), _dp(vbf), _dp(f)))
        self.rg.masses = m
        self.rg.velocities = vec_from_ref(v, ng)
        return dict(masses=m, velocities=vec_from_ref(v, ng), velocities_before_friction=vec_from_ref(vbf, ng),
                    forces=vec_from_ref(f, ng))

    def set_harvest(self, records_ptr: int | None, capacity: int = 0, stride: int = 1):
        """Collect (trial, projected) records from the exact return mapping of later steps
        into a caller-owned device buffer of `capacity` x 8 float32 (None stops)."""
        self._check(self._lib.aep_set_harvest(self._h, C.c_void_p(records_ptr or 0), int(capacity), int(stride)))

    def harvest_count(self) -> int:
        cnt = C.c_int64()
        self._check(self._lib.aep_get_harvest_count(self._h, C.byref(cnt)))
        return cnt.value

    def set_return_map(self, mlp=None, tolerance: float = 1e-3, abs_tolerance: float | None = None):
        """Use a trained ReturnMapMLP (None: the exact mapping of the reference).  A
        prediction is kept when the residuals of the optimality conditions of the
        projection it stands for (the yield condition and the flow rule, ln-strain
        units) are within max(tolerance x |prediction|, abs_tolerance) (abs_tolerance
        None: 2^-24, the spacing of FP32 numbers just below 1, what rounding a
        stretch near 1 to FP32 costs in ln s); otherwise the exact
        projection is used and counted as a fallback."""
        self._mlp_ref = mlp
        self._check(self._lib.aep_set_return_map(self._h, mlp.handle if mlp is not None else None, tolerance))
        if abs_tolerance is not None:
            self._check(self._lib.aep_set_return_map_bounds(self._h, tolerance, abs_tolerance))

    def set_stream(self, cuda_stream_ptr: int | None):
        """Order the solver's work on an external cudaStream_t (e.g. torch.cuda.Stream.cuda_stream)."""
        self._check(self._lib.aep_set_stream(self._h, C.c_void_p(cuda_stream_ptr or 0)))

    def set_profiling(self, on: bool):
        self._check(self._lib.aep_set_profiling(self._h, int(bool(on))))

    def phase_times(self) -> tuple[dict, int]:
        """Accumulated CUDA-event milliseconds per kernel phase since profiling was enabled."""
        ms = (C.c_double * len(capi.PHASES))()
        steps = C.c_int64(0)
        self._check(self._lib.aep_get_phase_times(self._h, ms, C.byref(steps)))
        return {k: ms[i] for i, k in enumerate(capi.PHASES)}, steps.value

    def stats(self) -> dict:
        s = capi.aep_stats()
        self._check(self._lib.aep_get_stats(self._h, C.byref(s)))
        return dict(steps=s.steps, num_particles=s.num_particles, active_blocks=s.active_blocks,
                    out_of_domain=s.out_of_domain, fp64_fallbacks=s.fp64_fallbacks, overflow=s.overflow,
                    active_nodes=s.active_nodes, learned_accepted=s.learned_accepted,
                    learned_fallbacks=s.learned_fallbacks, learned_exact=s.learned_exact,
                    sort_movers=s.sort_movers, orderings=s.orderings, fp64_apex=s.fp64_apex,
                    total_mass=s.total_mass, total_momentum=list(s.total_momentum))
