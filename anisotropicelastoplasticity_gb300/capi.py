"""ctypes mirror of include/aep.h (the C-ABI of libaep.so).

Structures here must match the C declarations field for field; the
`tests/test_capi_load.py` checks sizes against the header.  Loading never
falls back to anything: if libaep.so is missing or cannot be loaded, an
ImportError/OSError is raised.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from . import _build

AEP_OK = 0
AEP_INVALID_ARG = 1
AEP_CUDA_ERROR = 2
AEP_OVERFLOW = 3
AEP_OUT_OF_DOMAIN = 4
AEP_NOT_READY = 5
AEP_OUT_OF_MEMORY = 6
AEP_NO_DEVICE = 7
AEP_CAPACITY = 8
STATUS_NAMES = {
    0: "AEP_OK", 1: "AEP_INVALID_ARG", 2: "AEP_CUDA_ERROR", 3: "AEP_OVERFLOW", 4: "AEP_OUT_OF_DOMAIN",
    5: "AEP_NOT_READY", 6: "AEP_OUT_OF_MEMORY", 7: "AEP_NO_DEVICE", 8: "AEP_CAPACITY",
}
AEP_NOALLOC_MAX_NODES = 373248

AEP_SNOW = 0
AEP_SAND = 1
AEP_CLOTH_VERTEX = 2
AEP_CLOTH_ELEMENT = 3

AEP_SDF_PLANE = 0
AEP_SDF_SPHERE = 1
AEP_SDF_WALL2GROUND = 2

AEP_STAGE_P2G = 1
AEP_STAGE_FORCES = 2
AEP_STAGE_GRID = 3
AEP_STAGE_FULL = 4


class aep_sdf(C.Structure):
    _fields_ = [("type", C.c_int32), ("reserved", C.c_int32), ("p", C.c_double * 6)]


class aep_grid_desc(C.Structure):
    _fields_ = [("min", C.c_double * 3), ("max", C.c_double * 3), ("res", C.c_int32 * 3), ("reserved", C.c_int32)]


class aep_snow_params(C.Structure):
    _fields_ = [("E", C.c_double), ("nu", C.c_double), ("theta_c", C.c_double), ("theta_s", C.c_double),
                ("xi", C.c_double)]


class aep_sand_params(C.Structure):
    _fields_ = [("E", C.c_double), ("nu", C.c_double), ("h0", C.c_double), ("h1", C.c_double),
                ("h2", C.c_double), ("h3", C.c_double)]


class aep_params(C.Structure):
    _fields_ = [
        ("snow", aep_snow_params),
        ("sand", aep_sand_params),
        ("gravity", C.c_double * 3),
        ("friction", C.c_double),
        ("friction_bug", C.c_int32),
        ("track_plastic_F", C.c_int32),
        ("particle_damp", C.c_double),
        ("mass_bits", C.c_int32),
        ("momentum_bits", C.c_int32),
        ("mesh_damp", C.c_double),
        ("cloth_volume_weighting", C.c_int32),
        ("full_sort", C.c_int32),
        ("reorder_interval", C.c_int32),
        ("fp64_apex", C.c_int32),
        ("reserved", C.c_int64 * 5),
    ]


class aep_stats(C.Structure):
    _fields_ = [
        ("steps", C.c_int64),
        ("num_particles", C.c_int64),
        ("active_blocks", C.c_int64),
        ("out_of_domain", C.c_int64),
        ("fp64_fallbacks", C.c_int64),
        ("overflow", C.c_int64),
        ("active_nodes", C.c_int64),
        ("total_mass", C.c_double),
        ("total_momentum", C.c_double * 3),
        ("learned_accepted", C.c_int64),
        ("learned_fallbacks", C.c_int64),
        ("sort_movers", C.c_int64),
        ("learned_exact", C.c_int64),
        ("orderings", C.c_int64),
        ("fp64_apex", C.c_int64),
        ("reserved", C.c_double * 1),
    ]


class aep_solve_state(C.Structure):
    _fields_ = [
        ("t", C.c_double),
        ("inner_t", C.c_double),
        ("dt", C.c_double),
        ("steps", C.c_int64),
        ("frames", C.c_int32),
        ("frame_done", C.c_int32),
        ("reserved", C.c_double * 4),
    ]


_dp = C.POINTER(C.c_double)
_u8p = C.POINTER(C.c_uint8)
_solver_p = C.c_void_p

# int32_t (*)(aep_solver*, const aep_solve_state*, void*)
SOLVE_FN = C.CFUNCTYPE(C.c_int32, C.c_void_p, C.POINTER(aep_solve_state), C.c_void_p)

# name -> (restype, argtypes); every symbol declared in include/aep.h
SIGNATURES = {
    "aep_abi_version": (C.c_int32, []),
    "aep_default_params": (None, [C.POINTER(aep_params)]),
    "aep_solver_create": (C.c_int, [C.POINTER(aep_grid_desc), C.POINTER(aep_params), C.POINTER(_solver_p)]),
    "aep_solver_destroy": (C.c_int, [_solver_p]),
    "aep_set_particles": (C.c_int, [_solver_p, C.c_int64, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _u8p]),
    "aep_set_levelset": (C.c_int, [_solver_p, C.POINTER(aep_sdf), C.c_int32]),
    "aep_set_mesh": (C.c_int, [_solver_p, C.c_int64, C.c_int64, _dp, C.POINTER(C.c_int32), _dp, _dp, _dp, _dp, _dp,
                               _dp, _dp, _dp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double]),
    "aep_get_mesh": (C.c_int, [_solver_p, _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "aep_set_mesh_state": (C.c_int, [_solver_p, C.c_int64, C.c_int64, _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "aep_init_volumes": (C.c_int, [_solver_p]),
    "aep_step": (C.c_int, [_solver_p, C.c_double]),
    "aep_synchronize": (C.c_int, [_solver_p]),
    "aep_get_particles": (C.c_int, [_solver_p, C.c_int64, _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "aep_get_grid": (C.c_int, [_solver_p, _dp, _dp, _dp, _dp]),
    "aep_get_stats": (C.c_int, [_solver_p, C.POINTER(aep_stats)]),
    "aep_step_stage": (C.c_int, [_solver_p, C.c_double, C.c_int32]),
    "aep_step_split": (C.c_int, [_solver_p, C.c_double, C.c_double]),
    "aep_set_fixed_vertices": (C.c_int, [_solver_p, C.c_int64, _dp]),
    "aep_set_solve_callback": (C.c_int, [_solver_p, SOLVE_FN, C.c_void_p]),
    "aep_set_max_steps": (C.c_int, [_solver_p, C.c_int64]),
    "aep_solve": (C.c_int, [_solver_p, C.c_double, C.c_double, C.c_double]),
    "aep_get_solve_state": (C.c_int, [_solver_p, C.POINTER(aep_solve_state)]),
    "aep_get_weights": (C.c_int, [_solver_p, C.c_int64, C.POINTER(C.c_int64), C.POINTER(C.c_int64), _dp, _dp]),
    "aep_checkpoint_size": (C.c_int, [_solver_p, C.POINTER(C.c_int64)]),
    "aep_checkpoint_save": (C.c_int, [_solver_p, C.c_void_p, C.c_int64]),
    "aep_checkpoint_load": (C.c_int, [_solver_p, C.c_void_p, C.c_int64]),
    "aep_set_stream": (C.c_int, [_solver_p, C.c_void_p]),
    "aep_set_profiling": (C.c_int, [_solver_p, C.c_int32]),
    "aep_get_phase_times": (C.c_int, [_solver_p, C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
    "aep_p2g_noalloc": (C.c_int, [C.POINTER(aep_grid_desc), C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]),
    "aep_last_error": (C.c_char_p, [_solver_p]),
    "aep_sort_pairs_temp_bytes": (C.c_int64, [C.c_int64, C.c_int32]),
    "aep_sort_pairs": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p,
                                 C.c_int64, C.c_void_p]),
    "aep_mlp_create": (C.c_int, [C.c_uint64, C.POINTER(C.c_void_p)]),
    "aep_mlp_destroy": (C.c_int, [C.c_void_p]),
    "aep_mlp_get_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_int64]),
    "aep_mlp_set_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_int64]),
    "aep_mlp_gradient": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.POINTER(C.c_float), C.POINTER(C.c_double)]),
    "aep_mlp_train": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_int32, C.c_double, C.c_double,
                                C.POINTER(C.c_double), C.c_void_p]),
    "aep_mlp_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    "aep_mlp_forward_step_form": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    "aep_mlp_last_error": (C.c_char_p, [C.c_void_p]),
    "aep_set_harvest": (C.c_int, [_solver_p, C.c_void_p, C.c_int64, C.c_int32]),
    "aep_get_harvest_count": (C.c_int, [_solver_p, C.POINTER(C.c_int64)]),
    "aep_set_return_map": (C.c_int, [_solver_p, C.c_void_p, C.c_double]),
    "aep_set_return_map_bounds": (C.c_int, [_solver_p, C.c_double, C.c_double]),
}

AEP_MLP_NUM_PARAMS = 9928

PHASES = ["sort", "p2g", "normalize", "cloth_force", "force", "grid", "g2p", "mlp", "cloth_g2p"]

_lib = None


def lib_path() -> Path:
    return _build.LIB


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load libaep.so (building it first when missing).  Raises if it cannot load."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not path.exists():
        if not build_if_missing:
            raise ImportError(f"libaep.so not built: {path}")
        _build.build()
    lib = C.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class AepError(RuntimeError):
    def __init__(self, status: int, msg: str = ""):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")


# The reference's literal values, the same table as aep_default_params in
# csrc/aep_capi.cu (tests/test_capi_load.py checks that the two agree).  Filled here
# in Python so that building a scene does not load libaep.so: the CPU arms of the
# benchmark construct the same scenes without mapping the GPU library.
_DEFAULTS = {
    "snow": {"E": 1.4e5, "nu": 0.2, "theta_c": 2.5e-2, "theta_s": 7.5e-3, "xi": 10.0},  # ParticleSystem.cpp:173-176, HS:267
    "sand": {"E": 3.537e5, "nu": 0.3, "h0": 35.0, "h1": 9.0, "h2": 0.2, "h3": 10.0},  # ParticleSystem.cpp:233-234, HS:641-644
    "gravity": (0.0, 0.0, -9.8),  # HybridSolver.cpp:457
    "friction": 0.2,  # HybridSolver.cpp:465
    "friction_bug": 1,  # HybridSolver.cpp:500-501
    "track_plastic_F": 0,
    "particle_damp": 0.0,  # HybridSolver.cpp:916
    "mesh_damp": 1.0,  # HybridSolver.cpp:926,932
    "mass_bits": 34,
    "momentum_bits": 40,
    "cloth_volume_weighting": 0,
    "full_sort": 0,
    "reorder_interval": 4,
    "fp64_apex": 0,
}


def default_params() -> aep_params:
    """aep_params with the reference's literal values (no library call)."""
    p = aep_params()
    for k, v in _DEFAULTS.items():
        if isinstance(v, dict):
            sub = getattr(p, k)
            for kk, vv in v.items():
                setattr(sub, kk, vv)
        elif k == "gravity":
            for a in range(3):
                p.gravity[a] = v[a]
        else:
            setattr(p, k, v)
    return p
