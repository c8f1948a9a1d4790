"""aep_p2g_noalloc: the particle-to-grid transfer for callers that cannot allocate GPU
memory (a host application that owns all device memory through its own pool, or a
real-time loop that cannot afford the device-wide synchronisation of
cudaMalloc/cudaFree).  The caller hands over device arrays for the particles and for
the output grid; the library's only working memory is a fixed array compiled into
it.

The test calls the new entry point through the C-ABI twice in a row on the same
input.  Each result is checked against the FP64 oracle's grid after the first
P2G (HybridSolver.cpp:113-240) and against the grid the step's own P2G produces
(aep_step_stage up to AEP_STAGE_P2G, read back with aep_get_grid), with the
tolerances of the GPU parity suite; the two calls must agree bit for bit (the
fixed-point sums do not depend on the order of the atomics).  The second call
would expose a scratch array that was not cleared between calls.  This file is
collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from anisotropicelastoplasticity_gb300 import HybridSolver, capi
from anisotropicelastoplasticity_gb300.solver import rows_to_ref, vec_to_ref

from oracle.oracle import Oracle

from .parity_util import mass_weighted_rel, max_rel, perturbed, small_scene

pytestmark = pytest.mark.gpu


def _fp32_scene():
    sc = perturbed(small_scene("mixed"), seed=31)
    ps = sc.particles
    # round every input to FP32 once, so both entry points see identical numbers
    for name in ("positions", "velocities", "affine_momenta", "masses"):
        setattr(ps, name, getattr(ps, name).astype(np.float32).astype(np.float64))
    return sc


def test_noalloc_p2g_matches_step_p2g_on_two_calls():
    torch = pytest.importorskip("torch")
    sc = _fp32_scene()
    ps = sc.particles
    n, ng = len(ps), sc.grid.grid_number()

    gpu = HybridSolver(ps, sc.grid, sc.params)
    gpu.step_stage(sc.dt, capi.AEP_STAGE_P2G)
    ref = gpu.get_grid()
    gpu.close()
    orc = Oracle(sc.grid, sc.params)
    orc.set_particle_system(ps)
    orc.set_level_set(sc.levelset)
    orc.init(volumes=False)
    fp64 = orc.get_grid()
    orc.close()

    dev = torch.device("cuda", 0)
    x = torch.from_numpy(vec_to_ref(ps.positions).astype(np.float32)).to(dev)
    v = torch.from_numpy(vec_to_ref(ps.velocities).astype(np.float32)).to(dev)
    B = torch.from_numpy(rows_to_ref(ps.affine_momenta).astype(np.float32)).to(dev)
    m = torch.from_numpy(ps.masses.astype(np.float32)).to(dev)
    mass_out = torch.empty(ng, dtype=torch.float32, device=dev)
    vel_out = torch.empty(3 * ng, dtype=torch.float32, device=dev)
    lib = capi.load()
    desc = sc.grid.desc()
    results = []
    for _ in range(2):
        mass_out.fill_(float("nan"))
        vel_out.fill_(float("nan"))
        torch.cuda.synchronize()
        st = lib.aep_p2g_noalloc(C.byref(desc), n, x.data_ptr(), v.data_ptr(), B.data_ptr(), m.data_ptr(),
                                 float(ps.masses.max()), mass_out.data_ptr(), vel_out.data_ptr(), None)
        torch.cuda.synchronize()
        assert st == capi.AEP_OK, capi.STATUS_NAMES.get(st, st)
        mass = mass_out.double().cpu().numpy()
        vel = vel_out.double().cpu().numpy().reshape(3, ng).T
        assert np.all(np.isfinite(mass)) and np.all(np.isfinite(vel))
        # same bounds as tests/test_parity_gpu.py::test_p2g_grid_matches_oracle
        for want in (fp64, ref):
            assert max_rel(mass, want["masses"]) < 2e-6
            assert mass_weighted_rel(vel, want["velocities"], want["masses"]) < 2e-5
        results.append((mass, vel))
    # the two calls agree bit for bit (integer sums: the atomics' order does not matter)
    assert np.array_equal(results[1][0], results[0][0])
    assert np.array_equal(results[1][1], results[0][1])


def test_noalloc_rejects_grid_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    sc = small_scene("snow")
    desc = sc.grid.desc()
    for a in range(3):
        desc.res[a] = 128  # padded grid of 128^3 is larger than AEP_NOALLOC_MAX_NODES
    dev = torch.device("cuda", 0)
    buf = torch.zeros(16, dtype=torch.float32, device=dev)
    p = buf.data_ptr()
    st = capi.load().aep_p2g_noalloc(C.byref(desc), 4, p, p, p, p, 1.0, p, p, None)
    assert st == capi.AEP_CAPACITY
