"""The adaptive solve loop (HybridSolver::solve, HybridSolver.cpp:827-989) and the
split time step: the oracle's Dt logic against the reference's rules on the CPU
(first Dt from the P2G velocities, Dt = CFL / max(300, max|v| / h), frames of
exactly 1/60 s), then the GPU loop (Dt and frame clock on the device) against
the oracle: step count, per-step Dt, frame times and the final particle state."""
import numpy as np
import pytest

from anisotropicelastoplasticity_gb300 import HybridSolver, scenes
from oracle.oracle import Oracle

from .parity_util import max_rel

FRAME = 1.0 / 60.0


def _scene(seed=3):
    sc = scenes.snow_block(n=3000, res=32, seed=seed)
    sc.particles.velocities[:] = [0.0, 0.0, -2.0]
    return sc


def _oracle(sc):
    o = Oracle(sc.grid, sc.params)
    o.set_particle_system(sc.particles)
    o.set_level_set(sc.levelset)
    o.init(volumes=True)
    return o


def test_oracle_solve_dt_rules():
    # slow scene: max|v|/h < 300, every Dt but the frame clamp is CFL/300
    sc = _scene()
    o = _oracle(sc)
    cfl = 0.05
    r = o.solve(cfl, 0.0, trace=4096)
    dt = r["dt"]
    assert r["frames"] == 1 and r["t"] == FRAME and len(dt) == r["steps"]
    assert abs(dt.sum() - FRAME) < 1e-15  # the steps of one frame add up to 1/60
    assert np.all(dt[:-1] == cfl / 300.0) and 0 < dt[-1] <= cfl / 300.0
    # fast scene: max|v|/h > 300, Dt = CFL h / max|v| of the updated grid velocities
    sc = _scene()
    sc.particles.velocities[:] = [0.0, 0.0, -12.0]
    o = _oracle(sc)
    h = float(sc.grid.h.min())
    r = o.solve(cfl, 0.0, trace=4096)
    dt = r["dt"]
    vmax = cfl * h / dt[:-1]
    assert np.all(vmax > 300 * h) and np.all(np.abs(vmax - 12.0) < 0.5)
    assert abs(dt.sum() - FRAME) < 1e-15


def test_oracle_solve_two_frames_and_limit():
    sc = _scene()
    o = _oracle(sc)
    r = o.solve(0.1, FRAME * 1.5, trace=4096)
    assert r["frames"] == 2 and abs(r["t"] - 2 * FRAME) < 1e-15
    assert np.allclose(r["frame_t"], [FRAME, 2 * FRAME], rtol=0, atol=1e-15)
    o2 = _oracle(_scene())
    r2 = o2.solve(0.1, 10.0, max_steps=7)
    assert r2["steps"] == 7 and r2["frames"] == 0


@pytest.mark.gpu
def test_gpu_solve_matches_oracle():
    sc = _scene()
    cfl = 0.05
    o = _oracle(sc)
    ro = o.solve(cfl, 0.0, trace=4096)
    s = HybridSolver(sc.particles, sc.grid, sc.params)
    s.set_level_set(sc.levelset)
    trace = []
    st = s.solve(cfl, 0.0, callback=lambda d: trace.append(d) and False)
    assert st["steps"] == ro["steps"] and st["frames"] == 1 and st["t"] == FRAME
    dts = np.array([d["dt"] for d in trace])
    assert len(dts) == ro["steps"]
    assert np.abs(dts - ro["dt"]).max() <= 1e-5 * ro["dt"].max()
    assert [d["frame_done"] for d in trace] == [False] * (len(trace) - 1) + [True]
    gp, op = s.get_particles(), o.get_particles()
    assert np.abs(gp["positions"] - op["positions"]).max() < 2e-5
    assert max_rel(gp["velocities"], op["velocities"]) < 2e-3


@pytest.mark.gpu
def test_gpu_solve_callback_stops_and_max_steps():
    sc = _scene()
    s = HybridSolver(sc.particles, sc.grid, sc.params)
    s.set_level_set(sc.levelset)
    st = s.solve(0.05, 1.0, callback=lambda d: d["steps"] >= 5)
    assert st["steps"] == 5 and st["frames"] == 0
    st = s.solve(0.05, 1.0, max_steps=3)
    assert st["steps"] == 3


@pytest.mark.gpu
def test_gpu_split_step_matches_oracle():
    sc = _scene(seed=4)
    o = _oracle(sc)
    s = HybridSolver(sc.particles, sc.grid, sc.params)
    s.set_level_set(sc.levelset)
    s.init_volumes()
    for dt_force, dt in [(1e-4, 1.3e-4), (1.3e-4, 0.7e-4), (0.7e-4, 1e-4)]:
        s.step(dt, dt_force=dt_force)
        o.step(dt, dt_force=dt_force)
    gp, op = s.get_particles(), o.get_particles()
    assert np.abs(gp["positions"] - op["positions"]).max() < 2e-6
    assert max_rel(gp["velocities"], op["velocities"]) < 5e-4
