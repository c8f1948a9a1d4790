"""The snow block drop (32,768 particles, 64^3 grid, dt 1e-4, 200 steps) in full,
GPU against the FP64 oracle.  The block falls at 1 m/s from 0.325 above the
ground and does not reach it within the 200 steps.  The run therefore checks the
transfers, the stress of a nearly undeformed block and the integration over the
whole run length.  The bounds below are about 10x the differences measured on
GB300."""
import numpy as np
import pytest

from anisotropicelastoplasticity_gb300 import scenes

from .parity_util import make_pair, max_rel

pytestmark = pytest.mark.gpu


def test_snow_block_200_steps_match_oracle():
    sc = scenes.snow_block()
    assert len(sc.particles) == 32768 and sc.steps == 200
    gpu, orc = make_pair(sc)
    gpu.init_volumes()
    orc.init(volumes=True)
    for _ in range(sc.steps):
        gpu.step(sc.dt)
        orc.step(sc.dt)
    g, o = gpu.get_particles(), orc.get_particles()
    gpu.close()
    dx = np.abs(g["positions"] - o["positions"]).max()
    dv = max_rel(g["velocities"], o["velocities"])
    dF = np.abs(g["elastic_deformation_gradients"] - o["elastic_deformation_gradients"]).max()
    dq = np.abs(g["plastic"] - o["plastic"]).max()
    print(f"200 steps: |dx| {dx:.3g}, |dv|/|v| {dv:.3g}, |dF| {dF:.3g}, |dJp| {dq:.3g}")
    assert dx < 1e-5  # measured 1.1e-6
    assert dv < 1e-3  # 8.8e-5
    assert dF < 1e-4  # 9.7e-6
    assert dq < 1e-6  # 6.5e-14: J_P stays 1 without contact
    # the fall itself: the block's centre of mass follows the discrete free fall
    n = sc.steps
    z0 = float(np.mean(sc.particles.positions[:, 2]))
    fall = 1.0 * sc.dt * n + 9.8 * sc.dt * sc.dt * n * (n + 1) / 2
    assert abs((z0 - float(np.mean(g["positions"][:, 2]))) - fall) < 1e-4 * fall
