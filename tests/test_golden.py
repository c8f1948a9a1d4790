"""Golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py from the
FP64 oracle on small seeded scenes, inputs stored with outputs):

* CPU: the oracle reproduces every fixture (regression pin of the checker);
* GPU: the sm_103a step, started from the fixture's inputs, lands on the
  fixture's state after the same number of steps within FP32 tolerances.
"""
from pathlib import Path

import numpy as np
import pytest

from anisotropicelastoplasticity_gb300 import HybridSolver, make_params
from anisotropicelastoplasticity_gb300.solver import LevelSet, ParticleSystem, RegularGrid

GOLDEN = sorted((Path(__file__).parent / "golden").glob("*.npz"))


def load_case(path):
    d = np.load(path)
    grid = RegularGrid(d["grid_min"], d["grid_max"], d["grid_res"])
    ps = ParticleSystem(positions=d["x0"], velocities=d["v0"], masses=d["m"], volumes=np.zeros(len(d["m"])),
                        elastic_deformation_gradients=d["F0"], plastic_deformation_gradients=d["Fp0"],
                        affine_momenta=d["B0"], plastic_amount=d["q0"], material=d["mat"])
    ls = LevelSet([(int(r[0]), list(r[1:])) for r in d["levelset"]])
    prm = make_params(friction=float(d["friction"]))
    return d, grid, ps, ls, prm


def test_golden_fixtures_present():
    assert len(GOLDEN) >= 3


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: p.stem)
def test_oracle_reproduces_golden(path):
    from oracle.oracle import Oracle

    d, grid, ps, ls, prm = load_case(path)
    o = Oracle(grid, prm, threads=1)
    o.set_particle_system(ps)
    o.set_level_set(ls)
    o.init(volumes=True)
    for _ in range(int(d["steps"])):
        o.step(float(d["dt"]))
    r = o.get_particles()
    assert np.abs(r["positions"] - d["x"]).max() < 1e-13
    assert np.abs(r["velocities"] - d["v"]).max() < 1e-10
    assert np.abs(r["elastic_deformation_gradients"] - d["F"]).max() < 1e-12
    assert np.abs(r["plastic"] - d["plastic"]).max() < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: p.stem)
def test_gpu_matches_golden(path):
    d, grid, ps, ls, prm = load_case(path)
    gpu = HybridSolver(ps, grid, prm)
    gpu.set_level_set(ls)
    gpu.init_volumes()
    assert np.abs(gpu.get_particles()["volumes"] - d["vol_init"]).max() / d["vol_init"].max() < 1e-5
    for _ in range(int(d["steps"])):
        gpu.step(float(d["dt"]))
    r = gpu.get_particles()
    assert np.abs(r["positions"] - d["x"]).max() < 1e-6
    assert np.abs(r["velocities"] - d["v"]).max() / np.abs(d["v"]).max() < 2e-4
    assert np.abs(r["elastic_deformation_gradients"] - d["F"]).max() < 1e-5
    assert np.abs(r["plastic"] - d["plastic"]).max() < 1e-5
