"""The C++ host facade (include/aep/hybrid_solver.hpp): compiled with g++ against
libaep.so.  On the CPU its host logic runs (ObjMesh rules, RegularGrid indexing,
seeded scene factories, frame files); on the GPU a SandCylinder scene runs through
HybridSolver and the Python binding replays the same initial state through the
C-ABI: the two must agree bit for bit (same library, same inputs), which ties the
facade's array packing to the oracle-tested path.  Checkpoint resume and solve()
with frame files are checked inside the program."""
import subprocess

import numpy as np
import pytest

from anisotropicelastoplasticity_gb300 import HybridSolver, LevelSet, ParticleSystem, _build, make_params
from anisotropicelastoplasticity_gb300.solver import RegularGrid

from .conftest import ROOT

N = 20000


@pytest.fixture(scope="module")
def facade_exe(tmp_path_factory):
    lib = _build.build()
    out = tmp_path_factory.mktemp("facade") / "facade_check"
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}",
           str(ROOT / "tests" / "cpp" / "facade_check.cpp"), f"-L{lib.parent}", "-laep",
           f"-Wl,-rpath,{lib.parent}", "-o", str(out)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def test_facade_host_logic(facade_exe, tmp_path):
    r = subprocess.run([str(facade_exe), "host", str(tmp_path)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert "OK host" in r.stdout


def _read_state(path, n):
    a = np.fromfile(path, np.float64)
    o = 0

    def take(k):
        nonlocal o
        v = a[o:o + k]
        o += k
        return v

    x, v = take(3 * n).reshape(3, n).T, take(3 * n).reshape(3, n).T
    B = np.stack([take(3 * n).reshape(3, n).T for _ in range(3)], axis=1)  # (n, row a, col)
    F = take(9 * n).reshape(n, 3, 3).transpose(0, 2, 1)
    m, vol, q = take(n), take(n), take(n)
    assert o == len(a)
    return dict(x=x, v=v, B=B, F=F, m=m, vol=vol, q=q)


@pytest.mark.gpu
def test_facade_gpu_matches_python_binding(facade_exe, tmp_path):
    r = subprocess.run([str(facade_exe), "gpu", str(tmp_path)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "OK gpu" in r.stdout
    init = _read_state(tmp_path / "init.bin", N)
    got = _read_state(tmp_path / "stepped.bin", N)
    ps = ParticleSystem(init["x"], init["v"], init["m"], init["vol"], np.tile(np.eye(3), (N, 1, 1)),
                        affine_momenta=init["B"], plastic_amount=init["q"])
    grid = RegularGrid([0, 0, 0], [1, 1, 1], [32, 32, 32])
    s = HybridSolver(ps, grid, make_params())
    s.set_level_set(LevelSet.ground(0.05) | LevelSet.sphere([0.5, 0.5, 0.02], 0.05))
    s.init_volumes()
    for _ in range(20):
        s.step(1e-4)
    st = s.get_particles()
    assert np.array_equal(st["positions"], got["x"])
    assert np.array_equal(st["velocities"], got["v"])
    assert np.array_equal(st["affine_momenta"], got["B"])
    assert np.array_equal(st["elastic_deformation_gradients"], got["F"])
    assert np.array_equal(st["volumes"], got["vol"])
    assert np.array_equal(st["plastic"], got["q"])
