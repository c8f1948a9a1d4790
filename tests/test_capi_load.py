"""The C-ABI library builds, loads and exports every symbol include/aep.h declares;
the ctypes structures match the C layout (checked against gcc's sizeof/offsetof)."""
import ctypes as C
import re
import subprocess

import pytest

from anisotropicelastoplasticity_gb300 import _build, capi

from .conftest import ROOT

HEADER = ROOT / "include" / "aep.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(aep_[a-z_0-9]+)\s*\(", text)))


def test_build_and_load():
    lib = _build.build()
    assert lib.exists()
    capi.load()


def test_exports_every_declared_symbol():
    lib = capi.load()
    names = declared_functions()
    assert len(names) >= 14
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) <= set(capi.SIGNATURES), set(names) - set(capi.SIGNATURES)


def test_no_device_calls_without_gpu_are_safe():
    lib = capi.load()
    assert lib.aep_abi_version() == 2
    p = capi.default_params()
    assert p.gravity[2] == -9.8 and p.friction == 0.2 and p.friction_bug == 1
    assert p.sand.h0 == 35.0 and p.snow.xi == 10.0
    # the Python table (used where libaep.so must not be loaded) equals the library's
    q = capi.aep_params()
    lib.aep_default_params(C.byref(q))
    assert bytes(p) == bytes(q)


def test_scenes_do_not_load_the_gpu_library():
    """The CPU arms of the benchmark build scenes without mapping libaep.so."""
    import subprocess
    import sys

    code = ("import sys; sys.path.insert(0, %r)\n"
            "from anisotropicelastoplasticity_gb300 import scenes, capi\n"
            "scenes.sand_column(n=1000, res=32); scenes.sand_cloth(nside=16, n_sand=1000, res=32)\n"
            "assert capi._lib is None\n"
            "maps = open('/proc/self/maps').read()\n"
            "assert 'libaep.so' not in maps\n" % str(ROOT))
    subprocess.run([sys.executable, "-c", code], check=True)


def test_null_arguments_rejected():
    lib = capi.load()
    h = C.c_void_p()
    assert lib.aep_solver_create(None, None, C.byref(h)) == capi.AEP_INVALID_ARG
    g = capi.aep_grid_desc()
    g.res[0] = g.res[1] = g.res[2] = 0
    assert lib.aep_solver_create(C.byref(g), None, C.byref(h)) == capi.AEP_INVALID_ARG
    assert lib.aep_step(None, 1e-4) == capi.AEP_INVALID_ARG
    assert lib.aep_solver_destroy(None) == capi.AEP_INVALID_ARG


def test_struct_layout_matches_header(tmp_path):
    src = tmp_path / "sz.c"
    src.write_text(f'#include "{HEADER}"\n#include <stdio.h>\n#include <stddef.h>\n'
                   "int main(void){printf(\"%zu %zu %zu %zu %zu %zu %zu\\n\", sizeof(aep_sdf), sizeof(aep_grid_desc),"
                   " sizeof(aep_params), sizeof(aep_stats), offsetof(aep_params, friction_bug),"
                   " offsetof(aep_params, mass_bits), offsetof(aep_stats, total_mass)); return 0;}\n")
    exe = tmp_path / "sz"
    subprocess.run(["gcc", str(src), "-o", str(exe)], check=True)
    got = list(map(int, subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()))
    want = [C.sizeof(capi.aep_sdf), C.sizeof(capi.aep_grid_desc), C.sizeof(capi.aep_params),
            C.sizeof(capi.aep_stats), capi.aep_params.friction_bug.offset, capi.aep_params.mass_bits.offset,
            capi.aep_stats.total_mass.offset]
    assert got == want


def test_scene_runner_parses_its_arguments(capsys):
    """The scene runner (python -m anisotropicelastoplasticity_gb300.run_scene) lists
    the five seeded scenes and rejects others before touching a GPU."""
    import pytest

    from anisotropicelastoplasticity_gb300 import run_scene

    assert sorted(run_scene.SCENES) == ["cloth_drape", "sand_cloth", "sand_column", "snow_block",
                                        "snow_sand_collision"]
    with pytest.raises(SystemExit) as e:
        run_scene.main(["--help"])
    assert e.value.code == 0
    with pytest.raises(SystemExit) as e:
        run_scene.main(["no_such_scene"])
    assert e.value.code == 2
