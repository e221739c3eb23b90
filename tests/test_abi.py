"""The C-ABI surface on a host without a GPU: the library loads, exports every symbol
include/planetsim_gb300.h declares, and validates arguments before touching a device."""
import ctypes as C
import re

import numpy as np
import pytest

from conftest import ROOT


def header_functions():
    text = (ROOT / "include" / "planetsim_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(psgb_\w+)\s*\(", text)))


def test_library_loads_and_exports_every_declared_symbol():
    from planet_game_gb300 import capi

    lib = capi.load()
    declared = header_functions()
    assert len(declared) >= 20
    missing = [name for name in declared if not hasattr(lib, name)]
    assert not missing, missing
    assert sorted(capi.EXPORTED) == declared
    assert lib.psgb_abi_version() == 8


def test_library_is_in_tree_and_has_sm103a_code():
    from planet_game_gb300 import capi

    assert capi.LIBRARY.is_relative_to(ROOT)
    data = capi.LIBRARY.read_bytes()
    assert b"sm_103a" in data or b"sm_103" in data


def test_invalid_arguments_are_rejected_on_the_host():
    from planet_game_gb300 import capi

    lib = capi.load()
    h = C.c_void_p()
    assert lib.psgb_planet_create(3, -5.0, C.byref(h)) == capi.ERR_INVALID_ARGUMENT
    assert b"radius" in lib.psgb_last_error()
    assert lib.psgb_planet_create(3, 6.371e6, None) == capi.ERR_INVALID_ARGUMENT
    assert lib.psgb_laplacian(None, capi.DTYPE_F64, None, None, capi.MEMORY_HOST, None) == capi.ERR_INVALID_ARGUMENT
    assert lib.psgb_batch_create(None, 0, C.byref(h)) == capi.ERR_INVALID_ARGUMENT


def test_solver_options_are_validated_before_any_device_work(meshes):
    from planet_game_gb300 import api, capi

    m = meshes(3)
    n = m.cell_count
    x = np.zeros(n)
    for bad in ({"precision": 7}, {"method": 9}, {"tolerance": -1.0}, {"inner_tolerance": 2.0},
                {"max_iterations": 0}, {"pre_sweeps": 0}, {"jacobi_omega": 2.5}):
        with pytest.raises(ValueError):
            api.solve_newton_system(m, 1e13, np.ones(n), np.ones(n), x, **bad)
    with pytest.raises(ValueError):
        api.solve_newton_system(m, -1.0, np.ones(n), np.ones(n), x)
    assert capi.load().psgb_planet_info_get(m.handle, None) == capi.ERR_INVALID_ARGUMENT


def test_column_radiation_rejects_bad_layer_counts():
    from planet_game_gb300 import api, capi

    k = api.column_constants(gravity_m_s2=9.8, reference_pressure_Pa=1e5, in_cloud_water_path_kg_m2=0.05,
                             effective_radius_m=1e-5)
    z = np.zeros((17, 4))
    one = np.zeros(4)
    with pytest.raises(ValueError):
        api.column_radiation(k, z, z, z, one, one)
    with pytest.raises(ValueError):
        api.column_radiation(api.column_constants(), np.zeros((3, 4)), np.zeros((3, 4)), np.zeros((3, 4)), one, one)


def test_hierarchy_view_without_gpu(meshes):
    m = meshes(5)
    assert m.level_rows == [10242, 642, 42]
    lv = m.hierarchy_level(0)
    assert len(lv["aggregate"]) == 10242 and lv["aggregate"].max() == 641
    assert len(m.hierarchy_level(2)["aggregate"]) == 0


def test_missing_library_fails_loudly():
    """Without the built library every entry point raises: there is no CPU fallback."""
    import subprocess
    import sys

    code = ("import pathlib, planet_game_gb300 as pg\n"
            "from planet_game_gb300 import capi\n"
            "capi.LIBRARY = pathlib.Path('/nonexistent/libplanetsim_gb300.so')\n"
            "capi._lib = None\n"
            "try:\n"
            "    pg.make_icosphere(2, 6.371e6)\n"
            "except FileNotFoundError as e:\n"
            "    print('refused:', e)\n")
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.startswith("refused:"), out.stdout + out.stderr
