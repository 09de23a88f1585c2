"""The C-ABI library builds, loads and exports every entry point declared in
include/sesp.h (no GPU call is made here)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "sesp.h")).read()
    return sorted(set(re.findall(r"^\s*int\s+(sesp_\w+)\s*\(", src, flags=re.M)))


def test_library_exports_header_symbols():
    from surfactant_enhanced_spreading_gb300.csrc import build
    path = build.build()
    lib = ctypes.CDLL(path)
    names = _declared()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.sesp_abi_version() == 2


def test_python_binding_covers_header():
    from surfactant_enhanced_spreading_gb300 import engine
    assert sorted(engine.SYMBOLS) == _declared()


def test_params_layout_matches_header():
    from surfactant_enhanced_spreading_gb300 import engine
    from surfactant_enhanced_spreading_gb300.csrc import build
    build.build()
    p = engine.default_params()
    assert list(p.n_cells) == [12, 12, 12]
    assert p.rebuild_interval == 10 and abs(p.tr - 3.81087) < 1e-15 and p.shake_maxit == 100
    assert abs(p.tau_steps - 7.5) < 1e-15 and abs(p.shake_tol - 1e-4) < 1e-18
    assert p.preset == engine.PRESET_REFERENCE


def test_config_params_defaults():
    """The configuration preset's settings: 300 K, 0.1 ps thermostat (50 steps
    of 2 fs), SHAKE tolerance 1e-8 (host code, no GPU)."""
    from surfactant_enhanced_spreading_gb300 import config_preset as C
    from surfactant_enhanced_spreading_gb300 import engine
    p = engine.default_params((8, 8, 8), preset=engine.PRESET_CONFIG)
    assert p.preset == engine.PRESET_CONFIG and list(p.n_cells) == [8, 8, 8]
    assert abs(p.tr - C.TR) < 1e-12 and abs(p.tau_steps - 50.0) < 1e-9
    assert p.shake_tol == 1e-8 and p.shake_maxit == 100


def test_library_exports_common_layer():
    """include/sesp_common.h: the layout functions and the gfortran-named
    subroutines of the step loop are exported by the same library."""
    from surfactant_enhanced_spreading_gb300.csrc import build
    lib = ctypes.CDLL(build.build())
    src = open(os.path.join(ROOT, "include", "sesp_common.h")).read()
    names = set(re.findall(r"^\s*(?:int|void|sesp_ctx\s*\*|const\s+sesp_cmn_map\s*\*)\s*(\w+)\s*\(", src, flags=re.M))
    assert {"sesp_cmn_attach", "evalforces_", "move_w2_a_", "move_surfactant_b_"} <= names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    fmod = open(os.path.join(ROOT, "include", "sesp_common_mod.f90")).read().lower()
    for n in names:
        if n.startswith("sesp_cmn_") and not n.endswith("_") and n not in ("sesp_cmn_map_from_domains", "sesp_cmn_map_destroy",
                                                     "sesp_cmn_assign", "sesp_cmn_scatter", "sesp_cmn_gather",
                                                     "sesp_cmn_slot", "sesp_cmn_current_map"):
            assert f'name="{n}"' in fmod, n


def test_fortran_interface_module_lists_every_entry_point():
    src = open(os.path.join(ROOT, "include", "sesp_mod.f90")).read().lower()
    for n in _declared():
        assert f'name="{n}"' in src, n


def test_check_flags_follow_the_reference_rules():
    """Warning rules of get_molecule_count and computeOnm4, host side."""
    from surfactant_enhanced_spreading_gb300 import engine as E
    from surfactant_enhanced_spreading_gb300.csrc import build
    build.build()
    ok = [1010, 1010, 1e-12, 1000, 2000, 1000, 0]
    assert E.check_flags(ok) == 0
    assert E.check_flags([1009, 1010, 0, 1000, 2000, 1000, 3]) == E.CHECK_MOLECULES_LOST
    assert E.check_flags([1010, 1010, 0.0316, 1000, 2000, 1000, 0]) == 0           # q^2 = 0.000999
    assert E.check_flags([1010, 1010, 0.032, 1000, 2000, 1000, 0]) == E.CHECK_CHARGE
    assert E.check_flags([1010, 1010, -0.032, 1000, 2000, 1000, 0]) == E.CHECK_CHARGE
    # integer H / O: 2999 / 1000 = 2 passes, 1999 / 1000 = 1 does not
    assert E.check_flags([1010, 1010, 0, 1000, 2999, 1000, 0]) == 0
    assert E.check_flags([1010, 1010, 0, 1000, 1999, 1000, 0]) == E.CHECK_OH_RATIO
    assert E.check_flags([1010, 1010, 0, 999, 1998, 1000, 0]) == E.CHECK_MISSING_OXYGEN
    assert E.check_flags([10, 10, 0, 0, 0, 0, 0]) == 0                             # surfactants only
    assert E.check_flags([10, 10, 0, 0, 2, 0, 0]) == E.CHECK_OH_RATIO
    assert E.check_flags([9, 10, 0.5, 0, 2, 1, 3]) == 15
