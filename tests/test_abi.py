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
    assert lib.sesp_abi_version() == 1


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


def test_fortran_interface_module_lists_every_entry_point():
    src = open(os.path.join(ROOT, "include", "sesp_mod.f90")).read().lower()
    for n in _declared():
        assert f'name="{n}"' in src, n
