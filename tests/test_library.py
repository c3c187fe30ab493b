"""The C-ABI library builds, loads and exports every entry point declared in
include/vfvm_gb300.h (no GPU compute is called here)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def declared_functions():
    src = open(os.path.join(ROOT, "include", "vfvm_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b(vfvm_[a-z0-9_]+)\s*\(", src)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("vfvm_create", "vfvm_assemble", "vfvm_solve", "vfvm_evolve", "vfvm_destroy", "vfvm_pattern"):
        assert n in names


def test_library_exports_all_declared_symbols(vfvm):
    path = vfvm.build_library()
    lib = ctypes.CDLL(path)
    for name in declared_functions():
        assert hasattr(lib, name), f"{name} declared in include/vfvm_gb300.h but not exported"


def test_ctypes_binding_covers_header(vfvm):
    assert set(declared_functions()) == set(vfvm._lib.SIGNATURES)


def test_product_has_no_oracle_dependency():
    pkg = os.path.join(ROOT, "voronoifvm.jl_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h")):
                text = open(os.path.join(dirpath, f)).read()
                assert "import oracle" not in text and "oracle/" not in text, f


def test_control_struct_layout(vfvm):
    lib = vfvm._lib.load()
    c = vfvm._lib.Control_t()
    lib.vfvm_control_default(ctypes.byref(c))
    assert c.abstol == 1e-10 and c.maxiters == 100 and c.damp_growth == 1.2 and c.store_all == 1
    assert c.reltol_linear == 1e-4 and c.abstol_linear == 0.0 and c.maxiters_linear == 100 and c.dt_grow == 1.2


def header_defines(prefix):
    src = open(os.path.join(ROOT, "include", "vfvm_gb300.h")).read()
    return {m.group(1): int(m.group(2)) for m in re.finditer(rf"#define\s+{prefix}([A-Z0-9_]+)\s+(\d+)", src)}


def test_physics_and_coordinate_ids_match_header(vfvm, oracle):
    """Every VFVM_PHYS_* and VFVM_COORD_* id of the header has the same number in
    the Python binding and in the oracle, and the species counts agree."""
    phys = header_defines("VFVM_PHYS_")
    assert {k.lower(): v for k, v in phys.items()} == vfvm._lib.PHYSICS_IDS
    assert vfvm._lib.PHYSICS_IDS == oracle.PHYS
    assert set(vfvm._lib.PHYSICS_NSPEC) == set(phys.values())
    coord = header_defines("VFVM_COORD_")
    assert {k.lower(): v for k, v in coord.items()} == vfvm._lib.COORD == oracle.COORD
    assert tuple(vfvm._lib.COORD) == vfvm.grid.COORD_SYSTEMS
