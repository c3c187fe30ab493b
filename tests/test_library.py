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


def header_struct_fields(name):
    """(field, C type) in declaration order of `typedef struct name {...} name;`."""
    src = open(os.path.join(ROOT, "include", "vfvm_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    body = re.search(rf"typedef struct {name} \{{(.*?)\}} {name};", src, flags=re.S).group(1)
    fields = []
    for decl in body.split(";"):
        decl = " ".join(decl.split())
        if not decl:
            continue
        m = re.match(r"(const )?(int32_t|int64_t|double|float|int)(\*)? (.*)", decl)
        assert m, decl
        ctype = m.group(2) + ("*" if m.group(3) else "")
        for var in m.group(4).split(","):
            var = var.strip()
            fields.append((var.lstrip("*"), ctype + ("*" if var.startswith("*") else "")))
    return fields


@pytest.mark.parametrize("cname,pyname", [("vfvm_grid", "Grid_t"), ("vfvm_physics_desc", "Physics_t"),
                                          ("vfvm_control", "Control_t"), ("vfvm_history", "History_t")])
def test_struct_mirrors_match_header(vfvm, cname, pyname):
    """The ctypes structures passed across the C ABI have the header's fields in
    the header's order, with the same types (the layout the library reads)."""
    L = vfvm._lib
    ctype_of = {"int32_t": L.c_i32, "int": L.c_i32, "int64_t": L.c_i64, "double": L.c_d, "float": ctypes.c_float}
    want = header_struct_fields(cname)
    got = getattr(L, pyname)._fields_
    assert [f for f, _ in got] == [f for f, _ in want]
    for (field, pytype), (_, ctype) in zip(got, want):
        if ctype.endswith("*"):
            assert issubclass(pytype, ctypes._Pointer) and pytype._type_ == ctype_of[ctype[:-1]], field
        else:
            assert pytype == ctype_of[ctype], field
