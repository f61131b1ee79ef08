"""The C-ABI library loads without a GPU and exports every function that
include/lbgb300.h declares (no compute calls)."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import ROOT, load_package


def declared_functions():
    src = open(os.path.join(ROOT, "include", "lbgb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = set()
    for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*([A-Za-z_][A-Za-z0-9_]*)\s*\(",
                         src, flags=re.M):
        names.add(m.group(1))
    names.discard("copy_border_devices_d3q19")  # C++ linkage, checked by its mangled name
    return sorted(names)


@pytest.fixture(scope="module")
def built_lib():
    pkg = load_package()
    path = pkg.abi.LIB_PATH
    if not os.path.exists(path):
        import __graft_entry__
        __graft_entry__.build()
    return path


def test_header_parses():
    names = declared_functions()
    for n in ["collision_d3q19", "streaming_d2q9", "read_value_3d", "get_border_d2q9",
              "apply_border_d3q19", "copy_border_devices_d2q9", "lb_create", "lb_step"]:
        assert n in names


def test_every_declared_symbol_is_exported(built_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", built_lib], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    abi = load_package().abi
    for sym in abi.CXX_SYMBOLS:
        assert sym in exported, sym


def test_ctypes_prototypes_cover_header(built_lib):
    abi = load_package().abi
    lib = abi.load(built_lib)
    proto = {p[0] for p in abi.PROTOTYPES}
    assert set(declared_functions()) <= proto
    assert lib.lb_version().decode().startswith("lbgb300")


def test_struct_layout_matches_header():
    """DataD2Q9 / DataD3Q19 mirror the reference struct member by member."""
    abi = load_package().abi
    ptr = ctypes.sizeof(ctypes.c_void_p)
    # D3Q19: 4 moments + 2 flags + 19 pops + 20 border pointers, 5 ints, 3 pointers
    off_width = (4 + 2 + 19 + 20) * ptr
    assert abi.DataD3Q19.width.offset == off_width
    assert abi.DataD3Q19.plotBuffer.offset == off_width + 5 * 4 + 4  # padded to 8
    assert abi.DataD2Q9.width.offset == (3 + 2 + 9 + 12) * ptr
    assert abi.DataD2Q9.psi.offset == abi.DataD2Q9.stream.offset + ptr
