"""The C-ABI library loads and exports every function include/*.h declares
(no compute call: this runs without a GPU)."""
import ctypes
import re
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]


def declared_functions():
    names = []
    for h in sorted((REPO / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(amr_[a-z_0-9]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "amr_tree_create" in names and "amr_halo_exchange_f64" in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol():
    import __graft_entry__ as g

    lib_path = g.build_library()
    lib = ctypes.CDLL(str(lib_path))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.amr_version() == 1


def test_geometry_struct_matches_header():
    import amr_gb300 as A

    assert ctypes.sizeof(A.PatchGeometry) == 4 * 4 + 3 * 8
    assert A.HALO_META.itemsize == 36
