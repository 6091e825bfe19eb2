"""The C ABI: every function the public header declares is exported by the
in-tree library, and the library loads without a GPU."""

import os
import re

import pytest

REPO = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def header_functions():
    names = set()
    for h in ("rg300.h", "rg300_sim.h", "rg300_mlp.h"):
        text = open(os.path.join(REPO, "include", h)).read()
        names |= set(re.findall(r"^\s*(?:rg_status|const char\*|rg_ctx\*)\s+(rg_\w+)\s*\(", text, re.M))
    return sorted(names)


def test_header_lists_entry_points():
    names = header_functions()
    assert "rg_solve" in names and "rg_create" in names
    from rismo2d_gb300 import _lib
    assert sorted(_lib.EXPORTS) == sorted(names)


def test_library_exports_every_symbol():
    from rismo2d_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("librg300.so not built")
    lib = _lib.load()
    for name in header_functions():
        assert hasattr(lib, name), name
    assert lib.rg_version().decode().startswith("rg300")
