"""The C-ABI library builds, loads and exports every symbol include/*.h
declares (no GPU needed: nothing is called)."""
import ctypes
import glob
import os
import re

import pytest

import mdz

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(mdz_[A-Za-z0-9_]+)\s*\(", src):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(mdz.LIB_PATH):
        import mdz_build
        mdz_build.build_cuda()
    return ctypes.CDLL(mdz.LIB_PATH)


def test_header_declares_entry_points():
    names = _declared()
    for required in ("mdz_create", "mdz_destroy", "mdz_P2Mastah", "mdz_RogerGuntherII", "mdz_Interp_Grid2P"):
        assert required in names


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing

