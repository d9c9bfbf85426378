"""The C-ABI library builds, loads and exports every symbol include/*.h
declares (no GPU needed: nothing is called)."""
import ctypes
import glob
import os
import re

import pytest

import mdz

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


REFSHIM_HEADER = "mdoodz_refshim.h"   # declared by the drop-in library, libmdoodz_refshim.so


def _declared(refshim=False):
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        if (os.path.basename(h) == REFSHIM_HEADER) != refshim:
            continue
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


def test_refshim_exports_its_symbols(lib):
    """libmdoodz_refshim.so exports the mdz_gpu_* entry points of its header
    and the reference-named drop-ins."""
    import mdz_build
    if not os.path.exists(mdz_build.REFSHIM_LIB):
        mdz_build.build_refshim()
    shim = ctypes.CDLL(mdz_build.REFSHIM_LIB)
    names = _declared(refshim=True) + ["P2Mastah", "CountPartCell", "NonNewtonianViscosityGrid",
                                       "EvaluateStokesResidualDecoupled", "SolveStokesDefectDecoupled",
                                       "RogerGuntherII", "Interp_Grid2P", "UpdateParticleStress"]
    assert "mdz_gpu_init" in names
    missing = [n for n in names if not hasattr(shim, n)]
    assert not missing, missing


def test_struct_layouts_match_header(tmp_path):
    """The ctypes mirrors of the header's structs have the C compiler's size
    and field offsets (a C program built here against include/mdoodz_gpu.h
    prints them)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    mirrors = {"mdz_grid_desc": mdz.GridDesc, "mdz_fields": mdz.FieldsStruct, "mdz_materials": mdz.Materials,
               "mdz_rheo_params": mdz.RheoParams, "mdz_model": mdz.Model, "mdz_step_report": mdz.StepReport,
               "mdz_ref_breakpoint_desc": mdz.RefBreakpointDesc}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "mdoodz_gpu.h"', "int main(void) {"]
    for cname, py in mirrors.items():
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (cname, cname))
        for fname, _ in py._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, fname, cname, fname))
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = dict(l.split() for l in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n") if l)
    for cname, py in mirrors.items():
        assert int(out[cname]) == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert int(out[cname + "." + fname]) == getattr(py, fname).offset, (cname, fname)
