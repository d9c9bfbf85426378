"""The reference-signature drop-ins without a GPU: the generated layout view
of the reference's structures matches the reference's own header, the
drop-ins compile against that header (so their argument lists are the
reference's), and the built library exports every one of them."""
import ctypes as C
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REFSHIM = os.path.join(ROOT, "mdoodz6.0_gb300", "refshim")
REF_SRC = os.environ.get("MDZ_REF_SRC", "/root/reference/SOURCE")
HAVE_REF = os.path.exists(os.path.join(REF_SRC, "header_MDOODZ.h"))

DROP_INS = ("P2Mastah", "CountPartCell", "StrainRateComponents", "NonNewtonianViscosityGrid", "RheologicalOperators",
            "UpdateNonLinearity", "BuildStokesOperatorDecoupled", "BuildJacobianOperatorDecoupled",
            "EvaluateStokesResidualDecoupled", "SolveStokesDefectDecoupled", "LineSearchDecoupled", "Interp_Grid2P",
            "Interp_Grid2P_centroids2", "RogerGuntherII", "UpdateParticleStress", "AccumulatedStrainII",
            "mdz_gpu_init", "mdz_gpu_finalize", "mdz_gpu_last_status", "mdz_gpu_sync_to_host")


@pytest.mark.skipif(not HAVE_REF, reason="the reference's sources are not here")
def test_layout_view_matches_reference_header():
    r = subprocess.run([sys.executable, os.path.join(REFSHIM, "make_layout.py"), REF_SRC, "--check"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


@pytest.mark.skipif(not HAVE_REF, reason="the reference's sources are not here")
def test_drop_ins_compile_against_reference_header():
    """Definitions whose argument lists differ from the reference's
    prototypes fail to compile here (conflicting types)."""
    r = subprocess.run(["gcc", "-std=gnu99", "-fsyntax-only", "-Wall", "-Werror", "-DMDZ_WITH_REFERENCE_HEADER",
                        "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "oracle", "ref_stubs"),
                        "-I" + REF_SRC, os.path.join(REFSHIM, "mdz_refshim.c")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_drop_ins_compile_against_layout_view():
    r = subprocess.run(["gcc", "-std=gnu99", "-fsyntax-only", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"),
                        os.path.join(REFSHIM, "mdz_refshim.c")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_drop_in_library_exports():
    lib = os.path.join(ROOT, "mdoodz6.0_gb300", "lib", "libmdoodz_refshim.so")
    if not os.path.exists(lib):
        pytest.skip("not built")
    L = C.CDLL(lib)
    for name in DROP_INS:
        assert hasattr(L, name), name
