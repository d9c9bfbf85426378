"""Pin the oracle's restatement of StrainRateComponents, NonNewtonianViscosityGrid
/ Viscosity, RheologicalOperators and EvaluateRHS against the reference's own
functions (golden fixtures from tests/golden/make_golden.py)."""
import numpy as np
import pytest

import mdz
import oracle

RHEO_TOL = 1e-11   # local Newton stops at |r/Eii| < 1e-13: results agree to far below this

PHASES = None


def rheology_case(ref, avg, mech=False):
    """Grid, input fields, materials and parameters of a rheology fixture;
    mech: the fixture of Peierls creep, grain-boundary sliding and the
    tension cut-off (rheology_ref_mech.npz)."""
    from golden.make_golden import (RHEO_PHASES, RHEO_MODEL, RHEO_R, RHEO_PHASES_MECH, RHEO_MODEL_MECH, NX, NZ, XMIN,
                                    XMAX, ZMIN, ZMAX)
    g = mdz.Grid(NX, NZ, XMIN, XMAX, ZMIN, ZMAX).set_bc_pureshear(1.0)
    f = mdz.GridFields(g, 3)
    for k in ref:
        if k.startswith("in_"):
            f[k[3:]] = ref[k]
    m = dict(RHEO_MODEL_MECH if mech else RHEO_MODEL)
    m["eta_avg"] = avg
    prm = mdz.RheoParams.make(**m)
    mat = mdz.Materials.from_phases(RHEO_PHASES_MECH if mech else RHEO_PHASES, R=RHEO_R)
    return g, f, mat, prm


def _check(got, want, name, tol=RHEO_TOL):
    scale = max(np.abs(want).max(), 1e-300)
    err = np.abs(got - want).max() / scale
    assert err < tol, "%s: max rel err %.3e" % (name, err)


@pytest.mark.parametrize("avg,tag", [(0, ""), (1, "_harm"), (2, "_geom"), (0, "_mech")])
def test_rheology_chain_matches_reference(golden, avg, tag):
    ref = golden("rheology_ref%s.npz" % tag)
    g, f, mat, prm = rheology_case(ref, avg, mech=tag == "_mech")
    oracle.strain_rates(g, f)
    for k in ("div_u", "exxd", "ezzd", "exz", "exz_n", "exxd_s", "ezzd_s"):
        _check(f[k], ref["sr_" + k], k, 1e-13)
    nc = oracle.viscosity_grid(g, mat, prm, f)
    assert nc.sum() == 0
    for k in ref:
        if k.startswith("vg_"):
            _check(f[k[3:]], ref[k], k)
    oracle.rheo_operators(g, prm, f, 0)
    for k in ref:
        if k.startswith("op0_"):
            _check(f[k[4:]], ref[k], k)
    oracle.rheo_operators(g, prm, f, 1)
    for k in ref:
        if k.startswith("op1_"):
            _check(f[k[4:]], ref[k], k)
    oracle.rhs(g, prm, 0.0, float(ref["gz"]), f)
    for k in ("roger_x", "roger_z", "rhs_p"):
        _check(f[k], ref["rhs_" + k], k)
