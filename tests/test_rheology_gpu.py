"""GPU parity of strain rates, the local VEP rheology with its tangent, the
rheological operators and the RHS, through the C ABI, against the reference's
golden vectors and against the oracle on larger seeded grids."""
import numpy as np
import pytest

import mdz
import mdz_setups
import oracle
from test_oracle_rheology import rheology_case, _check

pytestmark = pytest.mark.gpu

GPU_TOL = 1e-10   # FMA contraction on the GPU vs none in the oracle; local Newton tol 1e-13


@pytest.mark.parametrize("avg,tag", [(0, ""), (1, "_harm"), (2, "_geom"), (0, "_mech")])
def test_rheology_chain_vs_reference(golden, avg, tag):
    ref = golden("rheology_ref%s.npz" % tag)
    g, f, mat, prm = rheology_case(ref, avg, mech=tag == "_mech")
    ctx = mdz.Context(g, 3, 1)
    ctx.StrainRateComponents(f)
    for k in ("div_u", "exxd", "ezzd", "exz", "exz_n", "exxd_s", "ezzd_s"):
        _check(f[k], ref["sr_" + k], k, 1e-13)
    assert ctx.NonNewtonianViscosityGrid(mat, prm, f) == 0
    for k in ref:
        if k.startswith("vg_"):
            _check(f[k[3:]], ref[k], k, GPU_TOL)
    ctx.RheologicalOperators(prm, f, 0)
    for k in ref:
        if k.startswith("op0_"):
            _check(f[k[4:]], ref[k], k, GPU_TOL)
    ctx.RheologicalOperators(prm, f, 1)
    for k in ref:
        if k.startswith("op1_"):
            _check(f[k[4:]], ref[k], k, GPU_TOL)
    ctx.EvaluateRHS(prm, 0.0, float(ref["gz"]), f)
    for k in ("roger_x", "roger_z", "rhs_p"):
        _check(f[k], ref["rhs_" + k], k, GPU_TOL)
    ctx.close()


@pytest.mark.parametrize("mech", [False, True])
def test_rheology_vs_oracle_seeded_large(mech):
    """257 x 129 grid, 3 phases, random fields: GPU and oracle agree node by
    node (mech: Peierls creep, grain-boundary sliding, tension cut-off)."""
    from golden.make_golden import (RHEO_PHASES, RHEO_MODEL, RHEO_R, RHEO_PHASES_MECH, RHEO_MODEL_MECH,
                                    rheology_inputs)
    if mech:
        RHEO_PHASES, RHEO_MODEL = RHEO_PHASES_MECH, RHEO_MODEL_MECH
    g = mdz.Grid(257, 129, -1.0, 1.0, -0.5, 0.5).set_bc_pureshear(1.0)
    rng = np.random.default_rng(42)
    nph = 3
    ins = rheology_inputs(g, rng)
    x, z = mdz_setups.seed_markers(g, 3, 3, 0.5, 9)
    ph = (rng.random(len(x)) * nph).astype(np.int32)
    o = oracle.Oracle(g, nph)
    o.set_markers(x, z, ph)
    pn = o.P2Mastah(np.zeros(nph), None, g.tags(1), 0, 0, 1, 1, 1)
    ps = o.P2Mastah(np.zeros(nph), None, g.tags(0), 0, 0, 1, 0, 1)
    mat = mdz.Materials.from_phases(RHEO_PHASES, R=RHEO_R)
    prm = mdz.RheoParams.make(**RHEO_MODEL)
    fo = mdz.GridFields(g, nph, ins)
    fo["phase_perc_n"], fo["phase_perc_s"] = pn, ps
    fo["sxxd0_s"] = rng.normal(size=g.size(0)) * 0.3
    fo["szzd0_s"] = rng.normal(size=g.size(0)) * 0.3
    fo["sxz0_n"] = rng.normal(size=g.size(1)) * 0.3
    fg = mdz.GridFields(g, nph, dict(fo.a))
    oracle.strain_rates(g, fo)
    oracle.viscosity_grid(g, mat, prm, fo)
    oracle.rheo_operators(g, prm, fo, 1)
    ctx = mdz.Context(g, nph, 1)
    ctx.StrainRateComponents(fg)
    ctx.NonNewtonianViscosityGrid(mat, prm, fg)
    ctx.RheologicalOperators(prm, fg, 1)
    for k in ("eta_n", "eta_s", "sxxd", "szzd", "sxz", "detadexx_n", "detadp_n", "detadgxz_s", "p_corr", "eII_pl",
              "D11_n", "D12_n", "D14_n", "D33_s", "D34_s", "ddivpdexx_n", "ddivpdp_n", "eII_exp", "eII_gbs"):
        _check(fg[k], fo[k], k, GPU_TOL)
    assert (fo["eII_pl"] > 0).any() and (fo["eII_pl"] == 0).any()
    if mech:   # every mechanism is exercised: Peierls, GBS and tensile yielding
        assert (fo["eII_exp"] > 0).any() and (fo["eII_gbs"] > 0).any() and (fo["ddivpdp_n"] != 0).any()
    ctx.close()


def test_unsupported_rheology_is_rejected():
    g = mdz.Grid(9, 9, 0, 1, 0, 1).set_bc_pureshear(1.0)
    ctx = mdz.Context(g, 2, 1)
    f = mdz.GridFields(g, 2)
    mat = mdz.Materials.from_phases([dict(cstv=1, eta0=1.0, n_vp=1.0), dict(gs=1, n_vp=1.0)])
    with pytest.raises(mdz.MdzError) as e:    # grain-size evolution: not implemented
        ctx.NonNewtonianViscosityGrid(mat, mdz.RheoParams.make(dt=1.0), f)
    assert e.value.status == 4
    mat = mdz.Materials.from_phases([dict(cstv=1, eta0=1.0, n_vp=1.0), dict(expv=1, Gexp=0.0, n_vp=1.0)])
    with pytest.raises(mdz.MdzError) as e:    # Peierls creep without a valid gamma
        ctx.NonNewtonianViscosityGrid(mat, mdz.RheoParams.make(dt=1.0), f)
    assert e.value.status == 1
    ctx.close()
