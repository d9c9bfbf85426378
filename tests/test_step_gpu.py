"""One full time step on the GPU (projection -> Newton loop with matrix-free
GCR/multigrid and line search -> marker update -> RK4) against the CPU oracle
time step (restated reference functions + direct linear solves)."""
import numpy as np
import pytest

import mdz
import mdz_setups
import oracle_step

pytestmark = pytest.mark.gpu

VEP_PHASES = [
    dict(cstv=1, eta0=1e3, mu=1.0, bet=1e-2, C=1.0, phi=np.pi / 6, psi=0.0, rho=1.0, Slim=1e10, eta_vp=0.05, n_vp=1.0,
         gs_ref=1.0, pls_start=0.0, pls_end=1.0),
    dict(cstv=1, eta0=1e3, mu=1.0, bet=1e-2, C=0.5, phi=np.pi / 6, psi=0.0, rho=1.0, Slim=1e10, eta_vp=0.05, n_vp=1.0,
         gs_ref=1.0, pls_start=0.0, pls_end=1.0),
]


def vep_case(N=33, nm=4, seed=5):
    g = mdz.Grid(N, N, -0.5, 0.5, -0.5, 0.5).set_bc_pureshear(1.0)
    x, z = mdz_setups.seed_markers(g, nm, nm, 0.5, seed)
    ph = mdz_setups.inclusion_phase(x, z, 0.0, 0.0, 0.08)
    rng = np.random.default_rng(seed)
    m = dict(x=x, z=z, phase=ph, sxxd=np.full(len(x), -0.7), szzd=np.full(len(x), 0.7),
             sxz=0.05 * rng.standard_normal(len(x)), strain_pl=np.zeros(len(x)), strain=np.zeros(len(x)),
             T=np.zeros(len(x)), cmul=1.0 + 0.01 * rng.standard_normal(len(x)), P=np.zeros(len(x)))
    u = (-g.xg[None, :] + 0 * g.zvx[:, None]).ravel()
    v = (g.zg[:, None] + 0 * g.xvz[None, :]).ravel()
    p = np.zeros(g.size(1))
    mat = mdz.Materials.from_phases(VEP_PHASES)
    return g, m, u, v, p, mat


def run_gpu(g, m, u, v, p, mat, model, cap=None):
    ctx = mdz.Context(g, mat.n_phases, cap or len(m["x"]))
    ctx.set_markers(m["x"], m["z"], m["phase"])
    for attr, key in ((mdz.M_SXXD, "sxxd"), (mdz.M_SZZD, "szzd"), (mdz.M_SXZ, "sxz"), (mdz.M_STRAIN_PL, "strain_pl"),
                      (mdz.M_STRAIN, "strain"), (mdz.M_T, "T"), (mdz.M_CMUL, "cmul"), (mdz.M_P, "P")):
        ctx.set_marker_attr(attr, m[key])
    f = mdz.GridFields(g, mat.n_phases)
    f["u"], f["v"], f["p"] = u, v, p
    s = f.struct()
    for name in mdz.FIELD_NAMES:
        if name not in ("u", "v", "p"):
            setattr(s, name, None)
    ctx._check(ctx.L.mdz_sync_fields(ctx.h, mdz.C.byref(s), 1))
    rep = ctx.time_step(mat, model)
    out = mdz.GridFields(g, mat.n_phases)
    ctx.download_fields(out)
    x, z, ph, vx, vz = ctx.get_markers()
    mk = dict(x=x, z=z, phase=ph, vx=vx, vz=vz, sxxd=ctx.get_marker_attr(mdz.M_SXXD),
              szzd=ctx.get_marker_attr(mdz.M_SZZD), sxz=ctx.get_marker_attr(mdz.M_SXZ),
              strain_pl=ctx.get_marker_attr(mdz.M_STRAIN_PL), strain=ctx.get_marker_attr(mdz.M_STRAIN),
              T=ctx.get_marker_attr(mdz.M_T), cmul=ctx.get_marker_attr(mdz.M_CMUL), P=ctx.get_marker_attr(mdz.M_P))
    ctx.close()
    return out, mk, rep


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("precision,fp32_rheo", [(64, 0), (32, 0), (32, 2)])
def test_vep_newton_step_vs_oracle(precision, fp32_rheo):
    """fp32_rheo > 0: the first non-linear iterations evaluate the local
    rheology in FP32; the converged step must not notice."""
    g, m, u, v, p, mat = vep_case()
    prm = mdz.RheoParams.make(dt=0.5, iselastic=1, step=1)
    model = mdz.Model.make(prm, newton=1, nit_max=12, rel_tol=1e-11, lin_rtol=1e-9, line_search=1,
                           precision=precision, fp32_rheology_its=fp32_rheo)
    out, mk, rep = run_gpu(g, dict((k, np.array(v_)) for k, v_ in m.items()), u, v, p, mat, model)
    mo = dict((k, np.array(v_)) for k, v_ in m.items())
    uo, vo, po, ro = oracle_step.time_step(g, mat, model, mo, u, v, p)
    assert rep.converged == 1 and ro["converged"] == 1, (rep.as_dict(), ro)
    assert (out["eII_pl"] > 0).any()                       # plasticity active
    assert _rel(out["u"], uo) < 1e-8 and _rel(out["v"], vo) < 1e-8
    assert _rel(out["p"] - out["p"].mean(), po - po.mean()) < 1e-8
    for k in ("sxxd", "szzd", "sxz", "strain_pl", "x", "z"):
        assert _rel(mk[k], mo[k]) < 1e-8, k
    assert np.array_equal(mk["phase"], mo["phase"])


@pytest.mark.parametrize("precision", [64, 32])
def test_adaptive_linear_tolerance_same_step(precision):
    """Eisenstat-Walker forcing (adaptive_lin_tol = 1) reaches the same
    converged step as fixed-tolerance solves, with fewer Krylov iterations."""
    g, m, u, v, p, mat = vep_case()
    prm = mdz.RheoParams.make(dt=0.5, iselastic=1, step=1)
    fixed = mdz.Model.make(prm, newton=1, nit_max=20, rel_tol=1e-11, lin_rtol=1e-9, line_search=0,
                           precision=precision)
    adapt = mdz.Model.make(prm, newton=1, nit_max=20, rel_tol=1e-11, lin_rtol=1e-9, line_search=0,
                           precision=precision, adaptive_lin_tol=1)
    out_f, mk_f, rep_f = run_gpu(g, dict((k, np.array(v_)) for k, v_ in m.items()), u, v, p, mat, fixed)
    out_a, mk_a, rep_a = run_gpu(g, dict((k, np.array(v_)) for k, v_ in m.items()), u, v, p, mat, adapt)
    assert rep_f.converged == 1 and rep_a.converged == 1, (rep_f.as_dict(), rep_a.as_dict())
    assert rep_a.linear_its < rep_f.linear_its, (rep_a.linear_its, rep_f.linear_its)
    assert _rel(out_a["u"], out_f["u"]) < 1e-8 and _rel(out_a["v"], out_f["v"]) < 1e-8
    assert _rel(out_a["p"] - out_a["p"].mean(), out_f["p"] - out_f["p"].mean()) < 1e-8
    for k in ("sxxd", "szzd", "sxz", "x", "z"):
        assert _rel(mk_a[k], mk_f[k]) < 1e-8, k


@pytest.mark.parametrize("direct", [1, 0])
def test_vep_step_with_reseeding_vs_oracle(direct):
    """model.reseed: CountPartCell(RESEED = 1) after the advection; the same
    markers are created (count, slots, positions, phases) as by the oracle
    step followed by the oracle reseeding, with the same attributes.  A short
    step (dt = 0.02 at unit pure-shear rate): a long one empties bands along
    the walls wider than two quarter cells, where the reference stops."""
    g, m, u, v, p, mat = vep_case()
    prm = mdz.RheoParams.make(dt=0.02, iselastic=1, step=1)
    model = mdz.Model.make(prm, newton=1, nit_max=12, rel_tol=1e-11, lin_rtol=1e-9, line_search=0, precision=64,
                           reseed=1, min_part_cell=16, direct_neighbour=direct)
    cap = len(m["x"]) + 4 * g.ncx * g.ncz
    out, mk, rep = run_gpu(g, dict((k, np.array(v_)) for k, v_ in m.items()), u, v, p, mat, model, cap=cap)
    mo = dict((k, np.array(v_)) for k, v_ in m.items())
    uo, vo, po, ro = oracle_step.time_step(g, mat, model, mo, u, v, p)
    assert rep.converged == 1 and ro["converged"] == 1
    assert rep.markers_added == ro["markers_added"] > 0, (rep.markers_added, ro["markers_added"])
    assert len(mk["x"]) == len(mo["x"])
    assert np.array_equal(mk["phase"], mo["phase"])
    for k in ("x", "z", "vx", "vz", "sxxd", "szzd", "sxz", "strain_pl", "strain", "T", "cmul", "P"):
        assert _rel(mk[k], mo[k]) < 1e-8, (k, _rel(mk[k], mo[k]))


def test_multigrid_reuse_same_step():
    """Keeping the multigrid hierarchy for nearly converged iterations
    (mg_reuse_below) reaches the same converged step."""
    g, m, u, v, p, mat = vep_case()
    prm = mdz.RheoParams.make(dt=0.5, iselastic=1, step=1)
    base = dict(newton=1, nit_max=20, rel_tol=1e-11, lin_rtol=1e-9, line_search=0, precision=32, adaptive_lin_tol=1)
    fresh = mdz.Model.make(prm, **base)
    reuse = mdz.Model.make(prm, mg_reuse_below=1e-2, **base)
    out_f, mk_f, rep_f = run_gpu(g, dict((k, np.array(v_)) for k, v_ in m.items()), u, v, p, mat, fresh)
    out_r, mk_r, rep_r = run_gpu(g, dict((k, np.array(v_)) for k, v_ in m.items()), u, v, p, mat, reuse)
    assert rep_f.converged == 1 and rep_r.converged == 1, (rep_f.as_dict(), rep_r.as_dict())
    assert _rel(out_r["u"], out_f["u"]) < 1e-8 and _rel(out_r["v"], out_f["v"]) < 1e-8
    assert _rel(out_r["p"] - out_r["p"].mean(), out_f["p"] - out_f["p"].mean()) < 1e-8
    for k in ("sxxd", "szzd", "sxz", "x", "z"):
        assert _rel(mk_r[k], mk_f[k]) < 1e-8, k
