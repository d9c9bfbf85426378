"""GPU linear defect solve (matrix-free GCR + multigrid): the solution of
K dx = F against a direct solve of the reference's assembled blocks (golden),
and on larger seeded problems through the oracle's independent operator."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import mdz
import oracle
from stokes_case import assembled, eqn_maps, reference_state, to_eqn, to_grid

pytestmark = pytest.mark.gpu


def bordered_solve(K, F, n_p):
    """Direct solve with the pressure null space fixed by a zero-mean constraint."""
    n = K.shape[0]
    e = np.zeros(n)
    e[n - n_p:] = 1.0
    Kb = sp.bmat([[K, sp.csr_matrix(e).T], [sp.csr_matrix(e), None]]).tocsc()
    x = spla.spsolve(Kb, np.concatenate([F, [0.0]]))
    return x[:n]


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("jacobian", [0])   # the fixture's random plastic state makes its Jacobian Schur
@pytest.mark.parametrize("precision", [64, 32])   # complement indefinite: Newton solves are covered by the step tests
def test_solve_vs_direct_on_reference_blocks(golden, jacobian, precision):
    ref = golden("rheology_ref.npz")
    g, f = reference_state(ref, jacobian)
    f["eta_n"], f["eta_s"] = ref["vg_eta_n"], ref["vg_eta_s"]
    K = assembled(ref, jacobian)
    maps = eqn_maps(ref)
    n_p = int((maps[2] >= 0).sum())
    F = to_eqn(ref["st_ru"], ref["st_rv"], ref["st_rp"], maps, K.shape[0])
    F[K.shape[0] - n_p:] -= F[K.shape[0] - n_p:].mean()   # compatible with the pressure null space
    want = bordered_solve(K, F, n_p)
    ctx = mdz.Context(g, 3, 1)
    du, dv, dp, its, rel = ctx.SolveStokesDefect(f, jacobian, precision, 1e-11, 400, *to_grid(F, maps, g))
    ctx.close()
    got = to_eqn(du, dv, dp - dp[maps[2] >= 0].mean() * (maps[2] >= 0), maps, K.shape[0])
    assert rel <= 1e-11
    nm = K.shape[0] - n_p
    assert _rel(got[:nm], want[:nm]) < 1e-8
    assert _rel(got[nm:], want[nm:]) < 1e-8


def inclusion_problem(N, contrast, seed=0):
    g = mdz.Grid(N, N, -0.5, 0.5, -0.5, 0.5).set_bc_pureshear(1.0)
    Xc, Zc = np.meshgrid(g.xc, g.zc)
    Xv, Zv = np.meshgrid(g.xg, g.zg)
    eta_n = np.where(np.hypot(Xc, Zc) < 0.1, contrast, 1.0).ravel()
    eta_s = np.where(np.hypot(Xv, Zv) < 0.1, contrast, 1.0).ravel()
    f = mdz.GridFields(g, 1)
    f["eta_n"], f["eta_s"] = eta_n, eta_s
    f["D11_n"], f["D22_n"], f["D33_s"] = 2 * eta_n, 2 * eta_n, eta_s
    # right-hand side of a known smooth solution (a random right-hand side puts
    # the answer in the operator's small singular values, where no solver can
    # verify 1e-8 in FP64)
    ph = float(seed)
    Xu, Zu = np.meshgrid(g.xg, g.zvx)
    Xv, Zv = np.meshgrid(g.xvz, g.zg)
    Xc, Zc = np.meshgrid(g.xc, g.zc)
    xu = (np.sin(3 * Xu + ph) * np.cos(2 * Zu)).ravel() * (g.BCu == -1)
    xv = (np.cos(2 * Xv) * np.sin(3 * Zv + ph)).ravel() * (g.BCv == -1)
    xp = (np.cos(4 * Xc) * Zc).ravel()
    xp -= xp.mean()
    Fu, Fv, Fp = oracle.stokes_apply(g, f, 0, xu, xv, xp)
    f.x_true = (xu, xv, xp)
    return g, f, Fu, Fv, Fp


# FP32 refinement reaches what FP32 stresses resolve on a 1e3 inclusion at
# h = 1/128 (a few 1e-5 of the defect); the Newton loop needs no more per solve
@pytest.mark.parametrize("precision,rtol", [(64, 1e-9), (32, 1e-4)])
def test_solve_inclusion_residual_via_oracle(precision, rtol):
    g, f, Fu, Fv, Fp = inclusion_problem(129, 1e3)
    ctx = mdz.Context(g, 1, 1)
    du, dv, dp, its, rel = ctx.SolveStokesDefect(f, 0, precision, rtol, 500, Fu, Fv, Fp)
    ctx.close()
    ru, rv, rp = oracle.stokes_apply(g, f, 0, du, dv, dp)
    res = np.sqrt(np.sum((ru - Fu) ** 2) + np.sum((rv - Fv) ** 2) + np.sum((rp - Fp) ** 2))
    nrm = np.sqrt(np.sum(Fu ** 2) + np.sum(Fv ** 2) + np.sum(Fp ** 2))
    assert res / nrm < 1.01 * rtol, (res / nrm, its)
    assert its < 60
    xu, xv, xp = f.x_true
    if precision == 64:   # velocity to 1e-6; the pressure of a 1e3 inclusion is conditioned ~100x worse
        assert _rel(du, xu) < 1e-6 and _rel(dv, xv) < 1e-6 and _rel(dp - dp.mean(), xp) < 1e-4


def test_fp32_refined_matches_fp64():
    g, f, Fu, Fv, Fp = inclusion_problem(257, 1e3, seed=2)
    ctx = mdz.Context(g, 1, 1)
    a = ctx.SolveStokesDefect(f, 0, 64, 1e-10, 600, Fu, Fv, Fp)
    b = ctx.SolveStokesDefect(f, 0, 32, 1e-4, 600, Fu, Fv, Fp)
    ctx.close()
    assert a[4] <= 1e-10 and b[4] <= 1e-4
    for x, y in zip(a[:2], b[:2]):
        assert _rel(y, x) < 1e-3


@pytest.mark.parametrize("precision", [64, 32])
def test_newton_defect_solve_vs_direct(precision):
    """The Newton-Jacobian defect equation of the lithosphere model's first
    non-linear iteration (dislocation + diffusion creep with their viscosity
    tangents, elasticity; plasticity off so that the Jacobian's pressure Schur
    complement stays definite): the matrix-free GCR solve against a direct
    solve of the oracle's assembled Jacobian, pressure mean fixed to zero."""
    import mdz_setups
    import oracle_step
    cfg = mdz_setups.config_lithosphere(Nx=65, Nz=33, precision=precision)
    for p in range(cfg["mat"].n_phases):
        cfg["mat"].C[p] = 1e90
    g = cfg["grid"]
    f, F = oracle_step.first_defect(g, cfg["mat"], cfg["model"], cfg["markers"], cfg["u"], cfg["v"], cfg["p"], 1)
    assert np.abs(f["detadexx_n"]).max() > 0   # the tangent is in the operator
    want = oracle_step.solve_defect(g, f, 1, F)
    nu, nv = g.size(-1), g.size(-2)
    Fu, Fv, Fp = F[:nu], F[nu:nu + nv], F[nu + nv:].copy()
    Fp[g.BCp == -1] -= Fp[g.BCp == -1].mean()
    ctx = mdz.Context(g, cfg["mat"].n_phases, 1)
    du, dv, dp, its, rel = ctx.SolveStokesDefect(f, 1, precision, 1e-11, 400, Fu, Fv, Fp)
    ctx.close()
    assert rel <= 1e-11, (rel, its)
    wu, wv, wp = want[:nu], want[nu:nu + nv], want[nu + nv:]
    assert _rel(du, wu) < 1e-8 and _rel(dv, wv) < 1e-8
    assert _rel(dp - dp.mean(), wp - wp.mean()) < 1e-8
