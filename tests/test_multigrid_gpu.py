"""Multigrid hierarchy on the device against its CPU restatement: the level-0
stencils equal the oracle's assembled velocity block, and every coarser level
equals the Galerkin product P^T A P of the level above."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

import mdz
import oracle_step
from mg_reference import prolongation, stencil_matrix, velocity_block
from test_solver_gpu import inclusion_problem

pytestmark = pytest.mark.gpu


def _rel(A, B):
    return spla.norm(A - B) / spla.norm(B)


@pytest.mark.parametrize("precision,tol", [(64, 1e-12), (32, 2e-6)])
def test_galerkin_hierarchy(precision, tol):
    g, f, Fu, Fv, Fp = inclusion_problem(65, 1e3)
    ctx = mdz.Context(g, 1, 1)
    ctx.SolveStokesDefect(f, 0, precision, 1e-6, 300, Fu, Fv, Fp)
    nl, nx, nz, su, sv = ctx.mg_stencils(precision, 0)
    assert nl >= 4
    A, dropped = stencil_matrix(nx, nz, su, sv)
    assert dropped == 0.0
    K, idx, n, n_p = oracle_step.assemble(g, f, 0)
    assert _rel(A, velocity_block(g, K, idx)) < tol
    for level in range(1, nl):
        _, ncx, ncz, suc, svc = ctx.mg_stencils(precision, level)
        Ac, dropped = stencil_matrix(ncx, ncz, suc, svc)
        assert dropped == 0.0
        P = prolongation(nx, nz)
        assert _rel(Ac, (P.T @ A @ P).tocsr()) < tol, level
        A, nx, nz = Ac, ncx, ncz
    ctx.close()


@pytest.mark.parametrize("precision,tol", [(64, 1e-12), (32, 2e-6)])
def test_newton_hierarchy_on_reference_state(golden, precision, tol):
    """Newton Jacobian blocks of the reference's fixture state: the probed
    level-0 stencils are the assembled Jacobian's velocity block."""
    from stokes_case import reference_state
    ref = golden("rheology_ref.npz")
    g, f = reference_state(ref, 1)
    f["eta_n"], f["eta_s"] = ref["vg_eta_n"], ref["vg_eta_s"]
    ctx = mdz.Context(g, 3, 1)
    ctx.set_solver_options(mg_jacobian=1)
    z = [np.zeros(g.size(-1)), np.zeros(g.size(-2)), np.zeros(g.size(1))]
    z[0][g.BCu == -1] = 1.0
    try:
        ctx.SolveStokesDefect(f, 1, precision, 1e-3, 20, *z)
    except mdz.MdzError:
        pass   # the hierarchy exists after the first preconditioner setup
    nl, nx, nz, su, sv = ctx.mg_stencils(precision, 0)
    A, dropped = stencil_matrix(nx, nz, su, sv)
    assert dropped == 0.0
    K, idx, n, n_p = oracle_step.assemble(g, f, 1)
    assert _rel(A, velocity_block(g, K, idx)) < tol
    for level in range(1, nl):
        _, ncx, ncz, suc, svc = ctx.mg_stencils(precision, level)
        Ac, _ = stencil_matrix(ncx, ncz, suc, svc)
        P = prolongation(nx, nz)
        assert _rel(Ac, (P.T @ A @ P).tocsr()) < tol, level
        A, nx, nz = Ac, ncx, ncz
    ctx.close()
