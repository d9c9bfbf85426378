"""GPU parity of the matrix-free Stokes residual and Picard / Newton
operators through the C ABI: against the reference's assembled blocks and
residual (golden), and against the oracle on a larger seeded state."""
import numpy as np
import pytest

import mdz
import oracle
from stokes_case import assembled, eqn_maps, reference_state, to_eqn, to_grid

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fixture", ["rheology_ref.npz", "rheology_ref_neumann.npz"])
def test_residual_vs_reference(golden, fixture):
    """Residual rows and norms; the second fixture has Neumann (tag 2) west,
    east and south walls with prescribed tractions and gravity along x."""
    ref = golden(fixture)
    g, f = reference_state(ref, 0)
    ctx = mdz.Context(g, 3, 1)
    norms = ctx.EvaluateStokesResidualDecoupled(f)
    np.testing.assert_allclose(norms, ref["st_norms"], rtol=1e-12)
    for k in ("ru", "rv", "rp"):
        assert np.abs(f[k] - ref["st_" + k]).max() <= 1e-12 * np.abs(ref["st_" + k]).max(), k
    ctx.close()


@pytest.mark.parametrize("fixture", ["rheology_ref.npz", "rheology_ref_neumann.npz"])
@pytest.mark.parametrize("jacobian", [0, 1])
def test_operator_vs_assembled_blocks(golden, jacobian, fixture):
    ref = golden(fixture)
    g, f = reference_state(ref, jacobian)
    K = assembled(ref, jacobian)
    maps = eqn_maps(ref)
    ctx = mdz.Context(g, 3, 1)
    rng = np.random.default_rng(10 + jacobian)
    for _ in range(3):
        x = rng.standard_normal(K.shape[0])
        want = K @ x
        got = to_eqn(*ctx.StokesOperatorApply(f, jacobian, *to_grid(x, maps, g)), maps, K.shape[0])
        assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
    ctx.close()


@pytest.mark.parametrize("jacobian", [0, 1])
def test_operator_vs_oracle_large(jacobian):
    g = mdz.Grid(513, 257, 0.0, 2.0, 0.0, 1.0).set_bc_pureshear(1.0)
    rng = np.random.default_rng(3)
    f = mdz.GridFields(g, 1)
    for k in ("D11_n", "D22_n", "D33_s"):
        f[k] = np.exp(rng.normal(size=f[k].size))
    if jacobian:
        for k in ("D12_n", "D13_n", "D14_n", "D21_n", "D23_n", "D24_n", "D31_s", "D32_s", "D34_s"):
            f[k] = 0.3 * rng.normal(size=f[k].size)
    xu = rng.normal(size=g.size(-1)) * (g.BCu == -1)
    xv = rng.normal(size=g.size(-2)) * (g.BCv == -1)
    xp = rng.normal(size=g.size(1))
    ctx = mdz.Context(g, 1, 1)
    got = ctx.StokesOperatorApply(f, jacobian, xu, xv, xp)
    want = oracle.stokes_apply(g, f, jacobian, xu, xv, xp)
    for a, b in zip(got, want):
        assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max()
    ctx.close()
