"""Pin the oracle's Stokes residual and its Picard / Newton operators against
the reference: residual rows and norms (EvaluateStokesResidualDecoupled) and
the assembled blocks of BuildStokesOperatorDecoupled / BuildJacobianOperatorDecoupled."""
import numpy as np
import pytest

import oracle
from stokes_case import assembled, eqn_maps, reference_state, to_eqn, to_grid


def test_residual_matches_reference(golden):
    ref = golden("rheology_ref.npz")
    g, f = reference_state(ref, 0)
    norms = oracle.residual(g, f)
    np.testing.assert_allclose(norms, ref["st_norms"], rtol=1e-12)
    for k in ("ru", "rv", "rp"):
        scale = np.abs(ref["st_" + k]).max()
        assert np.abs(f[k] - ref["st_" + k]).max() <= 1e-12 * scale, k


@pytest.mark.parametrize("jacobian", [0, 1])
def test_operator_matches_assembled_blocks(golden, jacobian):
    ref = golden("rheology_ref.npz")
    g, f = reference_state(ref, jacobian)
    K = assembled(ref, jacobian)
    maps = eqn_maps(ref)
    rng = np.random.default_rng(jacobian)
    for _ in range(3):
        x = rng.standard_normal(K.shape[0])
        want = K @ x
        got = to_eqn(*oracle.stokes_apply(g, f, jacobian, *to_grid(x, maps, g)), maps, K.shape[0])
        assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()


@pytest.mark.parametrize("jacobian", [0, 1])
def test_inner_rows_next_to_neumann_walls(golden, jacobian):
    """Inner rows of the operators beside Neumann (tag 2) west, east and south
    walls: in the Jacobian the reference leaves out the diagonal couplings to
    a Neumann node (its diagonal Vz neighbours are assembled only where their
    tag is -1).  The wall rows themselves are the GPU's Neumann kernel, pinned
    by the GPU tests."""
    ref = golden("rheology_ref_neumann.npz")
    g, f = reference_state(ref, jacobian)
    K = assembled(ref, jacobian)
    eu, ev, ep = maps = eqn_maps(ref)
    inner = np.ones(K.shape[0], bool)
    inner[eu[(g.BCu == 2) & (eu >= 0)]] = False
    inner[ev[(g.BCv == 2) & (ev >= 0)]] = False
    rng = np.random.default_rng(20 + jacobian)
    x = rng.standard_normal(K.shape[0])
    want = K @ x
    got = to_eqn(*oracle.stokes_apply(g, f, jacobian, *to_grid(x, maps, g)), maps, K.shape[0])
    assert np.abs(got - want)[inner].max() <= 1e-12 * np.abs(want).max()
