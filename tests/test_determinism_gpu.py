"""Run-to-run reproducibility: every reduction on the path (residual norms,
Krylov inner products, pressure means, the network's gradient sums) adds its
block partials in a fixed order, so the same inputs give the same bits.  Two
fresh contexts run the same time steps of the lithosphere model and must
agree exactly: iteration histories, fields and markers."""
import numpy as np
import pytest

import mdz
import mdz_setups

pytestmark = pytest.mark.gpu


def _steps(precision, learned, nsteps=2, N=(257, 129)):
    cfg = mdz_setups.config_lithosphere(Nx=N[0], Nz=N[1], precision=precision, learned=learned)
    ctx = mdz_setups.load_context(cfg)
    try:
        loss = mdz_setups.train_guess(ctx, cfg, steps=300, n=1 << 16) if learned else None
        reps = [ctx.time_step(cfg["mat"], cfg["model"]).as_dict() for _ in range(nsteps)]
        g = cfg["grid"]
        u, v, p = np.empty(g.size(-1)), np.empty(g.size(-2)), np.empty(g.size(1))
        ctx._check(ctx.L.mdz_get_velocity(ctx.h, mdz._dptr(u), mdz._dptr(v), mdz._dptr(p)))
        x, z, ph, vx, vz = ctx.get_markers()
        attrs = [ctx.get_marker_attr(a) for a in range(mdz.M_NATTR)]
        w = ctx.mlp_get_weights() if learned else None
    finally:
        ctx.close()
    return loss, reps, (u, v, p, x, z, ph, vx, vz, *attrs), w


@pytest.mark.parametrize("precision,learned", [(64, 0), (32, 1)])
def test_two_runs_identical(precision, learned):
    la, ra, fa, wa = _steps(precision, learned)
    lb, rb, fb, wb = _steps(precision, learned)
    assert la == lb
    if learned:
        assert np.array_equal(wa, wb)
    for a, b in zip(ra, rb):
        for key in ("nonlinear_its", "linear_its", "res_history", "lin_its_history", "lin_rel_history",
                    "local_iterations", "markers_added"):
            assert a[key] == b[key], key
    for a, b in zip(fa, fb):
        assert np.array_equal(a, b)
