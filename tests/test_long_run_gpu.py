"""Consecutive time steps of the lithosphere benchmark model (1025 x 513,
16 markers per cell) in both forms, as the benchmark runs them: every step
converges, the fields stay finite and the marker count stays bounded while
reseeding refills the cells the bottom inflow empties.  Without reseeding the
time step refuses the emptied state with a named status instead of carrying a
zero viscosity into the solver."""
import numpy as np
import pytest

import mdz
import mdz_setups

pytestmark = pytest.mark.gpu

STEPS = 25


def _run(precision, learned, steps, reseed=1):
    cfg = mdz_setups.config_lithosphere(precision=precision, learned=learned)
    cfg["model"].reseed = reseed
    cap = mdz_setups.marker_capacity(cfg)
    ctx = mdz_setups.load_context(cfg, max_markers=cap)
    if learned:
        mdz_setups.train_guess(ctx, cfg, steps=1000)
    reps, counts = [], []
    try:
        for _ in range(steps):
            reps.append(ctx.time_step(cfg["mat"], cfg["model"]))
            counts.append(ctx.n_markers)
        g = cfg["grid"]
        u, v, p = np.empty(g.size(-1)), np.empty(g.size(-2)), np.empty(g.size(1))
        ctx._check(ctx.L.mdz_get_velocity(ctx.h, mdz._dptr(u), mdz._dptr(v), mdz._dptr(p)))
        x, z, ph, _, _ = ctx.get_markers()
        sxx = ctx.get_marker_attr(mdz.M_SXXD)
    finally:
        ctx.close()
    return cfg, cap, reps, counts, (u, v, p), (x, z, ph, sxx)


@pytest.mark.parametrize("precision,learned", [(64, 0), (32, 1)])
def test_lithosphere_consecutive_steps(precision, learned):
    cfg, cap, reps, counts, (u, v, p), (x, z, ph, sxx) = _run(precision, learned, STEPS)
    g = cfg["grid"]
    for k, r in enumerate(reps):
        assert r.converged == 1, (k, r.as_dict())
        assert r.local_failures == 0, (k, r.local_failures)
    assert sum(r.markers_added for r in reps) > 0
    assert max(counts) <= cap
    for a in (u, v, p, sxx):
        assert np.all(np.isfinite(a))
    act = ph >= 0
    assert np.all((x[act] >= g.xmin) & (x[act] <= g.xmax) & (z[act] >= g.zmin) & (z[act] <= g.zmax))
    # every cell keeps markers: the bottom row is refilled by the reseeding
    cx = np.clip(np.floor((x[act] - g.xmin) / g.dx).astype(int), 0, g.ncx - 1)
    cz = np.clip(np.floor((z[act] - g.zmin) / g.dz).astype(int), 0, g.ncz - 1)
    per_cell = np.bincount(cx + cz * g.ncx, minlength=g.ncx * g.ncz)
    assert per_cell.min() >= 4, per_cell.min()


def test_emptied_cells_refused_without_reseeding():
    """The extension's inflow through the bottom wall (0.4 cm/yr, 40 m per
    10 kyr step against 781 m cells) empties the bottom vertex row within
    about ten steps when no markers are added."""
    with pytest.raises(mdz.MdzError) as e:
        _run(64, 0, STEPS, reseed=0)
    assert e.value.status == 7 and "no marker weight" in str(e.value)
