"""The benchmark's lithosphere model (four phases, dislocation + diffusion
creep, elasticity, Drucker-Prager plasticity, gravity, extension, reseeding)
at 257 x 129: one time step of each GPU form against the oracle's FP64 time
step (restated reference functions, exact defect solves) on the same inputs.
Velocity, pressure (mean removed), marker stresses, strains and positions
agree within 1e-8 relative in the 2-norm; markers created by the reseeding and
phases agree exactly."""
import numpy as np
import pytest

import mdz
import mdz_setups
import oracle_step

pytestmark = pytest.mark.gpu

TOL = 1e-8
N = (257, 129)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def oracle_result():
    cfg = mdz_setups.config_lithosphere(Nx=N[0], Nz=N[1], precision=64)
    m = {k: v.copy() for k, v in cfg["markers"].items()}
    u, v, p, rep = oracle_step.time_step(cfg["grid"], cfg["mat"], cfg["model"], m, cfg["u"], cfg["v"], cfg["p"])
    assert rep["converged"] == 1
    return dict(u=u, v=v, p=p, m=m, rep=rep)


def gpu_step(precision, learned):
    cfg = mdz_setups.config_lithosphere(Nx=N[0], Nz=N[1], precision=precision, learned=learned)
    ctx = mdz_setups.load_context(cfg)
    try:
        if learned:
            mdz_setups.train_guess(ctx, cfg, steps=1000, n=1 << 18)
        rep = ctx.time_step(cfg["mat"], cfg["model"])
        g = cfg["grid"]
        u, v, p = np.empty(g.size(-1)), np.empty(g.size(-2)), np.empty(g.size(1))
        ctx._check(ctx.L.mdz_get_velocity(ctx.h, mdz._dptr(u), mdz._dptr(v), mdz._dptr(p)))
        x, z, ph, vx, vz = ctx.get_markers()
        mk = dict(x=x, z=z, phase=ph, vx=vx, vz=vz)
        for a, key in enumerate(("sxxd", "szzd", "sxz", "strain_pl", "strain", "T", "cmul")):
            mk[key] = ctx.get_marker_attr(a)
    finally:
        ctx.close()
    return rep, dict(u=u, v=v, p=p, m=mk)


@pytest.mark.parametrize("precision,learned", [(64, 0), (32, 1)])
def test_lithosphere_step_vs_oracle(oracle_result, precision, learned):
    rep, out = gpu_step(precision, learned)
    o = oracle_result
    assert rep.converged == 1, rep.as_dict()
    assert rep.markers_added == o["rep"]["markers_added"]
    assert _rel(out["u"], o["u"]) < TOL and _rel(out["v"], o["v"]) < TOL
    assert _rel(out["p"] - out["p"].mean(), o["p"] - o["p"].mean()) < TOL
    mk, mo = out["m"], o["m"]
    assert len(mk["x"]) == len(mo["x"])
    assert np.array_equal(mk["phase"], mo["phase"])
    for k in ("x", "z", "sxxd", "szzd", "sxz", "strain", "vx", "vz"):
        assert _rel(mk[k], mo[k]) < TOL, (k, _rel(mk[k], mo[k]))
