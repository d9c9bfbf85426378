"""The benchmark configurations other than the lithosphere model, at their
stated sizes:

* inclusion (101 x 101, linear viscous pure shear, circular inclusion 1e3,
  4 x 4 markers per cell, one Stokes solve and one RK4 step, dt = 1e-3):
  both GPU forms against the oracle's time step;
* visco-elasto-plastic Drucker-Prager pure shear (401 x 401, G = 1,
  eta = 1e3, C = 1 with 1 % per-marker noise, phi = 30 deg, dt = 1e-2,
  4 x 4 markers per cell, box deforming with the flow): 20 steps of at most
  10 Newton iterations in both forms, every step converged, the two forms'
  fields in agreement, the walls where the pure shear puts them and the
  marker stresses on the Maxwell loading curve (the stress stays below the
  yield stress for these 20 steps), and the first two steps against the
  oracle at 101 x 101;
* shear-band localisation (2049 x 2049, cohesion softening linearly from 1 to
  0.5 over plastic strain 0-1, 1 % noise, 16 markers per cell = 67M markers,
  reseeding on, deforming box, Courant-limited step dt = dx, G = 100 so
  that yielding starts near step 9): 50 steps of at most 15 Newton
  iterations in the FP32-refined form, every step converged, the plastic
  strain growing where the material yields."""
import time

import numpy as np
import pytest

import mdz
import mdz_setups
import oracle_step

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _state(ctx, g):
    u, v, p = np.empty(g.size(-1)), np.empty(g.size(-2)), np.empty(g.size(1))
    ctx._check(ctx.L.mdz_get_velocity(ctx.h, mdz._dptr(u), mdz._dptr(v), mdz._dptr(p)))
    x, z, ph, _, _ = ctx.get_markers()
    return dict(u=u, v=v, p=p - p.mean(), x=x, z=z, phase=ph, sxxd=ctx.get_marker_attr(mdz.M_SXXD),
                sxz=ctx.get_marker_attr(mdz.M_SXZ), strain_pl=ctx.get_marker_attr(mdz.M_STRAIN_PL))


def _run(cfg, precision, steps):
    cfg["model"].precision = precision
    ctx = mdz_setups.load_context(cfg)
    reps, ms = [], []
    try:
        for _ in range(steps):
            t0 = time.perf_counter()
            reps.append(mdz_setups.time_step(ctx, cfg))
            ms.append((time.perf_counter() - t0) * 1e3)
        out = _state(ctx, cfg["grid"])
    finally:
        ctx.close()
    return reps, ms, out


def _oracle(cfg, steps):
    m = {k: v.copy() for k, v in cfg["markers"].items()}
    u, v, p = cfg["u"], cfg["v"], cfg["p"]
    for _ in range(steps):
        u, v, p, rep = oracle_step.time_step(cfg["grid"], cfg["mat"], cfg["model"], m, u, v, p)
        assert rep["converged"] == 1
        mdz_setups.renew_bcs(cfg)
    return dict(u=u, v=v, p=p - p.mean(), x=m["x"], z=m["z"], phase=m["phase"], sxxd=m["sxxd"], sxz=m["sxz"])


@pytest.mark.parametrize("precision", [64, 32])
def test_inclusion_101_vs_oracle(precision):
    reps, ms, out = _run(mdz_setups.config_inclusion(), precision, 1)
    assert reps[0].converged == 1
    want = _oracle(mdz_setups.config_inclusion(), 1)
    for k in ("u", "v", "p", "x", "z"):
        assert _rel(out[k], want[k]) < 1e-8, (k, _rel(out[k], want[k]))
    assert np.array_equal(out["phase"], want["phase"])


def test_vep_101_two_steps_vs_oracle():
    cfg = mdz_setups.config_vep(N=101)
    reps, ms, out = _run(cfg, 64, 2)
    assert all(r.converged == 1 for r in reps)
    want_cfg = mdz_setups.config_vep(N=101)
    want = _oracle(want_cfg, 2)
    g, h = cfg["grid"], want_cfg["grid"]
    assert (g.xmin, g.xmax, g.zmin, g.zmax) == (h.xmin, h.xmax, h.zmin, h.zmax)
    assert np.array_equal(g.xg, h.xg) and np.array_equal(g.zc, h.zc)
    assert len(out["x"]) == len(want["x"])
    for k in ("u", "v", "x", "z", "sxxd"):
        assert _rel(out[k], want[k]) < 1e-8, (k, _rel(out[k], want[k]))
    # homogeneous loading: pressure and shear stress are round-off of the
    # stress level (|sxxd| ~ 0.04), compared absolutely
    for k in ("p", "sxz"):
        assert np.abs(out[k] - want[k]).max() < 1e-12, (k, np.abs(out[k] - want[k]).max())
    assert np.array_equal(out["phase"], want["phase"])


def _maxwell_sxxd(steps, G=1.0, eta=1e3, dt=1e-2, exxd=-1.0):
    """Deviatoric stress of Maxwell loading at constant strain rate, stepped as
    the visco-elastic update does: s <- 2 eta_ve (exxd + s / (2 G dt))."""
    eta_ve = 1.0 / (1.0 / eta + 1.0 / (G * dt))
    s = 0.0
    for _ in range(steps):
        s = 2.0 * eta_ve * (exxd + s / (2.0 * G * dt))
    return s


def test_vep_401_twenty_steps_both_forms():
    r64, ms64, o64 = _run(mdz_setups.config_vep(), 64, 20)
    r32, ms32, o32 = _run(mdz_setups.config_vep(), 32, 20)
    for reps in (r64, r32):
        for k, r in enumerate(reps):
            assert r.converged == 1 and r.nonlinear_its <= 10, (k, r.as_dict())
    # the walls move with the pure shear: x = -/+0.5 (1 - dt)^n, z = -/+0.5 (1 + dt)^n
    last = r64[-1]
    np.testing.assert_allclose([last.xmin, last.xmax, last.zmin, last.zmax],
                               [-0.5 * 0.99 ** 20, 0.5 * 0.99 ** 20, -0.5 * 1.01 ** 20, 0.5 * 1.01 ** 20], rtol=1e-12)
    # homogeneous elastic loading, below the yield stress (C cos(phi) = 0.866)
    s20 = _maxwell_sxxd(20)
    assert abs(s20) < 0.866
    act = o64["phase"] >= 0
    np.testing.assert_allclose(o64["sxxd"][act], s20, rtol=1e-6)
    assert np.abs(o64["sxz"][act]).max() < 1e-8 * abs(s20)
    for k in ("u", "v", "p", "sxxd", "sxz"):
        assert _rel(o32[k], o64[k]) < 1e-6 or np.abs(o32[k] - o64[k]).max() < 1e-12, (k, _rel(o32[k], o64[k]))
    print("vep 401: ms/step plain %.1f, FP32-refined %.1f" % (np.mean(ms64[1:]), np.mean(ms32[1:])))


def test_shear_band_2049_fifty_steps():
    cfg = mdz_setups.config_shear_band(precision=32)
    n0 = len(cfg["markers"]["x"])
    assert n0 == 2048 * 2048 * 16
    reps, ms, out = _run(cfg, 32, 50)
    for k, r in enumerate(reps):
        assert r.converged == 1 and r.nonlinear_its <= 15, (k, r.as_dict())
    act = out["phase"] >= 0
    assert out["strain_pl"][act].max() > 0.0
    print("shear band 2049: ms/step %.1f (steps 2-50), markers %d -> %d" % (np.mean(ms[1:]), n0, len(out["x"])))
