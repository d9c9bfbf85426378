"""Pin the CPU oracle's marker updates against golden vectors produced by the
reference's own compiled functions (tests/golden/make_golden.py): the
reseeding (CountPartCell with RESEED = 1 on one thread: quarter-cell counts,
AddPartCell2, FindClosestPhase2, slot reuse, AssignMarkerProperties),
UpdateParticleStress and AccumulatedStrainII."""
import numpy as np
import pytest

import mdz
import oracle

ATTRS = ("vx", "vz", "sxxd", "szzd", "sxz", "strain", "strain_pl", "T", "P")


@pytest.fixture(scope="module")
def ref(golden):
    return golden("reseed_ref.npz")


def reseed_case(ref):
    """Grid and input markers of the fixture (the cohesion multiplier, which
    the reference does not carry, is the marker index)."""
    xmin, xmax, zmin, zmax = ref["box"]
    g = mdz.Grid(int(ref["Nx"]), int(ref["Nz"]), xmin, xmax, zmin, zmax).set_bc_pureshear(1.0)
    m = {k: np.array(ref["in_" + k]) for k in ("x", "z", "phase") + ATTRS}
    m["cmul"] = np.arange(len(m["x"]), dtype=np.float64)
    return g, m


@pytest.mark.parametrize("direct", [1, 0])
@pytest.mark.parametrize("mpc", [16, 9])
def test_reseed_matches_reference(ref, direct, mpc):
    g, m = reseed_case(ref)
    n = len(m["x"])
    cap = n + 4 * (g.Nx - 1) * (g.Nz - 1)
    out, added = oracle.reseed(g, m, cap, mpc, direct, ref["T_n"], ref["sxxd_n"], ref["szzd_n"], ref["sxz_s"],
                                 ref["p_n"])
    tag = "d%d_m%d_" % (direct, mpc)
    assert len(out["x"]) == int(ref[tag + "n"])
    slots = ref[tag + "slots"]
    assert added >= len(slots) - np.count_nonzero(slots < n) and added > 0
    for k in ("x", "z", "phase") + ATTRS:     # bit for bit, copies and interpolations alike
        assert np.array_equal(out[k][slots], ref[tag + k]), k
    untouched = np.setdiff1d(np.arange(n), slots)
    for k in ("x", "z", "phase", "cmul") + ATTRS:
        assert np.array_equal(out[k][untouched], m[k][untouched]), k
    # the cohesion multiplier (not a reference attribute) travels with the copied marker
    src = out["cmul"][slots].astype(np.int64)
    assert np.array_equal(out["phase"][slots], m["phase"][src])


def test_reseed_no_neighbours_raises(ref):
    g, m = reseed_case(ref)
    keep = m["x"] > 0.0           # the west half is empty: its quarter cells have no neighbours
    mm = {k: v[keep] for k, v in m.items()}
    with pytest.raises(RuntimeError):
        oracle.reseed(g, mm, len(mm["x"]) + 4 * (g.Nx - 1) * (g.Nz - 1), 16, 1)


def test_reseed_capacity(ref):
    g, m = reseed_case(ref)
    with pytest.raises(RuntimeError):
        oracle.reseed(g, m, len(m["x"]) + 1, 16, 1)


def test_accumulated_strain_matches_reference(golden):
    """The oracle step's AccumulatedStrainII restatement against the
    reference's own AccumulatedStrainII (RheologyParticles.c:191-537)."""
    import oracle_step
    ref = golden("strain_ref.npz")
    xmin, xmax, zmin, zmax = ref["box"]
    g = mdz.Grid(int(ref["Nx"]), int(ref["Nz"]), xmin, xmax, zmin, zmax).set_bc_pureshear(1.0)
    dt = float(ref["dt"])
    dstr = dt * (ref["eII_pl"] + ref["eII_pwl"] + ref["eII_lin"] + ref["eII_el"] + ref["eII_cst"])
    dstr_pl = dt * ref["eII_pl"]
    m = dict(x=ref["x"], z=ref["z"], phase=ref["phase"])
    e, ep = oracle_step._accumulated_strain(g, m, dstr, dstr_pl)
    for got, key, base in ((e, "strain", "strain0"), (ep, "strain_pl", "strain_pl0")):
        want = ref[key] - ref[base]
        assert np.allclose(got, want, rtol=1e-13, atol=1e-15), (key, np.abs(got - want).max())
    assert (e[ref["phase"] == -1] == 0).all() and (e > 0).any()


def test_update_particle_stress_matches_reference(golden):
    """The oracle step's UpdateParticleStress (no rotation, no subgrid
    diffusion) against the reference's own (RheologyParticles.c:1124-1447)."""
    import oracle_step
    from oracle import Oracle
    ref = golden("stress_ref.npz")
    xmin, xmax, zmin, zmax = ref["box"]
    g = mdz.Grid(int(ref["Nx"]), int(ref["Nz"]), xmin, xmax, zmin, zmax).set_bc_pureshear(1.0)
    o = Oracle(g, 3)
    o.set_markers(ref["x"], ref["z"], ref["phase"])
    f = {k: ref[k] for k in ("sxxd", "szzd", "sxxd0", "szzd0", "sxz", "sxz0")}
    m = {"phase": ref["phase"], **{k: np.array(ref["m0_" + k]) for k in ("sxxd", "szzd", "sxz")}}
    oracle_step.update_particle_stress(g, o, f, m)
    for k in ("sxxd", "szzd", "sxz"):
        want = ref["m_" + k]
        assert np.allclose(m[k], want, rtol=1e-13, atol=1e-14), (k, np.abs(m[k] - want).max())
        assert not np.array_equal(want, ref["m0_" + k])


def test_update_particle_pressure_matches_reference(golden):
    """UpdateParticlePressure (Plith_trick = 0, no subgrid diffusion): the
    oracle's centroid increment p_in - p0_n interpolated to the markers."""
    import oracle_step
    ref = golden("pressure_ref.npz")
    xmin, xmax, zmin, zmax = ref["box"]
    g = mdz.Grid(int(ref["Nx"]), int(ref["Nz"]), xmin, xmax, zmin, zmax).set_bc_pureshear(1.0)
    o = oracle.Oracle(g, 3)
    o.set_markers(ref["x"], ref["z"], ref["phase"])
    m = dict(phase=np.array(ref["phase"]), P=np.array(ref["P0"]))
    oracle_step.update_particle_pressure(g, o, ref["p0_n"], ref["p_in"], m)
    np.testing.assert_allclose(m["P"], ref["P_trick0"], rtol=1e-13, atol=1e-13)
