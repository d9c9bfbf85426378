"""GPU parity of the marker-side kernels (projection, counting, grid->marker,
RK4) through the C ABI, against the golden fixtures from the reference and
against the CPU oracle on larger seeded inputs."""
import numpy as np
import pytest

import mdz
import mdz_setups
from oracle import Oracle

pytestmark = pytest.mark.gpu

RTOL_FIELD = 1e-12     # tent-weighted fields: summation order differs from the reference


@pytest.fixture(scope="module")
def ref(golden):
    return golden("markers_ref.npz")


@pytest.fixture(scope="module")
def gctx(ref):
    xmin, xmax, zmin, zmax = ref["box"]
    g = mdz.Grid(int(ref["Nx"]), int(ref["Nz"]), xmin, xmax, zmin, zmax).set_bc_pureshear(1.0)
    ctx = mdz.Context(g, 3, len(ref["x"]) + 16)
    ctx.set_markers(ref["x"], ref["z"], ref["phase"])
    yield g, ctx
    ctx.close()


@pytest.mark.parametrize("centroid", [1, 0, -1, -2])
@pytest.mark.parametrize("stencil", [1, 9])
@pytest.mark.parametrize("avg", [0, 1, 2])
@pytest.mark.parametrize("flag", [0, 1])
def test_p2g_vs_reference(ref, gctx, centroid, stencil, avg, flag):
    g, ctx = gctx
    vals = ref["per_phase"] if flag == 0 else ref["per_marker"]
    got = ctx.P2Mastah(vals, np.full(g.size(centroid), -7.0), g.tags(centroid), flag, avg, 0, centroid, stencil)
    np.testing.assert_allclose(got, ref["p2g_c%d_s%d_a%d_f%d" % (centroid, stencil, avg, flag)], rtol=RTOL_FIELD)


@pytest.mark.parametrize("centroid", [1, 0])
@pytest.mark.parametrize("stencil", [1, 9])
def test_phase_fractions_vs_reference(ref, gctx, centroid, stencil):
    g, ctx = gctx
    got = ctx.P2Mastah(ref["per_phase"], None, g.tags(centroid), 0, 0, 1, centroid, stencil)
    np.testing.assert_allclose(got, ref["pp_c%d_s%d" % (centroid, stencil)], rtol=RTOL_FIELD, atol=1e-15)


def test_counts_bit_exact_vs_reference(ref, gctx):
    g, ctx = gctx
    c, v, pc, pv = ctx.count_markers()
    assert np.array_equal(c, ref["count_cell"]) and np.array_equal(v, ref["count_vert"])
    assert np.array_equal(pc, ref["pcount_cell"]) and np.array_equal(pv, ref["pcount_vert"])


def test_g2p_vs_reference(ref, gctx):
    g, ctx = gctx
    np.testing.assert_allclose(ctx.Interp_Grid2P(ref["g2p_vertex_field"], 0), ref["g2p_vertex"], rtol=1e-13,
                               atol=1e-15)
    np.testing.assert_allclose(ctx.Interp_Grid2P(ref["g2p_centroid_field"], 1), ref["g2p_centroid"], rtol=1e-13,
                               atol=1e-15)


def test_rk4_vs_reference(ref):
    xmin, xmax, zmin, zmax = ref["box"]
    g = mdz.Grid(int(ref["Nx"]), int(ref["Nz"]), xmin, xmax, zmin, zmax).set_bc_pureshear(1.0)
    ctx = mdz.Context(g, 3, len(ref["x"]))
    ctx.set_markers(ref["x"], ref["z"], ref["phase"])
    ctx.RogerGuntherII(ref["rk4_u"], ref["rk4_v"], float(ref["rk4_dt"]))
    x, z, ph, vx, vz = ctx.get_markers()
    ctx.close()
    assert np.array_equal(ph, ref["rk4_phase"])
    np.testing.assert_allclose(x, ref["rk4_x"], rtol=1e-14, atol=1e-15)
    np.testing.assert_allclose(z, ref["rk4_z"], rtol=1e-14, atol=1e-15)
    act = ph != -1
    np.testing.assert_allclose(vx[act], ref["rk4_vx"][act], rtol=1e-13, atol=1e-15)


# ---- larger seeded cases against the oracle ---------------------------------
def _seeded(Nx, Nz, nm, seed, nph=4):
    g = mdz.Grid(Nx, Nz, 0.0, 1.0 * (Nx - 1) / (Nz - 1), 0.0, 1.0).set_bc_pureshear(1.0)
    x, z = mdz_setups.seed_markers(g, nm, nm, 0.5, seed)
    rng = np.random.default_rng(seed)
    ph = rng.integers(0, nph, len(x)).astype(np.int32)
    ph[rng.random(len(x)) < 0.01] = -1
    perm = rng.permutation(len(x))          # arbitrary marker order
    return g, x[perm], z[perm], ph[perm]


@pytest.mark.parametrize("Nx,Nz,nm", [(101, 101, 4), (65, 33, 5), (3, 3, 2)])
def test_p2g_batched_vs_oracle(Nx, Nz, nm):
    g, x, z, ph = _seeded(Nx, Nz, nm, seed=Nx)
    rng = np.random.default_rng(1)
    vals = [np.exp(rng.normal(size=len(x))) for _ in range(3)]
    ctx = mdz.Context(g, 4, len(x))
    ctx.set_markers(x, z, ph)
    o = Oracle(g, 4)
    o.set_markers(x, z, ph)
    for centroid in (1, 0, -1, -2):
        for stencil in (1, 9):
            for avg, v in zip((0, 1, 2), vals):
                init = np.zeros(g.size(centroid))
                got = ctx.P2Mastah(v, init, g.tags(centroid), 1, avg, 0, centroid, stencil)
                want = o.P2Mastah(v, init, g.tags(centroid), 1, avg, 0, centroid, stencil)
                np.testing.assert_allclose(got, want, rtol=RTOL_FIELD, err_msg="c%d s%d a%d" % (centroid, stencil, avg))
    c, v, pc, pv = ctx.count_markers()
    oc, ov, opc, opv = o.count_markers()
    assert np.array_equal(c, oc) and np.array_equal(v, ov) and np.array_equal(pc, opc) and np.array_equal(pv, opv)
    ctx.close()


def test_p2g_deterministic_and_order_independent():
    g, x, z, ph = _seeded(129, 65, 4, seed=3)
    val = np.linspace(1.0, 2.0, len(x))
    ctx = mdz.Context(g, 4, len(x))
    ctx.set_markers(x, z, ph)
    a = ctx.P2Mastah(val, None, g.tags(0), 1, 0, 0, 0, 9)
    b = ctx.P2Mastah(val, None, g.tags(0), 1, 0, 0, 0, 9)
    assert np.array_equal(a, b)                      # bit-reproducible run to run
    perm = np.random.default_rng(0).permutation(len(x))
    ctx.set_markers(x[perm], z[perm], ph[perm])
    c = ctx.P2Mastah(val[perm], None, g.tags(0), 1, 0, 0, 0, 9)
    np.testing.assert_allclose(c, a, rtol=1e-13)     # marker order only changes rounding
    ctx.close()


def test_empty_marker_set_leaves_field_untouched():
    g = mdz.Grid(9, 9, 0, 1, 0, 1).set_bc_pureshear(1.0)
    ctx = mdz.Context(g, 2, 10)
    ctx.set_markers(np.zeros(0), np.zeros(0), np.zeros(0, np.int32))
    init = np.full(g.size(1), 3.25)
    assert np.array_equal(ctx.P2Mastah(np.array([1.0, 2.0]), init, g.tags(1), 0, 0, 0, 1, 1), init)
    c, v, pc, pv = ctx.count_markers()
    assert c.sum() == 0 and v.sum() == 0
    ctx.close()


def test_capacity_is_enforced():
    g = mdz.Grid(9, 9, 0, 1, 0, 1).set_bc_pureshear(1.0)
    ctx = mdz.Context(g, 2, 10)
    with pytest.raises(mdz.MdzError) as e:
        ctx.set_markers(np.zeros(11), np.zeros(11), np.zeros(11, np.int32))
    assert e.value.status == 3
    ctx.close()


def test_g2p_rk4_vs_oracle_large():
    g, x, z, ph = _seeded(257, 129, 4, seed=11)
    ctx = mdz.Context(g, 4, len(x))
    ctx.set_markers(x, z, ph)
    o = Oracle(g, 4)
    o.set_markers(x, z, ph)
    fv = np.sin(5 * g.xg)[None, :] * np.cos(3 * g.zg)[:, None]
    fc = np.cos(4 * g.xc)[None, :] * np.sin(2 * g.zc)[:, None]
    np.testing.assert_allclose(ctx.Interp_Grid2P(fv.ravel(), 0), o.Interp_Grid2P(fv.ravel(), 0), rtol=1e-13,
                               atol=1e-15)
    np.testing.assert_allclose(ctx.Interp_Grid2P(fc.ravel(), 1), o.Interp_Grid2P(fc.ravel(), 1), rtol=1e-13,
                               atol=1e-15)
    U = (-g.xg[None, :] + 0.2 * np.sin(np.pi * g.zvx[:, None])).ravel()
    V = (g.zg[:, None] + 0.1 * np.cos(np.pi * g.xvz[None, :])).ravel()
    ctx.RogerGuntherII(U, V, 0.02)
    ovx, ovz = o.RogerGuntherII(U, V, 0.02)
    gx, gz, gph, gvx, gvz = ctx.get_markers()
    assert np.array_equal(gph, o.phase)
    np.testing.assert_allclose(gx, o.x, rtol=1e-14, atol=1e-15)
    np.testing.assert_allclose(gz, o.z, rtol=1e-14, atol=1e-15)
    ctx.close()


def test_registered_host_round_trip(ref, gctx):
    """Markers uploaded from page-locked (registered) host arrays and read back
    into registered arrays come back bit for bit; attributes likewise."""
    g, ctx = gctx
    n = len(ref["x"])
    x = np.ascontiguousarray(ref["x"], np.float64).copy()
    z = np.ascontiguousarray(ref["z"], np.float64).copy()
    ph = np.ascontiguousarray(ref["phase"], np.int32).copy()
    out = [np.zeros(n), np.zeros(n), np.zeros(n, np.int32), np.zeros(n), np.zeros(n)]
    attr_in = np.linspace(-1.0, 1.0, n)
    attr_out = np.zeros(n)
    arrays = [x, z, ph, attr_in, attr_out] + out
    for a in arrays:
        mdz.host_register(a)
    try:
        ctx.set_markers(x, z, ph)
        ctx.set_marker_attr(mdz.M_SXXD, attr_in)
        ctx.get_markers(out=out)
        ctx.get_marker_attr(mdz.M_SXXD, out=attr_out)
    finally:
        for a in arrays:
            mdz.host_unregister(a)
        ctx.set_markers(ref["x"], ref["z"], ref["phase"])
    np.testing.assert_array_equal(out[0], x)
    np.testing.assert_array_equal(out[1], z)
    np.testing.assert_array_equal(out[2], ph)
    np.testing.assert_array_equal(attr_out, attr_in)
