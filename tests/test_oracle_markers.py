"""Pin the CPU oracle's marker-side restatement (P2Mastah, counting,
Interp_Grid2P, RogerGuntherII) against golden vectors produced by the
reference's own compiled functions (tests/golden/make_golden.py)."""
import numpy as np
import pytest

import mdz
from oracle import Oracle


@pytest.fixture(scope="module")
def ref(golden):
    return golden("markers_ref.npz")


def _setup(ref):
    xmin, xmax, zmin, zmax = ref["box"]
    g = mdz.Grid(int(ref["Nx"]), int(ref["Nz"]), xmin, xmax, zmin, zmax).set_bc_pureshear(1.0)
    o = Oracle(g, 3)
    o.set_markers(ref["x"], ref["z"], ref["phase"])
    return g, o


@pytest.mark.parametrize("centroid", [1, 0, -1, -2])
@pytest.mark.parametrize("stencil", [1, 9])
@pytest.mark.parametrize("avg", [0, 1, 2])
@pytest.mark.parametrize("flag", [0, 1])
def test_p2g_matches_reference(ref, centroid, stencil, avg, flag):
    g, o = _setup(ref)
    vals = ref["per_phase"] if flag == 0 else ref["per_marker"]
    init = np.full(g.size(centroid), -7.0)
    got = o.P2Mastah(vals, init, g.tags(centroid), flag, avg, 0, centroid, stencil)
    want = ref["p2g_c%d_s%d_a%d_f%d" % (centroid, stencil, avg, flag)]
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=0)


@pytest.mark.parametrize("centroid", [1, 0])
@pytest.mark.parametrize("stencil", [1, 9])
def test_phase_fractions_match_reference(ref, centroid, stencil):
    g, o = _setup(ref)
    got = o.P2Mastah(ref["per_phase"], None, g.tags(centroid), 0, 0, 1, centroid, stencil)
    np.testing.assert_allclose(got, ref["pp_c%d_s%d" % (centroid, stencil)], rtol=1e-12, atol=1e-15)


def test_counts_bit_exact(ref):
    g, o = _setup(ref)
    c, v, pc, pv = o.count_markers()
    assert np.array_equal(c, ref["count_cell"])
    assert np.array_equal(v, ref["count_vert"])
    assert np.array_equal(pc, ref["pcount_cell"])
    assert np.array_equal(pv, ref["pcount_vert"])


def test_g2p_matches_reference(ref):
    g, o = _setup(ref)
    np.testing.assert_allclose(o.Interp_Grid2P(ref["g2p_vertex_field"], 0), ref["g2p_vertex"], rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(o.Interp_Grid2P(ref["g2p_centroid_field"], 1), ref["g2p_centroid"], rtol=1e-13,
                               atol=1e-15)


def test_rk4_matches_reference(ref):
    g, o = _setup(ref)
    vx, vz = o.RogerGuntherII(ref["rk4_u"], ref["rk4_v"], float(ref["rk4_dt"]))
    assert np.array_equal(o.phase, ref["rk4_phase"])
    assert (ref["rk4_phase"] == -1).sum() > (ref["phase"] == -1).sum()   # some markers left the box
    np.testing.assert_allclose(o.x, ref["rk4_x"], rtol=1e-14, atol=1e-15)
    np.testing.assert_allclose(o.z, ref["rk4_z"], rtol=1e-14, atol=1e-15)
    act = ref["rk4_phase"] != -1
    np.testing.assert_allclose(vx[act], ref["rk4_vx"][act], rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(vz[act], ref["rk4_vz"][act], rtol=1e-13, atol=1e-15)
