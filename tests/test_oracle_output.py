"""Pin the output-preparation oracle to the reference: the phase maps of
Interp_Phase2VizGrid at 1x and 2x resolution (golden fixture, bit for bit)."""
import numpy as np
import pytest

import oracle_output


@pytest.mark.parametrize("res", [1, 2])
def test_phase_map_matches_reference(golden, res):
    ref = golden("phasemap_ref.npz")
    Nx, Nz = int(ref["Nx"]), int(ref["Nz"])
    xmin, xmax, zmin, zmax = ref["box"]
    import mdz
    g = mdz.Grid(Nx, Nz, xmin, xmax, zmin, zmax)
    compo, X, Z = oracle_output.phase_viz(g.xg[0], g.zg[0], g.dx, g.dz, g.xc[0], g.zc[0], Nx - 1, Nz - 1, ref["BCp"],
                                          ref["x"], ref["z"], ref["phase"], res)
    assert np.array_equal(X, ref["xviz_r%d" % res]) and np.array_equal(Z, ref["zviz_r%d" % res])
    assert np.array_equal(compo, ref["compo_r%d" % res])
    assert (compo == -1).sum() > 0 and len(np.unique(compo)) == 4   # air cells and all three phases present


def test_cast_scale_rounds_twice():
    a = np.array([1.0 / 3.0, 2.0 ** -30, -7.25, 1e300])
    out = oracle_output.cast_scale(a, 3.0)
    assert out.dtype == np.float32
    assert out[0] == np.float32(np.float64(np.float32(1.0 / 3.0)) * 3.0)
    assert np.isinf(out[3])
