"""UpdateParticlePressure on the GPU (mdz_UpdateParticlePressure) against the
reference's own function (golden fixture pressure_ref.npz: random marker
pressures, random p_in and p0_n on a 21 x 17 grid, Plith_trick = 0)."""
import numpy as np
import pytest

import mdz

pytestmark = pytest.mark.gpu


def test_update_particle_pressure_vs_reference(golden):
    ref = golden("pressure_ref.npz")
    xmin, xmax, zmin, zmax = ref["box"]
    g = mdz.Grid(int(ref["Nx"]), int(ref["Nz"]), xmin, xmax, zmin, zmax).set_bc_pureshear(1.0)
    ctx = mdz.Context(g, 3, len(ref["x"]))
    ctx.set_markers(ref["x"], ref["z"], ref["phase"])
    ctx.set_marker_attr(mdz.M_P, ref["P0"])
    f = mdz.GridFields(g, 3)
    f["p"], f["p0_n"] = ref["p_in"], ref["p0_n"]
    ctx.UpdateParticlePressure(f)
    P = ctx.get_marker_attr(mdz.M_P)
    sxx = ctx.get_marker_attr(mdz.M_SXXD)
    ctx.close()
    act = ref["phase"] != -1
    np.testing.assert_allclose(P[act], ref["P_trick0"][act], rtol=1e-13, atol=1e-13)
    assert np.array_equal(P[~act], ref["P0"][~act])
    assert not sxx.any()   # the other attributes are left alone
