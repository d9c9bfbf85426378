"""ShearModCompExpGrid and CohesionFrictionDilationGrid on the GPU against the
reference's own functions (golden fixture gridprops_ref.npz: phase fractions
projected from jittered markers of three phases, random plastic strains across
the softening windows, itp_stencil 1 and 9)."""
import numpy as np
import pytest

import mdz

pytestmark = pytest.mark.gpu

PHASES = [
    dict(mu=1.0, bet=1e-2, C=1.0, phi=0.5, psi=0.1, C_end=0.5, phi_end=0.3, psi_end=0.0, pls_start=0.1, pls_end=0.9,
         coh_soft=1, phi_soft=1, psi_soft=1),
    dict(mu=2.0, bet=2e-2, C=2.0, phi=0.6, psi=0.0, C_end=0.2, phi_end=0.6, psi_end=0.0, pls_start=0.0, pls_end=0.5,
         coh_soft=1, phi_soft=0, psi_soft=0),
    dict(mu=0.5, bet=5e-3, C=0.7, phi=0.4, psi=0.05, C_end=0.7, phi_end=0.4, psi_end=0.05, pls_start=0.0,
         pls_end=1.0, coh_soft=0, phi_soft=0, psi_soft=0),
]


@pytest.mark.parametrize("stencil", [1, 9])
def test_grid_properties_vs_reference(golden, stencil):
    ref = golden("gridprops_ref.npz")
    xmin, xmax, zmin, zmax = ref["box"]
    g = mdz.Grid(int(ref["Nx"]), int(ref["Nz"]), xmin, xmax, zmin, zmax).set_bc_pureshear(1.0)
    mat = mdz.Materials.from_phases([dict(p, rho=1.0, Slim=1e10, n_vp=1.0, gs_ref=1.0, cstv=1, eta0=1.0)
                                     for p in PHASES])
    ctx = mdz.Context(g, 3, len(ref["x"]))
    ctx.set_markers(ref["x"], ref["z"], ref["phase"])
    ctx.set_marker_attr(mdz.M_STRAIN_PL, ref["strain_pl"])
    f = mdz.GridFields(g, 3)
    f["phase_perc_n"] = ref["s%d_pp_c1" % stencil]
    f["phase_perc_s"] = ref["s%d_pp_c0" % stencil]
    ctx.ShearModCompExpGrid(mat, f)
    ctx.CohesionFrictionDilationGrid(mat, stencil, f)
    ctx.close()
    for k in ("mu_n", "mu_s", "bet_n", "bet_s", "C_n", "C_s", "fric_n", "fric_s", "dil_n", "dil_s"):
        want = ref["s%d_%s" % (stencil, k)]
        np.testing.assert_allclose(f[k], want, rtol=1e-12, atol=1e-14, err_msg=k)
