"""Output preparation on the GPU: the closest-marker phase maps of
Interp_Phase2VizGrid against the reference's (golden, bit for bit) and the
oracle on a larger seeded state with air cells, and the float cast +
ScaleBack of resident fields against the oracle (bit for bit)."""
import numpy as np
import pytest

import mdz
import mdz_setups
import oracle_output

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("res", [1, 2])
def test_phase_map_vs_reference(golden, res):
    ref = golden("phasemap_ref.npz")
    Nx, Nz = int(ref["Nx"]), int(ref["Nz"])
    xmin, xmax, zmin, zmax = ref["box"]
    g = mdz.Grid(Nx, Nz, xmin, xmax, zmin, zmax).set_bc_pureshear(1.0)
    g.BCp[:] = ref["BCp"]
    ctx = mdz.Context(g, 3, len(ref["x"]))
    ctx.set_markers(ref["x"], ref["z"], ref["phase"])
    compo, X, Z = ctx.Interp_Phase2VizGrid(res)
    ctx.close()
    assert np.array_equal(X, ref["xviz_r%d" % res]) and np.array_equal(Z, ref["zviz_r%d" % res])
    assert np.array_equal(compo, ref["compo_r%d" % res])


def test_phase_map_vs_oracle_large():
    Nx, Nz = 129, 65
    g = mdz.Grid(Nx, Nz, -1.0, 1.0, -0.5, 0.0).set_bc_pureshear(1.0)
    g.BCp.reshape(Nz - 1, Nx - 1)[-5:, 40:70] = 30
    x, z = mdz_setups.seed_markers(g, 4, 4, 0.5, seed=9)
    rng = np.random.default_rng(9)
    ph = rng.integers(0, 4, len(x)).astype(np.int32)
    ph[::53] = -1
    perm = rng.permutation(len(x))              # an arbitrary marker order
    x, z, ph = x[perm], z[perm], ph[perm]
    ctx = mdz.Context(g, 4, len(x))
    ctx.set_markers(x, z, ph)
    for res in (1, 2):
        got, X, Z = ctx.Interp_Phase2VizGrid(res)
        want, Xo, Zo = oracle_output.phase_viz(g.xg[0], g.zg[0], g.dx, g.dz, g.xc[0], g.zc[0], Nx - 1, Nz - 1, g.BCp,
                                               x, z, ph, res)
        assert np.array_equal(X, Xo) and np.array_equal(Z, Zo)
        assert np.array_equal(got, want)
    ctx.close()


def test_output_field_cast_and_scale():
    g = mdz.Grid(33, 17, 0.0, 2.0, 0.0, 1.0).set_bc_pureshear(1.0)
    ctx = mdz.Context(g, 1, 1)
    f = mdz.GridFields(g, 1)
    rng = np.random.default_rng(2)
    for k in ("sxxd", "u", "rho_s"):
        f[k] = rng.normal(size=f[k].size) * 10.0 ** rng.uniform(-8, 8, f[k].size)
    ctx.upload_fields(f)
    for k, scale in (("sxxd", 5e7), ("u", 3.17e-10), ("rho_s", 1.0)):
        got = ctx.output_field(k, scale, f[k].size)
        assert np.array_equal(got, oracle_output.cast_scale(f[k], scale)), k
    with pytest.raises(mdz.MdzError):
        ctx.output_field("no_such_field", 1.0, 4)
    ctx.close()
