"""The implicit energy step on the GPU (mdz_EnergyDirectSolve: matrix-free
rows of EnergyDirectSolve, Jacobi-preconditioned conjugate gradients in FP64)
against the reference's own solve (golden fixture) and against the oracle on
a larger seeded grid with air cells."""
import numpy as np
import pytest

import mdz
import oracle_thermal
from test_oracle_thermal import case, grid_spacing

pytestmark = pytest.mark.gpu


def _fields(g, f):
    fl = mdz.GridFields(g, 1)
    for k, v in f.items():
        fl[k] = v
    return fl


def test_energy_step_vs_reference(golden):
    ref = golden("thermal_ref.npz")
    Nx, Nz, dx, dz = grid_spacing(ref)
    xmin, xmax, zmin, zmax = ref["box"]
    for q in (0, 1):
        pre = "c%d_" % q
        f, bc, dt, shear, adiab, gz = case(ref, q)
        g = mdz.Grid(Nx, Nz, xmin, xmax, zmin, zmax).set_bc_pureshear(1.0)
        fl = _fields(g, f)
        ctx = mdz.Context(g, 1, 1)
        its, rel = ctx.EnergyDirectSolve(fl, bc, dt, gz, shear, adiab)
        assert 0 < its < 200 and rel <= 1e-13
        assert np.abs(fl["T"] - ref[pre + "T"]).max() <= 1e-11 * np.abs(ref[pre + "T"]).max()
        assert np.abs(fl["dT"] - ref[pre + "dT"]).max() <= 1e-9 * np.abs(ref[pre + "dT"]).max()
        ctx.close()


def test_energy_step_vs_oracle_large_with_air():
    from golden.make_golden import thermal_inputs
    Nx, Nz = 257, 129
    g = mdz.Grid(Nx, Nz, 0.0, 2.0, 0.0, 1.0).set_bc_pureshear(1.0)
    rng = np.random.default_rng(7)
    f, bc = thermal_inputs(rng, Nx - 1, Nz - 1, Nx, Nz)
    bc["type"].reshape(Nz - 1, Nx - 1)[-3:, 100:140] = 30   # a patch of air under the north wall
    ctx = mdz.Context(g, 1, 1)
    fl = _fields(g, f)
    its, rel = ctx.EnergyDirectSolve(fl, bc, 0.02, -1.0, 1, 1)
    T, dT = oracle_thermal.energy_step(Nx, Nz, g.dx, g.dz, f, bc, 0.02, -1.0, 1, 1)
    assert np.abs(fl["T"] - T).max() <= 1e-10 * np.abs(T).max()
    assert np.array_equal(fl["T"][bc["type"] == 30], T[bc["type"] == 30])
    assert np.abs(fl["dT"] - dT).max() <= 1e-8 * np.abs(dT).max()
    # the same solve again: identical bits and iterations (fixed-order sums)
    fl2 = _fields(g, f)
    its2, rel2 = ctx.EnergyDirectSolve(fl2, bc, 0.02, -1.0, 1, 1)
    assert its2 == its and rel2 == rel and np.array_equal(fl2["T"], fl["T"])
    ctx.close()


def test_energy_step_rejects_free_surface_tags():
    from golden.make_golden import thermal_inputs
    g = mdz.Grid(9, 9, 0.0, 1.0, 0.0, 1.0).set_bc_pureshear(1.0)
    f, bc = thermal_inputs(np.random.default_rng(1), 8, 8, 9, 9)
    bc["type"][5] = 1
    ctx = mdz.Context(g, 1, 1)
    with pytest.raises(mdz.MdzError) as e:
        ctx.EnergyDirectSolve(_fields(g, f), bc, 0.1)
    assert e.value.status == 4
    ctx.close()
