"""Pin the oracle's restatement of the implicit energy step (EnergyDirectSolve,
SOURCE/ThermalRoutines.c:72-551) against the matrix, right-hand side and new
temperature the reference's own function produced (tests/golden/thermal_ref.npz,
its CHOLMOD call replaced by a dense solve in the harness)."""
import numpy as np
import scipy.sparse as sp

import oracle_thermal


def case(ref, q):
    pre = "c%d_" % q
    f = {k[len(pre) + 3:]: ref[k] for k in ref if k.startswith(pre + "in_")}
    bc = {k[len(pre) + 3:]: ref[k] for k in ref if k.startswith(pre + "bc_")}
    dt, shear, adiab, gz = ref[pre + "case"]
    return f, bc, float(dt), int(shear), int(adiab), float(gz)


def grid_spacing(ref):
    xmin, xmax, zmin, zmax = ref["box"]
    Nx, Nz = int(ref["Nx"]), int(ref["Nz"])
    return Nx, Nz, (xmax - xmin) / (Nx - 1), (zmax - zmin) / (Nz - 1)


def test_energy_step_matches_reference(golden):
    ref = golden("thermal_ref.npz")
    Nx, Nz, dx, dz = grid_spacing(ref)
    for q in (0, 1):
        pre = "c%d_" % q
        f, bc, dt, shear, adiab, gz = case(ref, q)
        A, rhs, eqn = oracle_thermal.assemble(Nx, Nz, dx, dz, f, bc, dt, gz, shear, adiab)
        n = rhs.size
        Aref = sp.csr_matrix((ref[pre + "A_data"], ref[pre + "A_indices"], ref[pre + "A_indptr"]), shape=(n, n))
        assert abs(A - Aref).max() <= 1e-14 * abs(Aref).max()
        assert np.abs(rhs - ref[pre + "rhs"]).max() <= 1e-14 * np.abs(ref[pre + "rhs"]).max()
        T, dT = oracle_thermal.energy_step(Nx, Nz, dx, dz, f, bc, dt, gz, shear, adiab)
        assert np.abs(T - ref[pre + "T"]).max() <= 1e-12 * np.abs(ref[pre + "T"]).max()
        assert np.abs(dT - ref[pre + "dT"]).max() <= 1e-11 * np.abs(ref[pre + "dT"]).max()
