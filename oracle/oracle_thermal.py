"""CPU restatement of the implicit energy step of EnergyDirectSolve
(SOURCE/ThermalRoutines.c:72-551, one iteration, Cartesian) for the tests:
the five-point matrix and right-hand side in the reference's equation
numbering, solved with SciPy's sparse LU in place of CHOLMOD.

Test infrastructure only: the parity checker of mdz_EnergyDirectSolve, pinned
to the matrices and solutions the reference itself produced
(tests/golden/thermal_ref.npz).
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

ZEROC = 273.15


def numbering(bc_type):
    """EvalNumEqTemp (ThermalRoutines.c:39-55): consecutive numbers for the
    centroids whose tag is not 30."""
    eqn = np.full(bc_type.size, -1, np.int64)
    act = bc_type != 30
    eqn[act] = np.arange(int(act.sum()))
    return eqn


def assemble(Nx, Nz, dx, dz, f, bc, dt, gz, shear_heating, adiab_heating):
    """Matrix (CSR, equation numbering) and right-hand side b + bbc
    (ThermalRoutines.c:158-187 right-hand side, :190-395 rows)."""
    ncx, ncz, nxvz = Nx - 1, Nz - 1, Nx + 1
    eqn = numbering(bc["type"])
    n = int((eqn >= 0).sum())
    b = np.zeros(n)
    bbc = np.zeros(n)
    rows, cols, vals = [], [], []
    ixx, izz = 1.0 / dx / dx, 1.0 / dz / dz
    T, rho, Cv, kx, kz = f["T"], f["rho_n"], f["Cv"], f["kx"], f["kz"]
    for l in range(ncz):
        for k in range(ncx):
            c2 = k + l * ncx
            if bc["type"][c2] == 30:
                continue
            e = eqn[c2]
            rhoCp = rho[c2] * Cv[c2]
            bb = 1.0 * rhoCp * T[c2] / dt
            bb += 1.0 * f["Qr"][c2]
            if shear_heating == 1:
                bb += f["Wdiss"][c2]
            if adiab_heating == 1:
                c3 = k + l * nxvz
                bb += T[c2] * f["alp"][c2] * 0.5 * (f["v"][c3 + 1] + f["v"][c3 + 1 + nxvz]) * gz * rho[c2]
            elif adiab_heating == 2:
                bb += T[c2] * f["alp"][c2] * (f["p"][c2] - f["p0_n"][c2]) / dt
            b[e] = bb
            c1, c3 = k + (l + 1) * Nx, k + l * nxvz + 1
            AW, AE, AS, AN = kx[c1], kx[c1 + 1], kz[c3], kz[c3 + nxvz]
            act = lambda c: bc["type"][c] != 30
            if l > 0 and act(c2 - ncx):
                rows.append(e); cols.append(eqn[c2 - ncx]); vals.append(-1.0 * AS * izz)
            if k > 0 and act(c2 - 1):
                rows.append(e); cols.append(eqn[c2 - 1]); vals.append(-1.0 * AW * ixx)
            val = 1.0 * rhoCp / dt
            if l > 0 and act(c2 - ncx):
                val += AS * izz
            if k > 0 and act(c2 - 1):
                val += AW * ixx
            if k < ncx - 1 and act(c2 + 1):
                val += AE * ixx
            if l < ncz - 1 and act(c2 + ncx):
                val += AN * izz
            if l == 0 and bc["typS"][k] == 1:
                val += 2.0 * AS * izz
                bbc[e] += 2.0 * AS * izz * bc["valS"][k]
            if l == 0 and bc["typS"][k] == 2:
                bbc[e] += -1.0 / dx * bc["valS"][k]
            if k == 0 and bc["typW"][l] == 1:
                val += 2.0 * AW * ixx
                bbc[e] += 2.0 * AW * ixx * bc["valW"][l]
            if k == ncx - 1 and bc["typE"][l] == 1:
                val += 2.0 * AE * ixx
                bbc[e] += 2.0 * AE * ixx * bc["valE"][l]
            if l == ncz - 1 and bc["typN"][k] == 1:
                val += 2.0 * AN * izz
                bbc[e] += 2.0 * AN * izz * bc["valN"][k]
            rows.append(e); cols.append(e); vals.append(val)
            if k < ncx - 1 and act(c2 + 1):
                rows.append(e); cols.append(eqn[c2 + 1]); vals.append(-1.0 * AE * ixx)
            if l < ncz - 1 and act(c2 + ncx):
                rows.append(e); cols.append(eqn[c2 + ncx]); vals.append(-1.0 * AN * izz)
    A = sp.csr_matrix((vals, (rows, cols)), shape=(n, n))
    return A, b + 1.0 * bbc, eqn


def energy_step(Nx, Nz, dx, dz, f, bc, dt, gz, shear_heating, adiab_heating, scale_T=1.0):
    """New temperature and its increment (ThermalRoutines.c:426-448): the
    solution on the active centroids, 0 C on air cells."""
    A, rhs, eqn = assemble(Nx, Nz, dx, dz, f, bc, dt, gz, shear_heating, adiab_heating)
    x = spla.spsolve(A.tocsc(), rhs)
    T = np.array(f["T"], np.float64)
    dT = np.zeros_like(T)
    act = eqn >= 0
    dT[act] = 1.0 * (x[eqn[act]] - T[act])
    T[act] = T[act] + dT[act]
    T[~act] = ZEROC / scale_T
    return T, dT
