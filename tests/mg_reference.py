"""CPU reference of the multigrid hierarchy: sparse matrices of the 31-point
velocity stencils, the staggered prolongation P, and the Galerkin product
R A P with R = P^T (scipy), to check the device hierarchy level by level."""
import numpy as np
import scipy.sparse as sp


def unknown_maps(Nx, Nz):
    """Dense numbering of the velocity unknowns of the free-slip box: Vx (k, l),
    k in 1..Nx-2, l in 1..Nz-1, then Vz (i, j), i in 1..Nx-1, j in 1..Nz-2."""
    iu = -np.ones((Nz + 1, Nx), int)
    iv = -np.ones((Nz, Nx + 1), int)
    nu = (Nx - 2) * (Nz - 1)
    iu[1:Nz, 1:Nx - 1] = np.arange(nu).reshape(Nz - 1, Nx - 2)
    iv[1:Nz - 1, 1:Nx] = nu + np.arange((Nx - 1) * (Nz - 2)).reshape(Nz - 2, Nx - 1)
    return iu, iv, nu + (Nx - 1) * (Nz - 2)


def stencil_matrix(Nx, Nz, su, sv):
    """Sparse velocity block from the stencil planes; returns (A, dropped) where
    dropped is the largest coefficient pointing at a non-unknown."""
    iu, iv, n = unknown_maps(Nx, Nz)
    rows, cols, vals = [], [], []
    dropped = 0.0
    L, K = np.nonzero(iu >= 0)
    ru = iu[L, K]
    cu = K + L * Nx

    def add(rsel, tk, tl, tmap, coef, W, H):
        nonlocal dropped
        inside = (tk >= 0) & (tk < W) & (tl >= 0) & (tl < H)
        tgt = np.full(len(rsel), -1)
        tgt[inside] = tmap[tl[inside], tk[inside]]
        ok = tgt >= 0
        if np.any(~ok):
            dropped = max(dropped, float(np.max(np.abs(coef[~ok]), initial=0.0)))
        rows.append(rsel[ok]); cols.append(tgt[ok]); vals.append(coef[ok])

    for q in range(15):
        add(ru, K + q % 3 - 1, L + q // 3 - 2, iu, su[q, cu], Nx, Nz + 1)
    for q in range(16):
        add(ru, K + q % 4 - 1, L + q // 4 - 2, iv, su[15 + q, cu], Nx + 1, Nz)
    J, I = np.nonzero(iv >= 0)
    rv = iv[J, I]
    cv = I + J * (Nx + 1)
    for q in range(15):
        add(rv, I + q % 5 - 2, J + q // 5 - 1, iv, sv[q, cv], Nx + 1, Nz)
    for q in range(16):
        add(rv, I + q % 4 - 2, J + q // 4 - 1, iu, sv[15 + q, cv], Nx, Nz + 1)
    A = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))
    return A, dropped


def _cc(j, ncc):
    r = j - 1
    R = r >> 1
    J0 = R + 1
    J1 = J0 + 1 if (r & 1) else J0 - 1
    if J1 < 1 or J1 > ncc:
        return J0, 1.0, J0, 0.0
    return J0, 0.75, J1, 0.25


def prolongation(Nxf, Nzf):
    """P from the coarse (cell-doubled) level to the fine level, on the unknowns."""
    Nxc, Nzc = (Nxf - 1) // 2 + 1, (Nzf - 1) // 2 + 1
    iuf, ivf, nf = unknown_maps(Nxf, Nzf)
    iuc, ivc, nc = unknown_maps(Nxc, Nzc)
    rows, cols, vals = [], [], []
    for (l, k) in zip(*np.nonzero(iuf >= 0)):
        J0, w0, J1, w1 = _cc(l, Nzc - 1)
        Ia, Ib = k >> 1, (k + 1) >> 1
        wa, wb = (0.5, 0.5) if k & 1 else (1.0, 0.0)
        for I, J, w in ((Ia, J0, wa * w0), (Ia, J1, wa * w1), (Ib, J0, wb * w0), (Ib, J1, wb * w1)):
            if w and iuc[J, I] >= 0:
                rows.append(iuf[l, k]); cols.append(iuc[J, I]); vals.append(w)
    for (j, i) in zip(*np.nonzero(ivf >= 0)):
        I0, w0, I1, w1 = _cc(i, Nxc - 1)
        Ja, Jb = j >> 1, (j + 1) >> 1
        wa, wb = (0.5, 0.5) if j & 1 else (1.0, 0.0)
        for I, J, w in ((I0, Ja, wa * w0), (I1, Ja, wa * w1), (I0, Jb, wb * w0), (I1, Jb, wb * w1)):
            if w and ivc[J, I] >= 0:
                rows.append(ivf[j, i]); cols.append(ivc[J, I]); vals.append(w)
    return sp.csr_matrix((vals, (rows, cols)), shape=(nf, nc))


def velocity_block(g, K, idx):
    """Velocity block of an assembled operator (oracle numbering) in the dense
    unknown numbering of unknown_maps."""
    iu, iv, n = unknown_maps(g.Nx, g.Nz)
    nu_box = g.Nx * (g.Nz + 1)
    perm = np.full(n, -1)
    L, Kk = np.nonzero(iu >= 0)
    perm[iu[L, Kk]] = idx[Kk + L * g.Nx]
    J, I = np.nonzero(iv >= 0)
    perm[iv[J, I]] = idx[nu_box + I + J * (g.Nx + 1)]
    assert np.all(perm >= 0)
    return K[perm][:, perm]
