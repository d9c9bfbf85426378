"""CPU oracle of one time step (test infrastructure only): the sequence of
SOURCE/Main_DOODZ.c:459-1320 restricted to the mechanical hot path, driven in
Python over the oracle's C restatements (mdz_oracle*.c).  The linear defect
equation of each non-linear iteration is solved directly (SciPy SuperLU on
the operator assembled by probing the oracle's matrix-free rows, with the
pressure null space fixed by a zero-mean constraint) -- the CHOLMOD-free
stand-in for KillerSolver (SOURCE/Solvers.c:2226).
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla
from scipy.special import erfc

import oracle as orc


def _sizes(g):
    return g.size(-1), g.size(-2), g.size(1)


def assemble(g, f, jacobian, period=5):
    """CSR of the linear Stokes operator on the equation nodes, probed from
    the oracle's rows with a 5-periodic colouring per component."""
    nu, nv, npc = _sizes(g)
    eu = np.flatnonzero(g.BCu == -1)
    ev = np.flatnonzero(g.BCv == -1)
    ep = np.flatnonzero(g.BCp == -1)
    idx = np.full(nu + nv + npc, -1)
    idx[eu] = np.arange(len(eu))
    idx[nu + ev] = len(eu) + np.arange(len(ev))
    idx[nu + nv + ep] = len(eu) + len(ev) + np.arange(len(ep))
    n = len(eu) + len(ev) + len(ep)
    rows, cols, vals = [], [], []
    widths = [(g.Nx, g.Nz + 1), (g.Nx + 1, g.Nz), (g.Nx - 1, g.Nz - 1)]
    offs = [0, nu, nu + nv]
    eqn_sets = [eu, ev, ep]
    for comp in range(3):
        W, H = widths[comp]
        nodes = eqn_sets[comp]
        ki, li = nodes % W, nodes // W
        for cx in range(period):
            for cz in range(period):
                sel = nodes[(ki % period == cx) & (li % period == cz)]
                if len(sel) == 0:
                    continue
                x = np.zeros(nu + nv + npc)
                x[offs[comp] + sel] = 1.0
                yu, yv, yp = orc.stokes_apply(g, f, jacobian, x[:nu], x[nu:nu + nv], x[nu + nv:])
                y = np.concatenate([yu, yv, yp])
                # owner of each response: the probed node of this colour nearest to the row
                r = np.flatnonzero(y)
                r = r[idx[r] >= 0]
                rows.append(idx[r])
                cols.append(idx[_owner(r, comp, offs, widths, period, cx, cz)])
                vals.append(y[r])
    rows, cols, vals = np.concatenate(rows), np.concatenate(cols), np.concatenate(vals)
    return sp.csr_matrix((vals, (rows, cols)), shape=(n, n)), idx, n, len(ep)


def _owner(r, comp, offs, widths, period, cx, cz):
    """Column of each response row r: the unique probed node of colour
    (cx, cz) of component comp within two nodes of the row's position."""
    rc = np.zeros(len(r), int)
    rc[r >= offs[1]] = 1
    rc[r >= offs[2]] = 2
    Wr = np.array([w for w, _ in widths])[rc]
    loc = r - np.array(offs)[rc]
    rk, rl = loc % Wr, loc // Wr
    W2, _ = widths[comp]
    k = rk - ((rk - cx) % period)
    k[rk - k > 2] += period
    l = rl - ((rl - cz) % period)
    l[rl - l > 2] += period
    return offs[comp] + k + l * W2


def solve_defect(g, f, jacobian, F):
    """Solve K x = F on the equation nodes with the pressure mean fixed to
    zero: the bordered system [K e; e^T 0] [x; lam] = [F; 0] (e: ones on the
    pressure equations).  Factorised as M = K + c u u^T (u: one pressure
    unknown; nonsingular where K's null space is the constant pressure) by
    sparse LU without the dense border, then the border and the rank-one term
    resolved from three solves with M (2 x 2 system).  Two steps of iterative
    refinement with the same factors follow: the pressure of a strong
    viscosity contrast is conditioned far worse than the residual (a 1e3
    inclusion at 101 x 101 keeps ~1e-7 relative pressure error after the
    direct solve alone, at a 2e-14 relative residual; ~1e-12 after them)."""
    K, idx, n, n_p = assemble(g, f, jacobian)
    b = F[idx >= 0][np.argsort(idx[idx >= 0])]
    b = b.copy()
    b[n - n_p:] -= b[n - n_p:].mean()
    e = np.zeros(n)
    e[n - n_p:] = 1.0
    r = n - 1
    c = np.abs(K.diagonal()[:n - n_p]).mean()
    u = np.zeros(n)
    u[r] = 1.0
    M = (K + sp.csr_matrix(([c], ([r], [r])), shape=(n, n))).tocsc()
    lu = spla.splu(M, permc_spec="COLAMD")
    yu, ye = lu.solve(u), lu.solve(e)
    A2 = np.array([[1.0 - c * yu[r], ye[r]], [c * (e @ yu), -(e @ ye)]])

    def solve(rhs):
        yb = lu.solve(rhs)
        s_, lam = np.linalg.solve(A2, np.array([yb[r], -(e @ yb)]))
        return yb + c * s_ * yu - lam * ye
    x = solve(b)
    for _ in range(2):
        res = b - K @ x
        res[n - n_p:] -= res[n - n_p:].mean()
        x = x + solve(res)
    out = np.zeros(len(F))
    out[idx >= 0] = x[idx[idx >= 0]]
    return out


def grid_props(g, mat, nph, pp, strain, cmul, tags, law):
    """ShearModCompExpGrid (harmonic mu, bet) and CohesionFrictionDilationGrid
    (SOURCE/RheologyDensity.c:1422-1791) from phase fractions."""
    n = pp.shape[1]
    imu, ibet, rho, d0 = np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(n)
    fs, ds, Cs = np.zeros(n), np.zeros(n), np.zeros(n)
    for p in range(nph):
        w = pp[p]
        imu += w / mat.mu[p]
        ibet += w / mat.bet[p]
        rho += w * mat.rho[p]
        d0 += w * mat.gs_ref[p]
        fric, dil, C = mat.phi[p] + 0 * strain, mat.psi[p] + 0 * strain, mat.C[p] + 0 * strain
        dst = mat.pls_end[p] - mat.pls_start[p]
        if law == 0:
            mu = 0.5 * (mat.pls_end[p] + mat.pls_start[p])
            for flag, a0, a1, name in ((mat.phi_soft[p], mat.phi[p], mat.phi_end[p], "f"),
                                       (mat.psi_soft[p], mat.psi[p], mat.psi_end[p], "d"),
                                       (mat.coh_soft[p], mat.C[p], mat.C_end[p], "c")):
                if flag == 1:
                    dd = a0 - a1
                    v = a0 - dd / 2.0 * erfc(-(strain - mu) / dst) - a1
                    v0 = a0 - dd / 2.0 * erfc(-(0.0 - mu) / dst) - a1
                    v = v * dd / v0 + a1
                    if name == "f":
                        fric = v
                    elif name == "d":
                        dil = v
                    else:
                        C = v
        else:
            for flag, a0, a1, name in ((mat.phi_soft[p], mat.phi[p], mat.phi_end[p], "f"),
                                       (mat.psi_soft[p], mat.psi[p], mat.psi_end[p], "d"),
                                       (mat.coh_soft[p], mat.C[p], mat.C_end[p], "c")):
                if flag == 1:
                    v = np.where(strain >= mat.pls_end[p], a1,
                                 np.where(strain >= mat.pls_start[p], a0 + (a1 - a0) / dst * strain, a0))
                    if name == "f":
                        fric = v
                    elif name == "d":
                        dil = v
                    else:
                        C = v
        fs += w * fric
        ds += w * dil
        Cs += w * C
    return 1.0 / imu, 1.0 / ibet, rho, d0, Cs * cmul, fs, ds


def project(g, mat, model, markers):
    """The projections of a time step (P2Mastah calls of Main_DOODZ.c:501-594)
    and the grid properties (ShearModCompExpGrid, CohesionFrictionDilationGrid):
    returns (GridFields, Oracle holding the markers)."""
    import mdz
    nph = mat.n_phases
    f = mdz.GridFields(g, nph)
    o = orc.Oracle(g, nph)
    o.set_markers(markers["x"], markers["z"], markers["phase"])
    st = model.itp_stencil
    # 1. projections
    f["phase_perc_n"] = o.P2Mastah(np.zeros(nph), None, g.tags(1), 0, 0, 1, 1, st)
    f["phase_perc_s"] = o.P2Mastah(np.zeros(nph), None, g.tags(0), 0, 0, 1, 0, st)
    for name, key in (("sxxd0", "sxxd"), ("szzd0", "szzd"), ("T", "T"), ("strain_n", "strain_pl"), ("p0_n", "P")):
        f[name] = o.P2Mastah(markers[key], f[name], g.tags(1), 1, 0, 0, 1, st)
    cmul_n = o.P2Mastah(markers["cmul"], np.zeros(g.size(1)), g.tags(1), 1, 0, 0, 1, st)
    f["sxz0"] = o.P2Mastah(markers["sxz"], f["sxz0"], g.tags(0), 1, 0, 0, 0, st)
    f["strain_s"] = o.P2Mastah(markers["strain_pl"], f["strain_s"], g.tags(0), 1, 0, 0, 0, st)
    cmul_s = o.P2Mastah(markers["cmul"], np.zeros(g.size(0)), g.tags(0), 1, 0, 0, 0, st)
    L = orc.lib()
    import ctypes as C
    desc = g.desc()
    s = f.struct()
    L.orc_c2v(C.byref(desc), s.sxxd0, s.sxxd0_s)
    L.orc_c2v(C.byref(desc), s.szzd0, s.szzd0_s)
    L.orc_v2c(C.byref(desc), s.sxz0_n, s.sxz0)
    pn = f["phase_perc_n"].reshape(nph, -1)
    ps = f["phase_perc_s"].reshape(nph, -1)
    (f["mu_n"], f["bet_n"], f["rho_n"], f["d0_n"], f["C_n"], f["fric_n"], f["dil_n"]) = grid_props(
        g, mat, nph, pn, f["strain_n"], cmul_n, g.BCp, model.softening)
    (f["mu_s"], f["bet_s"], f["rho_s"], _, f["C_s"], f["fric_s"], f["dil_s"]) = grid_props(
        g, mat, nph, ps, f["strain_s"], cmul_s, g.BCg, model.softening)
    return f, o


def first_defect(g, mat, model, markers, u, v, p, jacobian):
    """State of a time step's first non-linear iteration: projections, BCs,
    UpdateNonLinearity and the residual F (grid layout u | v | p), with the
    Picard (jacobian 0) or Newton (jacobian 1) D-tensor in the fields."""
    f, _ = project(g, mat, model, markers)
    u = np.array(u, np.float64)
    v = np.array(v, np.float64)
    u[g.BCu == 0] = g.BCu_val[g.BCu == 0]
    v[g.BCv == 0] = g.BCv_val[g.BCv == 0]
    _mirror(g, u, v)
    f["u"], f["v"], f["p"] = u, v, np.array(p, np.float64)
    prm = model.rheo
    orc.strain_rates(g, f)
    orc.viscosity_grid(g, mat, prm, f)
    orc.rhs(g, prm, model.gx, model.gz, f)
    orc.rheo_operators(g, prm, f, 0)
    orc.residual(g, f)
    if jacobian:
        orc.rheo_operators(g, prm, f, 1)
    return f, np.concatenate([f["ru"], f["rv"], f["rp"]])


def pure_shear_ale(g, u, v, dt):
    """PureShearALE (SOURCE/AdvectionRoutines.c:634-734, no free surface):
    each wall moves by dt times the mean velocity of its Dirichlet nodes,
    summed in the reference's loop order (west / east: Vx rows 0..Nz-1 of the
    first / last column, tag 0; south / north: Vz columns 0..Nx-1 of the first
    / last row, tag 0, or 0 and 30 on the north), then the grid lines are
    regenerated over the new box (g.regrid, SetGridCoordinates).  g changes in
    place; returns the new (xmin, xmax, zmin, zmax)."""
    Nx, Nz = g.Nx, g.Nz
    uu, bu = np.asarray(u).reshape(Nz + 1, Nx), g.BCu.reshape(Nz + 1, Nx)
    vv, bv = np.asarray(v).reshape(Nz, Nx + 1), g.BCv.reshape(Nz, Nx + 1)

    def mean(vals, take):
        s, c = 0.0, 0
        for x, t in zip(vals.tolist(), take.tolist()):
            if t:
                s += x
                c += 1
        return s / c if c > 0 else s
    VxW = mean(uu[:Nz, 0], bu[:Nz, 0] == 0)
    VxE = mean(uu[:Nz, Nx - 1], bu[:Nz, Nx - 1] == 0)
    VzS = mean(vv[0, :Nx], bv[0, :Nx] == 0)
    VzN = mean(vv[Nz - 1, :Nx], (bv[Nz - 1, :Nx] == 0) | (bv[Nz - 1, :Nx] == 30))
    g.regrid(g.xmin + VxW * dt, g.xmax + VxE * dt, g.zmin + VzS * dt, g.zmax + VzN * dt)
    return g.xmin, g.xmax, g.zmin, g.zmax


def time_step(g, mat, model, markers, u, v, p, fields_out=None):
    """markers: dict with x, z, phase, sxxd, szzd, sxz, strain_pl, strain, T, cmul (updated in place).
    Returns (u, v, p, report dict)."""
    f, o = project(g, mat, model, markers)
    u = np.array(u, np.float64)
    v = np.array(v, np.float64)
    p = np.array(p, np.float64)
    u[g.BCu == 0] = g.BCu_val[g.BCu == 0]
    v[g.BCv == 0] = g.BCv_val[g.BCv == 0]
    _mirror(g, u, v)
    prm = model.rheo

    def update_nonlinearity():
        f["u"], f["v"], f["p"] = u, v, p
        orc.strain_rates(g, f)
        orc.viscosity_grid(g, mat, prm, f)
        orc.rhs(g, prm, model.gx, model.gz, f)
        orc.rheo_operators(g, prm, f, 0)

    def res_norms():
        return orc.residual(g, f)

    rep = dict(nonlinear_its=0, converged=0, stagnated=0)
    r0 = None
    nit = 0
    use_newton = bool(model.newton) and not getattr(model, "picard2newton", 0)
    for nit in range(model.nit_max + 1):
        update_nonlinearity()
        r = res_norms()
        if r0 is None:
            r0 = r.copy()
        if _converged(model, r, r0) and (nit > 0 or np.all(r < model.abs_tol)):
            rep["converged"] = 1
            break
        if nit == model.nit_max:
            break
        # Picard -> Newton switch (Main_DOODZ.c:735-743)
        if model.newton and not use_newton and nit > 0 and (
                r[0] < model.pic2newt_cond * r0[0] or r[1] < model.pic2newt_cond * r0[1] or nit >= model.nit_pic_max):
            use_newton = True
        F = np.concatenate([f["ru"], f["rv"], f["rp"]])
        if use_newton:
            orc.rheo_operators(g, prm, f, 1)
        dx = solve_defect(g, f, use_newton, F)
        u0, v0, p0 = u.copy(), v.copy(), p.copy()
        alpha = -1.0
        if model.line_search:
            ntry = 6
            amin, amax = (-1.0, -model.line_search_min) if use_newton else (-2.5, -0.0)
            da = abs(amax - amin) / (ntry - 1)
            a = amax
            trials = []
            for kk in range(ntry):
                if kk > 0:
                    a -= da
                u, v, p = _trial(g, u0, v0, p0, dx, a)
                update_nonlinearity()
                t = res_norms()
                trials.append((a, t))
            f0 = np.sqrt(np.sum(r ** 2))
            fx = [np.sqrt(np.sum(t ** 2)) for _, t in trials]
            ib = int(np.argmin(fx))
            ok = fx[ib] < f0
            if not ok:
                fxz = [np.hypot(t[0], t[1]) for _, t in trials]
                ixz = int(np.argmin(fxz))
                ix = int(np.argmin([t[0] for _, t in trials]))
                iz = int(np.argmin([t[1] for _, t in trials]))
                if trials[ixz][1][0] < r[0] and trials[ixz][1][1] < r[1]:
                    ok, ib = True, ixz
                elif trials[ix][1][0] < r[0]:
                    ok, ib = True, ix
                elif trials[iz][1][1] < r[1]:
                    ok, ib = True, iz
            if not ok or abs(trials[ib][0]) < 1e-13:
                rep["stagnated"] = 1
                alpha = 0.0
            else:
                alpha = trials[ib][0]
        u, v, p = _trial(g, u0, v0, p0, dx, alpha)
        if rep["stagnated"]:
            nit += 1
            break
    rep["nonlinear_its"] = nit
    rep["res0"], rep["res"] = r0, r
    update_nonlinearity()
    p = f["p_corr"].copy()
    if model.advect:
        dt = prm.dt
        update_particle_stress(g, o, f, markers)
        update_particle_pressure(g, o, f["p0_n"], p, markers)
        dstr = dt * (f["eII_pl"] + f["eII_pwl"] + f["eII_lin"] + f["eII_el"] + f["eII_cst"])
        dstr_pl = dt * f["eII_pl"]
        if getattr(model, "ispureshear_ale", 0) == 1:   # before the advection (Main_DOODZ.c:1107-1109)
            pure_shear_ale(g, u, v, dt)
            o._desc = g.desc()
        markers["vx"], markers["vz"] = o.RogerGuntherII(u, v, dt)
        markers["x"], markers["z"], markers["phase"] = o.x, o.z, o.phase
        # AccumulatedStrainII after the advection (Main_DOODZ.c:1134-1140)
        e, ep = _accumulated_strain(g, markers, dstr, dstr_pl)
        markers["strain"] += e
        markers["strain_pl"] += ep
        rep["markers_added"] = 0
        if getattr(model, "reseed", 0):   # CountPartCell(RESEED = 1) after the advection
            cap = len(markers["x"]) + 4 * (g.Nx - 1) * (g.Nz - 1)
            new, rep["markers_added"] = orc.reseed(g, markers, cap, model.min_part_cell, model.direct_neighbour,
                                                   f["T"], f["sxxd"], f["szzd"], f["sxz"], p)
            markers.update(new)
    if fields_out is not None:
        fields_out.update({k: f[k].copy() for k in f.a})
    return u, v, p, rep


def _converged(model, r, r0):
    rmax = max(r0)
    for q in range(3):
        ref = r0[q] if r0[q] > 1e-6 * rmax else rmax
        if not (r[q] < model.abs_tol or (ref > 0 and r[q] / ref < model.rel_tol)):
            return False
    return True


def _mirror(g, u, v):
    Nx, Nz = g.Nx, g.Nz
    U = u.reshape(Nz + 1, Nx)
    V = v.reshape(Nz, Nx + 1)
    bu = g.BCu.reshape(Nz + 1, Nx)
    bv = g.BCv.reshape(Nz, Nx + 1)
    U[0, bu[0] == 13] = U[1, bu[0] == 13]
    U[Nz, bu[Nz] == 13] = U[Nz - 1, bu[Nz] == 13]
    V[bv[:, 0] == 13, 0] = V[bv[:, 0] == 13, 1]
    V[bv[:, Nx] == 13, Nx] = V[bv[:, Nx] == 13, Nx - 1]


def _trial(g, u0, v0, p0, dx, a):
    nu, nv, npc = _sizes(g)
    u = np.where(g.BCu == -1, u0 + a * dx[:nu], u0)
    v = np.where(g.BCv == -1, v0 + a * dx[nu:nu + nv], v0)
    p = np.where(g.BCp == -1, p0 + a * dx[nu + nv:], p0)
    _mirror(g, u, v)
    return u, v, p


def update_particle_stress(g, o, f, markers):
    """UpdateParticleStress without rotation and subgrid diffusion
    (SOURCE/RheologyParticles.c:1124-1447): the grid stress increments
    (centroids sxxd - sxxd0, szzd - szzd0; vertices sxz - sxz0) interpolated to
    the active markers (Interp_Grid2P_centroids2 / Interp_Grid2P) and added.
    o: an Oracle holding the markers' positions and phases."""
    act_n = (g.BCp != 30) & (g.BCp != 31)
    dsxx = np.where(act_n, f["sxxd"] - f["sxxd0"], 0.0)
    dszz = np.where(act_n, f["szzd"] - f["szzd0"], 0.0)
    dsxz = np.where(g.BCg != 30, f["sxz"] - f["sxz0"], 0.0)
    act = markers["phase"] != -1
    markers["sxxd"] += np.where(act, o.Interp_Grid2P(dsxx, 1), 0.0)
    markers["szzd"] += np.where(act, o.Interp_Grid2P(dszz, 1), 0.0)
    markers["sxz"] += np.where(act, o.Interp_Grid2P(dsxz, 0), 0.0)


def update_particle_pressure(g, o, p0_n, p, markers):
    """UpdateParticlePressure (SOURCE/RheologyParticles.c:1004-1123) with
    Plith_trick = 0 and no subgrid diffusion: dp = p_in - p0_n where the
    centroid tag is not 30, interpolated to the active markers
    (Interp_Grid2P_centroids2) and added to their pressure.  o: an Oracle
    holding the markers' positions and phases."""
    dp = np.where(g.BCp != 30, p - p0_n, 0.0)
    markers["P"] += np.where(markers["phase"] != -1, o.Interp_Grid2P(dp, 1), 0.0)


def _accumulated_strain(g, m, dstr, dstr_pl):
    """AccumulatedStrainII (SOURCE/RheologyParticles.c:191-537): bilinear on the
    centroid lines with a clamped lower-left cell and signed offsets."""
    ncx, ncz = g.ncx, g.ncz
    x, z = m["x"], m["z"]
    jp = np.clip(np.ceil((x - g.xc[0]) / g.dx).astype(int) - 1, 0, ncx - 2)
    ip = np.clip(np.ceil((z - g.zc[0]) / g.dz).astype(int) - 1, 0, ncz - 2)
    dxm = x - g.xc[jp]
    dzm = z - g.zc[ip]
    SW = jp + ip * ncx
    idx = [SW, SW + 1, SW + ncx, SW + ncx + 1]
    w = [(1 - dxm / g.dx) * (1 - dzm / g.dz), (dxm / g.dx) * (1 - dzm / g.dz), (1 - dxm / g.dx) * (dzm / g.dz),
         (dxm / g.dx) * (dzm / g.dz)]
    e = sum(wi * dstr[ii] for wi, ii in zip(w, idx))
    ep = sum(wi * dstr_pl[ii] for wi, ii in zip(w, idx))
    s = sum(w)
    e = np.where(s > 1e-13, e / s, e)
    ep = np.where(s > 1e-13, ep / s, ep)
    act = m["phase"] != -1
    return np.where(act, e, 0.0), np.where(act, ep, 0.0)
