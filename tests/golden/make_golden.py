"""Generate the golden fixtures in tests/golden/ from the REFERENCE's own C
functions (MDOODZ 6.0 compiled in place by `make -C oracle ref`, driven through
oracle/ref_harness.c).  Run in a container that has the reference sources:

    python tests/golden/make_golden.py

Each fixture is a small .npz holding the inputs and the reference outputs.
The GPU tests and the oracle self-tests read these files; nothing at test time
needs the reference itself.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "oracle"), os.path.join(ROOT, "mdoodz6.0_gb300")]

import mdz  # noqa: E402  (grid / tag helpers only; no GPU use)
import mdz_setups  # noqa: E402
from refharness import RefMDOODZ  # noqa: E402

# small, non-square grid; two phases; 4x4 jittered markers per cell
NX, NZ, XMIN, XMAX, ZMIN, ZMAX = 21, 17, -0.5, 0.5, -0.4, 0.4


def _grid():
    return mdz.Grid(NX, NZ, XMIN, XMAX, ZMIN, ZMAX).set_bc_pureshear(1.0)


def _markers(g, seed=7):
    x, z = mdz_setups.seed_markers(g, 4, 4, 0.5, seed)
    ph = mdz_setups.inclusion_phase(x, z, 0.05, -0.02, 0.18)
    # a few inactive markers, and a third phase stripe
    ph[(z > 0.25) & (x < -0.2)] = 2
    ph[::97] = -1
    return x, z, ph


def make_markers_fixture():
    g = _grid()
    r = RefMDOODZ(NX, NZ, XMIN, XMAX, ZMIN, ZMAX, 3)
    r.set_bc_pureshear(1.0)
    # the harness grid must equal ours bit for bit
    for name, ours in [("xg_coord", g.xg), ("zg_coord", g.zg), ("xc_coord", g.xc), ("zc_coord", g.zc),
                       ("xvz_coord", g.xvz), ("zvx_coord", g.zvx)]:
        assert np.array_equal(r.field(name), ours), name
    assert np.array_equal(r.tags("BCu"), g.BCu) and np.array_equal(r.tags("BCv"), g.BCv)
    assert np.array_equal(r.field("BCu_val"), g.BCu_val) and np.array_equal(r.field("BCv_val"), g.BCv_val)
    x, z, ph = _markers(g)
    r.set_markers(x, z, ph)
    rng = np.random.default_rng(3)
    per_phase = np.array([1.0, 1e3, 7.5])
    per_marker = np.exp(rng.normal(0.0, 1.0, len(x)))
    out = dict(Nx=NX, Nz=NZ, box=np.array([XMIN, XMAX, ZMIN, ZMAX]), x=x, z=z, phase=ph, per_phase=per_phase,
               per_marker=per_marker)
    for centroid in (1, 0, -1, -2):
        for stencil in (1, 9):
            for avg in (0, 1, 2):
                for flag in (0, 1):
                    vals = per_phase if flag == 0 else per_marker
                    init = np.full(g.size(centroid), -7.0)   # untouched nodes keep this
                    out["p2g_c%d_s%d_a%d_f%d" % (centroid, stencil, avg, flag)] = r.p2g(vals, flag, avg, 0, centroid,
                                                                                       stencil, init)
    for centroid in (1, 0):
        for stencil in (1, 9):
            r.p2g(per_phase, 0, 0, 1, centroid, stencil)
            out["pp_c%d_s%d" % (centroid, stencil)] = np.array([r.phase_perc(centroid, p).copy() for p in range(3)])
    # counts (CountPartCell_Old): totals, and per-phase counts recovered from
    # the phase fractions it stores (fraction x total is an exact small integer)
    r.count_old()
    cc, cv = r.counts(1).copy(), r.counts(0).copy()
    out["count_cell"], out["count_vert"] = cc, cv
    out["pcount_cell"] = np.rint(np.array([r.phase_perc(1, p) * cc for p in range(3)])).astype(np.int32)
    out["pcount_vert"] = np.rint(np.array([r.phase_perc(0, p) * cv for p in range(3)])).astype(np.int32)
    # grid -> marker
    fv = np.sin(3 * g.xg)[None, :] * np.cos(2 * g.zg)[:, None]
    fc = np.cos(2 * g.xc)[None, :] * (1 + g.zc)[:, None] ** 2
    out["g2p_vertex_field"], out["g2p_centroid_field"] = fv.ravel(), fc.ravel()
    out["g2p_vertex"] = r.g2p(fv.ravel(), 0)
    out["g2p_centroid"] = r.g2p(fc.ravel(), 1)
    # RK4 in a pure-shear + vortex velocity (some markers leave the box)
    U = (-g.xg[None, :] * 1.0 + 0.3 * np.sin(np.pi * g.zvx[:, None])).ravel()
    V = (g.zg[:, None] * 1.0 + 0.2 * np.cos(np.pi * g.xvz[None, :])).ravel()
    r.field("u_in")[:] = U
    r.field("v_in")[:] = V
    r.set_param("dt", 0.07)
    r.rk4()
    out["rk4_u"], out["rk4_v"], out["rk4_dt"] = U, V, 0.07
    out["rk4_x"], out["rk4_z"] = r.marker_field("x").copy(), r.marker_field("z").copy()
    out["rk4_vx"], out["rk4_vz"] = r.marker_field("Vx").copy(), r.marker_field("Vz").copy()
    out["rk4_phase"] = r.marker_phase().copy()
    np.savez_compressed(os.path.join(HERE, "markers_ref.npz"), **out)
    print("markers_ref.npz:", len(out), "arrays")




# ---- local rheology -------------------------------------------------------------
RHEO_PHASES = [
    # constant viscosity + elasticity + Drucker-Prager
    dict(cstv=1, eta0=1.0, rho=1.0, Slim=1e10, eta_vp=0.0, n_vp=1.0, gs_ref=1.0),
    # dislocation creep + elasticity + plasticity with a viscoplastic regularisation
    dict(pwlv=1, npwl=3.0, Apwl=2.0e-3, Qpwl=1.2e4, Vpwl=0.05, mpwl=0.0, rpwl=0.0, fpwl=1.0, apwl=0.0, Fpwl=1.0,
         pref_pwl=1.0, rho=1.1, Slim=1e10, eta_vp=0.02, n_vp=1.0, gs_ref=1.0),
    # diffusion + dislocation creep, von Mises cap
    dict(linv=1, nlin=1.0, Alin=0.3, Qlin=5.0e3, Vlin=0.0, mlin=0.0, rlin=0.0, flin=1.0, alin=0.0, Flin=1.0,
         pwlv=1, npwl=3.5, Apwl=1.0e-3, Qpwl=1.5e4, Vpwl=0.0, mpwl=0.0, rpwl=0.0, fpwl=1.0, apwl=0.0, Fpwl=1.0,
         pref_pwl=1.0, rho=0.9, Slim=1.3, eta_vp=0.0, n_vp=1.0, gs_ref=1.0),
]
RHEO_MODEL = dict(dt=0.5, iselastic=1, step=1, eta_avg=0, mineta=1e-3, maxeta=1e6)
RHEO_R = 8.314
# the other mechanisms of Viscosity(): Peierls creep, grain-boundary sliding
# and the tension cut-off (tension pressure -25 MPa / scale_S = -0.5 here, so
# that the fixture's pressures, -0.2 .. 1.4, straddle it)
RHEO_PHASES_MECH = [
    # constant viscosity + Peierls creep + elasticity + Drucker-Prager with the tension cut-off
    dict(cstv=1, eta0=3.0, expv=1, Qexp=5.4e4, Sexp=10.0, Eexp=1.0, Gexp=0.1, nexp=2.0, is_tensile=1,
         rho=1.0, Slim=1e10, eta_vp=0.02, n_vp=1.0, gs_ref=1.0),
    # dislocation creep + grain-boundary sliding + tension cut-off
    dict(pwlv=1, npwl=3.0, Apwl=2.0e-3, Qpwl=1.2e4, Vpwl=0.05, mpwl=0.0, rpwl=0.0, fpwl=1.0, apwl=0.0, Fpwl=1.0,
         pref_pwl=1.0, gbsv=1, ngbs=2.0, Agbs=1.0e-2, Qgbs=1.0e4, Vgbs=0.02, mgbs=0.0, rgbs=0.0, fgbs=1.0, agbs=0.0,
         Fgbs=1.0, is_tensile=1, rho=1.1, Slim=1e10, eta_vp=0.02, n_vp=1.0, gs_ref=1.0),
    # diffusion creep + Peierls + grain-boundary sliding, von Mises cap
    dict(linv=1, nlin=1.0, Alin=0.3, Qlin=5.0e3, Vlin=0.0, mlin=0.0, rlin=0.0, flin=1.0, alin=0.0, Flin=1.0,
         expv=1, Qexp=4.0e4, Sexp=5.0, Eexp=2.0, Gexp=0.2, nexp=1.5,
         gbsv=1, ngbs=2.5, Agbs=5.0e-3, Qgbs=8.0e3, Vgbs=0.0, mgbs=0.0, rgbs=0.0, fgbs=1.0, agbs=0.0, Fgbs=1.0,
         rho=0.9, Slim=1.3, eta_vp=0.0, n_vp=1.0, gs_ref=1.0),
]
RHEO_MODEL_MECH = dict(RHEO_MODEL, scale_S=5e7)


def rheology_inputs(g, rng):
    """Smooth random grid fields for the rheology fixtures."""
    Nx, Nz = g.Nx, g.Nz
    X, Z = np.meshgrid(g.xg, g.zvx)
    u = (-X + 0.3 * np.sin(2.3 * Z + 0.4) * np.cos(1.7 * X)).ravel()
    X, Z = np.meshgrid(g.xvz, g.zg)
    v = (Z + 0.25 * np.cos(1.9 * X) * np.sin(2.1 * Z + 0.2)).ravel()
    Xc, Zc = np.meshgrid(g.xc, g.zc)
    Xv, Zv = np.meshgrid(g.xg, g.zg)
    f = dict(
        u=u, v=v,
        p=(0.6 + 0.8 * np.sin(3 * Xc) * np.cos(2 * Zc)).ravel(),
        T=(900.0 + 400.0 * Zc + 100 * Xc).ravel(),
        mu_n=np.full(Xc.size, 1.0), mu_s=np.full(Xv.size, 1.0),
        C_n=(0.3 + 0.3 * rng.random(Xc.size)), C_s=(0.3 + 0.3 * rng.random(Xv.size)),
        fric_n=np.full(Xc.size, np.pi / 6), fric_s=np.full(Xv.size, np.pi / 6),
        dil_n=np.zeros(Xc.size), dil_s=np.zeros(Xv.size),
        bet_n=np.full(Xc.size, 1e-2), bet_s=np.full(Xv.size, 1e-2),
        sxxd0=0.3 * rng.standard_normal(Xc.size), szzd0=0.3 * rng.standard_normal(Xc.size),
        sxz0=0.3 * rng.standard_normal(Xv.size),
        d0_n=np.full(Xc.size, 1.0), phi0_n=np.zeros(Xc.size),
        rho_n=np.full(Xc.size, 1.0), rho_s=np.full(Xv.size, 1.0),
    )
    return f


def set_neumann_walls(tu, vu, tv, vv, seed=21):
    """Neumann (tag 2) west and east Vx lines and south Vz line with seeded
    tractions; the north wall stays Dirichlet (arrays in grid layout, changed
    in place)."""
    rng = np.random.default_rng(seed)
    Nx, Nz = NX, NZ
    tu, vu = tu.reshape(Nz + 1, Nx), vu.reshape(Nz + 1, Nx)
    tv, vv = tv.reshape(Nz, Nx + 1), vv.reshape(Nz, Nx + 1)
    for k in (0, Nx - 1):
        tu[1:Nz, k] = 2
        vu[1:Nz, k] = 0.3 * rng.standard_normal(Nz - 1)
    tv[0, 1:Nx] = 2
    vv[0, 1:Nx] = 0.2 * rng.standard_normal(Nx - 1)


def make_phasemap_fixture():
    """Interp_Phase2VizGrid as WriteOutputHDF5 calls it (visualisation grids of
    1x and 2x the grid resolution) on the markers of the markers fixture, with
    a patch of air centroids (BCp 30) whose markers must not mark the map."""
    g = _grid()
    r = RefMDOODZ(NX, NZ, XMIN, XMAX, ZMIN, ZMAX, 3)
    r.set_bc_pureshear(1.0)
    bcp = r.tags("BCp").reshape(NZ - 1, NX - 1)
    bcp[-2:, 3:9] = 30
    x, z, ph = _markers(g, seed=5)
    r.set_markers(x, z, ph)
    out = dict(Nx=NX, Nz=NZ, box=np.array([XMIN, XMAX, ZMIN, ZMAX]), x=x, z=z, phase=ph,
               BCp=r.tags("BCp").copy())
    for res in (1, 2):
        compo, xv, zv = r.phase_viz(res)
        out["compo_r%d" % res], out["xviz_r%d" % res], out["zviz_r%d" % res] = compo, xv, zv
    np.savez_compressed(os.path.join(HERE, "phasemap_ref.npz"), **out)


# scales of the breakpoint fixture (a lithosphere-like set: km, cm/yr, 10 MPa)
BRK_SCALE = {"L": 1.0e4, "V": 3.0e-10, "S": 2.0e7, "T": 700.0, "t": 1.0e4 / 3.0e-10, "E": 3.0e-14,
             "rho": 3300.0, "eta": 1.0e21, "rhoE": 6.6e10}
BRK_MARKER = ("P", "Vx", "Vz", "sxxd", "szzd", "sxz", "strain", "strain_pl", "T")


def make_breakpoint_fixture():
    """The reference's own breakpoint file: MakeBreakpointParticles
    (iselastic = 1, no free surface) of a seeded state given in scaled units,
    with non-trivial scales, and what LoadBreakpointParticles reads back from
    that file into cleared arrays (the expected restart state)."""
    import tempfile
    g = _grid()
    r = RefMDOODZ(NX, NZ, XMIN, XMAX, ZMIN, ZMAX, 3)
    r.set_bc_pureshear(1.0)
    r.set_param("iselastic", 1)
    r.set_param("dt", 0.37)
    for k, v in BRK_SCALE.items():
        r.set_scale(k, v)
    x, z, ph = (a[::8].copy() for a in _markers(g, seed=13))   # 640 markers keep the file small
    r.set_markers(x, z, ph)
    rng = np.random.default_rng(17)
    for nm in BRK_MARKER:
        r.marker_field(nm)[:] = rng.normal(0.0, 1.0, len(x))
    for nm in ("u_in", "v_in", "p_in"):
        r.field(nm)[:] = rng.normal(0.0, 1.0, r.field(nm).size)
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as d:
        os.chdir(d)
        try:
            r.make_breakpoint()
            with open("BreakpointXXXXX.dat", "rb") as f:
                data = f.read()
            for nm in BRK_MARKER + ("x", "z"):
                r.marker_field(nm)[:] = 0.0
            r.marker_phase()[:] = -9
            for nm in ("u_in", "v_in", "p_in"):
                r.field(nm)[:] = 0.0
            n = r.load_breakpoint()
        finally:
            os.chdir(cwd)
    out = dict(Nx=NX, Nz=NZ, n_phases=3, image=np.frombuffer(data, np.uint8).copy(), n=n,
               scale=np.array([BRK_SCALE[k] for k in ("L", "V", "S", "T", "t")]),
               dt=r.model("dt"), time=r.model("time"),
               box=np.array([r.model(k) for k in ("xmin", "xmax", "zmin", "zmax")]),
               phase=r.marker_phase().copy(), u=r.field("u_in").copy(), v=r.field("v_in").copy(),
               p=r.field("p_in").copy())
    for nm in BRK_MARKER + ("x", "z"):
        out["m_" + nm] = r.marker_field(nm).copy()
    np.savez_compressed(os.path.join(HERE, "breakpoint_ref.npz"), **out)
    print("breakpoint_ref.npz: %d markers, %d bytes" % (n, len(data)))


def make_rheology_fixture(avg=0, tag="", phases=None, model=None, neumann=False):
    g = _grid()
    r = RefMDOODZ(NX, NZ, XMIN, XMAX, ZMIN, ZMAX, 3)
    r.set_bc_pureshear(1.0)
    if neumann:
        set_neumann_walls(r.tags("BCu"), r.field("BCu_val"), r.tags("BCv"), r.field("BCv_val"))
    for k, v in (model or RHEO_MODEL).items():
        r.set_param(k, v)
    r.set_param("eta_avg", avg)
    r.set_param("R", RHEO_R)
    for p, props in enumerate(phases or RHEO_PHASES):
        for k, v in props.items():
            r.set_mat(k, p, v)
    x, z, ph = _markers(g, seed=11)
    ph[ph == -1] = 0
    r.set_markers(x, z, ph)
    pp = {}
    for centroid, key in ((1, "phase_perc_n"), (0, "phase_perc_s")):
        r.p2g(np.zeros(3), 0, 0, 1, centroid, 1)
        pp[key] = np.array([r.phase_perc(centroid, p).copy() for p in range(3)])
    rng = np.random.default_rng(5)
    f = rheology_inputs(g, rng)
    for name, arr in f.items():
        key = {"u": "u_in", "v": "v_in", "p": "p_in"}.get(name, name)
        r.field(key)[:] = arr
    for p in range(3):
        r.phase_perc(1, p)[:] = pp["phase_perc_n"][p]
        r.phase_perc(0, p)[:] = pp["phase_perc_s"][p]
    # old stresses on the other node sets, as the time loop prepares them
    # (InterpCentroidsToVerticesDouble / InterpVerticesToCentroidsDouble)
    r.strain_rates()
    out = dict(inputs=np.array(sorted(f)), **{"in_" + k: v for k, v in f.items()}, **{"in_" + k: v for k, v in pp.items()})
    # sxxd0_s, szzd0_s, sxz0_n are inputs too: build them like the time loop does
    import ctypes
    Lr = r.lib
    Lr.ref_field.restype = ctypes.POINTER(ctypes.c_double)
    sxxd0_s = _c2v_np(g, f["sxxd0"])
    szzd0_s = _c2v_np(g, f["szzd0"])
    sxz0_n = _v2c_np(g, f["sxz0"])
    r.field("sxxd0_s")[:] = sxxd0_s
    r.field("szzd0_s")[:] = szzd0_s
    r.field("sxz0_n")[:] = sxz0_n
    out["in_sxxd0_s"], out["in_szzd0_s"], out["in_sxz0_n"] = sxxd0_s, szzd0_s, sxz0_n
    for name in ("div_u", "exxd", "ezzd", "exz", "exz_n", "exxd_s", "ezzd_s"):
        out["sr_" + name] = r.field(name).copy()
    r.viscosity_grid()
    for name in ("eta_n", "eta_s", "eta_phys_n", "eta_phys_s", "VE_n", "VE_s", "sxxd", "szzd", "sxz", "sxz_n",
                 "eII_el", "eII_pl", "eII_pwl", "eII_lin", "eII_cst", "d_n", "exx_el", "ezz_el", "exz_el",
                 "exx_diss", "ezz_diss", "exz_diss", "detadexx_n", "detadezz_n", "detadgxz_n", "detadp_n",
                 "ddivpdexx_n", "ddivpdezz_n", "ddivpdgxz_n", "ddivpdp_n", "detadexx_s", "detadezz_s",
                 "detadgxz_s", "detadp_s", "p_corr", "div_u_el", "div_u_pl", "div_u_r", "Wtot", "Wel", "Wdiss",
                 "OverS_n", "OverS_s", "T_s", "P_s", "div_u_s") + (("eII_exp", "eII_gbs") if phases else ()):
        out["vg_" + name] = r.field(name).copy()
    r.rheo_operators(0)
    for name in ("D11_n", "D12_n", "D13_n", "D14_n", "D21_n", "D22_n", "D23_n", "D24_n", "D31_s", "D32_s", "D33_s",
                 "D34_s"):
        out["op0_" + name] = r.field(name).copy()
    r.rheo_operators(1)
    for name in ("D11_n", "D12_n", "D13_n", "D14_n", "D21_n", "D22_n", "D23_n", "D24_n", "D31_s", "D32_s", "D33_s",
                 "D34_s"):
        out["op1_" + name] = r.field(name).copy()
    r.set_param("gz", -1.0)
    if neumann:
        r.set_param("gx", 0.2)
    r.rhs()
    for name in ("roger_x", "roger_z", "rhs_p"):
        out["rhs_" + name] = r.field(name).copy()
    out["gz"] = -1.0
    out["gx"] = 0.2 if neumann else 0.0
    if neumann:
        for name in ("BCu", "BCv"):
            out["bc_" + name] = r.tags(name).copy()
            out["bc_" + name + "_val"] = r.field(name + "_val").copy()
    if avg == 0:
        # decoupled Stokes: non-linear residual (Picard operator, p_corr) and
        # the assembled Picard and Newton blocks in the reference's numbering
        r.rheo_operators(0)
        if neumann:   # the Neumann rows take their Dirichlet terms from the last assembly
            r.assemble(0)
        norms, Fm, Fc = r.residual()
        out["st_norms"] = norms
        for name in ("ru", "rv", "rp"):
            out["st_" + name] = r.field(name).copy()
        for w in range(3):
            out["st_eqn%d" % w] = r.eqn(w)
        for jac in (0, 1):
            if jac:
                r.rheo_operators(1)
            blocks = r.assemble(jac)
            for b, M in zip("ABCD", blocks):
                out["st_J%d_%s_data" % (jac, b)] = M.data
                out["st_J%d_%s_indices" % (jac, b)] = M.indices
                out["st_J%d_%s_indptr" % (jac, b)] = M.indptr
                out["st_J%d_%s_shape" % (jac, b)] = np.array(M.shape)
    np.savez_compressed(os.path.join(HERE, "rheology_ref%s.npz" % tag), **out)
    print("rheology_ref%s.npz: plastic centroids %d / %d" % (tag, (out["vg_eII_pl"] > 0).sum(), out["vg_eII_pl"].size))


THERMAL_CASES = [dict(dt=0.05, shear_heating=1, adiab_heating=1, gz=-1.0),
                 dict(dt=0.2, shear_heating=0, adiab_heating=2, gz=0.0)]


def thermal_inputs(rng, ncx, ncz, Nx, Nz):
    """Seeded energy-equation inputs and thermal boundaries: Dirichlet south
    and north walls (a few south cells with a prescribed flux instead), a
    Dirichlet west wall on the lower half, zero flux elsewhere."""
    Xc, Zc = np.meshgrid(np.arange(ncx), np.arange(ncz))
    f = dict(T=(1.0 + 0.3 * np.sin(0.4 * Xc) * np.cos(0.3 * Zc) + 0.05 * rng.random(Xc.shape)).ravel(),
             rho_n=1.0 + 0.1 * rng.random(ncx * ncz), Cv=0.8 + 0.4 * rng.random(ncx * ncz),
             Qr=0.1 * rng.random(ncx * ncz), Wdiss=0.2 * rng.random(ncx * ncz), alp=0.05 * rng.random(ncx * ncz),
             kx=np.exp(0.5 * rng.standard_normal(Nx * (Nz + 1))), kz=np.exp(0.5 * rng.standard_normal((Nx + 1) * Nz)),
             p=rng.standard_normal(ncx * ncz), p0_n=rng.standard_normal(ncx * ncz),
             v=rng.standard_normal((Nx + 1) * Nz))
    bc = dict(type=np.full(ncx * ncz, -1, np.int8), typS=np.ones(ncx, np.int8), typN=np.ones(ncx, np.int8),
              typW=np.zeros(ncz, np.int8), typE=np.zeros(ncz, np.int8),
              valS=1.0 + 0.1 * rng.random(ncx), valN=0.5 + 0.1 * rng.random(ncx), valW=0.8 + 0.1 * rng.random(ncz),
              valE=np.zeros(ncz))
    bc["typS"][3:6] = 2
    bc["typW"][:ncz // 2] = 1
    return f, bc


def make_thermal_fixture():
    """EnergyDirectSolve (one implicit step) for two settings of the heating
    switches: the matrix and right-hand side it assembled and the new T."""
    Nx, Nz = NX, NZ
    ncx, ncz = Nx - 1, Nz - 1
    out = dict(Nx=Nx, Nz=Nz, box=np.array([XMIN, XMAX, ZMIN, ZMAX]))
    for q, case in enumerate(THERMAL_CASES):
        r = RefMDOODZ(NX, NZ, XMIN, XMAX, ZMIN, ZMAX, 1)
        r.set_bc_pureshear(1.0)
        rng = np.random.default_rng(40 + q)
        f, bc = thermal_inputs(rng, ncx, ncz, Nx, Nz)
        for name, arr in f.items():
            r.field({"p": "p_in", "v": "v_in"}.get(name, name))[:] = arr
        for name in ("type", "typW", "typE", "typS", "typN"):
            r.bct_tags(name)[:] = bc[name]
        for name in ("valW", "valE", "valS", "valN"):
            r.bct_vals(name)[:] = bc[name]
        r.set_param("gz", case["gz"])
        r.set_param("dt", case["dt"])
        r.energy_solve(case["dt"], case["shear_heating"], case["adiab_heating"])
        A, b, x = r.energy_system()
        pre = "c%d_" % q
        out.update({pre + "in_" + k: v for k, v in f.items()})
        out.update({pre + "bc_" + k: v for k, v in bc.items()})
        out[pre + "T"] = r.field("T").copy()
        out[pre + "dT"] = r.field("dT").copy()
        out[pre + "A_data"], out[pre + "A_indices"], out[pre + "A_indptr"] = A.data, A.indices, A.indptr
        out[pre + "rhs"], out[pre + "x"] = b, x
        out[pre + "case"] = np.array([case["dt"], case["shear_heating"], case["adiab_heating"], case["gz"]])
    np.savez_compressed(os.path.join(HERE, "thermal_ref.npz"), **out)
    print("thermal_ref.npz: %d unknowns" % (ncx * ncz))


def _c2v_np(g, cen):
    ncx, ncz = g.ncx, g.ncz
    t = np.zeros((ncz + 2, ncx + 2))
    t[1:-1, 1:-1] = cen.reshape(ncz, ncx)
    t[0, 1:-1] = t[1, 1:-1]
    t[-1, 1:-1] = t[-2, 1:-1]
    t[1:-1, 0] = t[1:-1, 1]
    t[1:-1, -1] = t[1:-1, -2]
    t[0, 0], t[0, -1], t[-1, 0], t[-1, -1] = t[1, 1], t[1, -2], t[-2, 1], t[-2, -2]
    return (0.25 * (t[:-1, :-1] + t[:-1, 1:] + t[1:, :-1] + t[1:, 1:])).ravel()


def _v2c_np(g, ver):
    V = ver.reshape(g.Nz, g.Nx)
    return (0.25 * (V[:-1, :-1] + V[:-1, 1:] + V[1:, :-1] + V[1:, 1:])).ravel()


RESEED_ATTRS = (("Vx", "vx"), ("Vz", "vz"), ("sxxd", "sxxd"), ("szzd", "szzd"), ("sxz", "sxz"),
                ("strain", "strain"), ("strain_pl", "strain_pl"), ("T", "T"), ("P", "P"))


def reseed_inputs(g, seed=11):
    """Markers thinned at random, one cell emptied and some made inactive
    (their slots are reused), random attributes and grid fields."""
    rng = np.random.default_rng(seed)
    x, z = mdz_setups.seed_markers(g, 4, 4, 0.5, seed)
    keep = rng.random(len(x)) > 0.25
    keep &= ~((x > g.xc[6] - 0.5 * g.dx) & (x < g.xc[6] + 0.5 * g.dx) & (z > g.zc[5] - 0.5 * g.dz) &
              (z < g.zc[5] + 0.5 * g.dz))
    x, z = x[keep], z[keep]
    ph = mdz_setups.inclusion_phase(x, z, 0.05, -0.02, 0.18)
    ph[(z > 0.25) & (x < -0.2)] = 2
    ph[::53] = -1
    m = dict(x=x, z=z, phase=ph.astype(np.int32))
    for _, k in RESEED_ATTRS:
        m[k] = rng.normal(size=len(x))
    nc, nv = (g.Nx - 1) * (g.Nz - 1), g.Nx * g.Nz
    fields = dict(T_n=rng.normal(size=nc), sxxd_n=rng.normal(size=nc), szzd_n=rng.normal(size=nc),
                  sxz_s=rng.normal(size=nv), p_n=rng.normal(size=nc))
    return m, fields


def make_strain_fixture():
    """AccumulatedStrainII: random non-negative strain rates on the centroids,
    the markers of the markers fixture (some inactive) with random strains."""
    g = _grid()
    x, z, ph = _markers(g)
    rng = np.random.default_rng(17)
    nc = (NX - 1) * (NZ - 1)
    rates = {k: np.abs(rng.normal(size=nc)) for k in ("eII_el", "eII_pl", "eII_pwl", "eII_lin", "eII_cst")}
    strain0, strain_pl0 = rng.random(len(x)), rng.random(len(x))
    r = RefMDOODZ(NX, NZ, XMIN, XMAX, ZMIN, ZMAX, 3)
    r.set_bc_pureshear(1.0)
    r.set_param("dt", 0.3)
    r.set_markers(x, z, ph)
    r.marker_field("strain")[:] = strain0
    r.marker_field("strain_pl")[:] = strain_pl0
    for k, v in rates.items():
        r.field(k)[:] = v
    r.accumulated_strain()
    np.savez_compressed(os.path.join(HERE, "strain_ref.npz"), Nx=NX, Nz=NZ, box=np.array([XMIN, XMAX, ZMIN, ZMAX]),
                        x=x, z=z, phase=ph, dt=0.3, strain0=strain0, strain_pl0=strain_pl0,
                        strain=r.marker_field("strain").copy(), strain_pl=r.marker_field("strain_pl").copy(),
                        **rates)


def make_stress_fixture():
    """UpdateParticleStress (StressUpdate 0, no rotation, no subgrid
    diffusion): random grid stresses before and after, markers with random
    stresses, zero velocity."""
    g = _grid()
    x, z, ph = _markers(g)
    rng = np.random.default_rng(23)
    nc, nv = (NX - 1) * (NZ - 1), NX * NZ
    flds = dict(sxxd=rng.normal(size=nc), szzd=rng.normal(size=nc), sxxd0=rng.normal(size=nc),
                szzd0=rng.normal(size=nc), sxz=rng.normal(size=nv), sxz0=rng.normal(size=nv))
    m0 = {k: rng.normal(size=len(x)) for k in ("sxxd", "szzd", "sxz")}
    r = RefMDOODZ(NX, NZ, XMIN, XMAX, ZMIN, ZMAX, 3)
    r.set_bc_pureshear(1.0)
    for name, v in (("dt", 0.3), ("StressUpdate", 0), ("StressRotation", 0), ("subgrid_diff", 0)):
        r.set_param(name, v)
    r.set_markers(x, z, ph)
    for k, v in m0.items():
        r.marker_field(k)[:] = v
    for k, v in flds.items():
        r.field(k)[:] = v
    r.update_particle_stress()
    np.savez_compressed(os.path.join(HERE, "stress_ref.npz"), Nx=NX, Nz=NZ, box=np.array([XMIN, XMAX, ZMIN, ZMAX]),
                        x=x, z=z, phase=ph, **flds, **{"m0_" + k: v for k, v in m0.items()},
                        **{"m_" + k: r.marker_field(k).copy() for k in m0})


def make_reseed_fixture():
    g = _grid()
    m, fields = reseed_inputs(g)
    out = dict(Nx=NX, Nz=NZ, box=np.array([XMIN, XMAX, ZMIN, ZMAX]), **{"in_" + k: v for k, v in m.items()},
               **fields)
    n = len(m["x"])
    cap = n + 4 * (NX - 1) * (NZ - 1)
    for direct in (1, 0):
        for mpc in (16, 9):
            r = RefMDOODZ(NX, NZ, XMIN, XMAX, ZMIN, ZMAX, 3)
            r.set_bc_pureshear(1.0)
            r.set_markers_cap(m["x"], m["z"], m["phase"], cap)
            for ref_name, key in RESEED_ATTRS:
                r.marker_field(ref_name)[:] = m[key]
            r.field("T")[:] = fields["T_n"]
            r.field("sxxd")[:] = fields["sxxd_n"]
            r.field("szzd")[:] = fields["szzd_n"]
            r.field("sxz")[:] = fields["sxz_s"]
            r.field("p_in")[:] = fields["p_n"]
            n_new = r.reseed(direct, mpc)
            tag = "d%d_m%d_" % (direct, mpc)
            # only the slots the reseeding wrote (inactive ones reused, then
            # appended ones) are stored; every other marker is unchanged
            ph_out = r.marker_phase().copy()
            written = np.concatenate([np.flatnonzero(m["phase"] == -1), np.arange(n, n_new)])
            written = written[(written >= n) | (ph_out[np.minimum(written, n_new - 1)] != -1)]
            untouched = np.setdiff1d(np.arange(n), written)
            assert np.array_equal(r.marker_field("x")[untouched], m["x"][untouched])
            assert np.array_equal(ph_out[untouched], m["phase"][untouched])
            out[tag + "n"] = n_new
            out[tag + "slots"] = written
            out[tag + "x"] = r.marker_field("x")[written].copy()
            out[tag + "z"] = r.marker_field("z")[written].copy()
            out[tag + "phase"] = ph_out[written]
            for ref_name, key in RESEED_ATTRS:
                vals = r.marker_field(ref_name)
                assert np.array_equal(vals[untouched], m[key][untouched]), key
                out[tag + key] = vals[written].copy()
            print("reseed direct=%d min_part_cell=%d: %d -> %d markers" % (direct, mpc, n, n_new))
    np.savez_compressed(os.path.join(HERE, "reseed_ref.npz"), **out)


# ---- grid properties (ShearModCompExpGrid, CohesionFrictionDilationGrid) ------------
GRIDPROP_PHASES = [
    # friction, dilation and cohesion all soften
    dict(mu=1.0, bet=1e-2, C=1.0, phi=0.5, psi=0.1, C_end=0.5, phi_end=0.3, psi_end=0.0, pls_start=0.1, pls_end=0.9,
         coh_soft=1, phi_soft=1, psi_soft=1),
    # cohesion softening only, another strain window
    dict(mu=2.0, bet=2e-2, C=2.0, phi=0.6, psi=0.0, C_end=0.2, phi_end=0.6, psi_end=0.0, pls_start=0.0, pls_end=0.5,
         coh_soft=1, phi_soft=0, psi_soft=0),
    # no softening
    dict(mu=0.5, bet=5e-3, C=0.7, phi=0.4, psi=0.05, C_end=0.7, phi_end=0.4, psi_end=0.05, pls_start=0.0,
         pls_end=1.0, coh_soft=0, phi_soft=0, psi_soft=0),
]


def make_gridprops_fixture():
    """Phase fractions projected from the markers, then the reference's
    ShearModCompExpGrid (harmonic shear modulus and compressibility) and
    CohesionFrictionDilationGrid (smooth softening by the markers' plastic
    strain: P2Mastah to the centroids, Interp_P2N to the vertices), for
    itp_stencil 1 and 9."""
    g = _grid()
    x, z, ph = _markers(g)
    rng = np.random.default_rng(31)
    strain_pl = np.abs(rng.normal(0.5, 0.4, len(x)))
    out = dict(Nx=NX, Nz=NZ, box=np.array([XMIN, XMAX, ZMIN, ZMAX]), x=x, z=z, phase=ph, strain_pl=strain_pl)
    for stencil in (1, 9):
        r = RefMDOODZ(NX, NZ, XMIN, XMAX, ZMIN, ZMAX, 3)
        r.set_bc_pureshear(1.0)
        r.set_param("itp_stencil", stencil)
        for p, props in enumerate(GRIDPROP_PHASES):
            for k, v in props.items():
                r.set_mat(k, p, v)
        r.set_markers(x, z, ph)
        r.marker_field("strain_pl")[:] = strain_pl
        for centroid in (1, 0):
            r.p2g(np.zeros(3), 0, 0, 1, centroid, stencil)
            out["s%d_pp_c%d" % (stencil, centroid)] = np.array([r.phase_perc(centroid, p).copy() for p in range(3)])
        r.shear_mod_grid()
        r.cohesion_grid()
        for k in ("mu_n", "mu_s", "bet_n", "bet_s", "C_n", "C_s", "fric_n", "fric_s", "dil_n", "dil_s"):
            out["s%d_%s" % (stencil, k)] = r.field(k).copy()
    np.savez_compressed(os.path.join(HERE, "gridprops_ref.npz"), **out)
    print("gridprops_ref.npz:", len(out), "arrays")


def make_pressure_fixture():
    """UpdateParticlePressure: marker pressures plus the centroid increment
    p_in - p0_n (Plith_trick 0) or its dynamic part (Plith_trick 1), without
    subgrid diffusion."""
    g = _grid()
    x, z, ph = _markers(g)
    rng = np.random.default_rng(41)
    nc = (NX - 1) * (NZ - 1)
    flds = dict(p_in=rng.normal(size=nc), p0_n=rng.normal(size=nc), p_lith=rng.normal(size=nc),
                p_lith0=rng.normal(size=nc))
    P0 = rng.normal(size=len(x))
    out = dict(Nx=NX, Nz=NZ, box=np.array([XMIN, XMAX, ZMIN, ZMAX]), x=x, z=z, phase=ph, P0=P0, **flds)
    for trick in (0, 1):
        r = RefMDOODZ(NX, NZ, XMIN, XMAX, ZMIN, ZMAX, 3)
        r.set_bc_pureshear(1.0)
        r.set_param("Plith_trick", trick)
        r.set_param("subgrid_diff", 0)
        r.set_markers(x, z, ph)
        r.marker_field("P")[:] = P0
        for k, v in flds.items():
            r.field(k)[:] = v
        r.update_particle_pressure()
        out["P_trick%d" % trick] = r.marker_field("P").copy()
    np.savez_compressed(os.path.join(HERE, "pressure_ref.npz"), **out)
    print("pressure_ref.npz:", len(out), "arrays")


if __name__ == "__main__":
    what = sys.argv[1:] or ["markers", "rheology", "reseed", "strain", "stress", "gridprops", "pressure", "thermal",
                            "phasemap", "breakpoint"]
    if "gridprops" in what:
        make_gridprops_fixture()
    if "pressure" in what:
        make_pressure_fixture()
    if "stress" in what:
        make_stress_fixture()
    if "strain" in what:
        make_strain_fixture()
    if "reseed" in what:
        make_reseed_fixture()
    if "markers" in what:
        make_markers_fixture()
    if "rheology" in what:
        make_rheology_fixture(0)
        make_rheology_fixture(1, "_harm")
        make_rheology_fixture(2, "_geom")
    if "rheology" in what or "mech" in what:
        make_rheology_fixture(0, "_mech", RHEO_PHASES_MECH, RHEO_MODEL_MECH)
    if "thermal" in what:
        make_thermal_fixture()
    if "phasemap" in what:
        make_phasemap_fixture()
    if "breakpoint" in what:
        make_breakpoint_fixture()
    if "rheology" in what or "neumann" in what:
        make_rheology_fixture(0, "_neumann", neumann=True)
