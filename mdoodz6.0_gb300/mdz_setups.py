"""Synthetic model setups: the harness's own SetParticles / SetBCs for the
benchmark configurations (the reference keeps these in per-model plugins,
SOURCE/set_*.c).  Markers are seeded on a regular sub-grid of each cell with a
uniform jitter from a fixed seed; BCs are the reference's free-slip pure-shear
tags (shear_style = 0).
"""
import numpy as np


def seed_markers(grid, nmx, nmz, jitter=0.5, seed=12345):
    """nmx x nmz markers per cell, each displaced uniformly by up to
    +/- jitter x (marker spacing) in x and z, clipped into the box.
    Returned in cell-major order (all markers of cell 0, then cell 1, ...;
    inside a cell by sub-row, then sub-column)."""
    rng = np.random.default_rng(seed)
    ncx, ncz = grid.ncx, grid.ncz
    hx, hz = grid.dx / nmx, grid.dz / nmz
    # sub-grid indices in (cell row, cell column, sub-row, sub-column) order
    cz = np.arange(ncz)[:, None, None, None]
    cx = np.arange(ncx)[None, :, None, None]
    j = np.arange(nmz)[None, None, :, None]
    i = np.arange(nmx)[None, None, None, :]
    shape = (ncz, ncx, nmz, nmx)
    x = np.broadcast_to(grid.xmin + ((cx * nmx + i) + 0.5) * hx, shape).ravel()
    z = np.broadcast_to(grid.zmin + ((cz * nmz + j) + 0.5) * hz, shape).ravel()
    n = x.size
    x = x + rng.uniform(-jitter, jitter, n) * hx
    z = z + rng.uniform(-jitter, jitter, n) * hz
    x = np.clip(x, grid.xmin, grid.xmax)
    z = np.clip(z, grid.zmin, grid.zmax)
    return x, z


def inclusion_phase(x, z, xc, zc, r):
    return (np.hypot(x - xc, z - zc) < r).astype(np.int32)


# ---------------------------------------------------------------------------
# Benchmark configurations.  Each builder returns a dict with the grid, the
# markers (positions, phases and attributes), the materials, the step model
# and the initial velocity / pressure.  `N` overrides the grid size so the same
# physics runs small in tests.

class Scales:
    """Characteristic scales of the lithosphere setup (the reference
    non-dimensionalises every input with such a set, ScaleMe in
    SOURCE/InputOutput.c): viscosity, length, velocity; time, stress and
    strain rate follow.  Temperature stays in kelvin."""

    def __init__(self, eta=1e22, L=1e3, V=1e-10):
        self.eta, self.L, self.V = eta, L, V
        self.t = L / V
        self.E = 1.0 / self.t
        self.S = eta * self.E


def _markers_dict(x, z, ph, **attrs):
    n = len(x)
    m = dict(x=x, z=z, phase=ph.astype(np.int32))
    for k in ("sxxd", "szzd", "sxz", "strain_pl", "strain", "T", "P"):
        m[k] = np.zeros(n)
    m["cmul"] = np.ones(n)
    m.update(attrs)
    return m


def pure_shear_velocity(grid, eps):
    u = (-grid.xg[None, :] * eps + 0.0 * grid.zvx[:, None]).ravel()
    v = (grid.zg[:, None] * eps + 0.0 * grid.xvz[None, :]).ravel()
    return u, v


def config_inclusion(N=101, nm=4, seed=12345):
    """Linear-viscous pure shear, unit square, circular inclusion r = 0.1 with
    viscosity 1e3 in a matrix of viscosity 1; free-slip walls, eps_BG = 1."""
    import mdz
    g = mdz.Grid(N, N, -0.5, 0.5, -0.5, 0.5).set_bc_pureshear(1.0)
    x, z = seed_markers(g, nm, nm, 0.5, seed)
    ph = inclusion_phase(x, z, 0.0, 0.0, 0.1)
    phases = [dict(cstv=1, eta0=1.0, mu=1.0, bet=1.0, C=1e90, phi=0.0, rho=1.0, Slim=1e90, n_vp=1.0, gs_ref=1.0),
              dict(cstv=1, eta0=1e3, mu=1.0, bet=1.0, C=1e90, phi=0.0, rho=1.0, Slim=1e90, n_vp=1.0, gs_ref=1.0)]
    mat = mdz.Materials.from_phases(phases)
    prm = mdz.RheoParams.make(dt=1e-3, iselastic=0, step=1, eta_avg=0)
    # a linear problem: one defect solve, to 1e-12 (the pressure around a 1e3
    # inclusion is conditioned far worse than the velocity: a 1e-9 solve leaves
    # ~1e-6 relative pressure error)
    model = mdz.Model.make(prm, newton=0, nit_max=4, rel_tol=1e-8, lin_rtol=1e-12, line_search=0)
    u, v = pure_shear_velocity(g, 1.0)
    return dict(name="inclusion", grid=g, markers=_markers_dict(x, z, ph), mat=mat, model=model, u=u, v=v,
                p=np.zeros(g.size(1)))


def config_vep(N=401, nm=4, seed=12345, noise=0.01):
    """Visco-elasto-plastic Drucker-Prager pure shear: G = 1, eta = 1e3, C = 1
    with 1 % seeded per-marker noise, phi = 30 deg, psi = 0, dt = 1e-2,
    eps_BG = 1; viscoplastic regularisation eta_vp = 0.05.

    The box deforms with the flow (ispureshear_ALE = 1, as the reference's
    shear-band setup BENCHMARKS_old_input/SH_Duretz14.txt runs it): at
    dt = 1e-2 the inflow through fixed walls would move markers two cells
    (401 x 401) to ten cells (2049 x 2049) per step, more than the reseeding's
    two-quarter-cell neighbourhood (CountPartCell) can refill.  The material
    is homogeneous, so until the stress reaches the yield stress the
    pure-shear start is the solution (residual at round-off, ~1e-19): the
    absolute tolerance abs_tol = 1e-14 (the reference's abs_tol_u / abs_tol_p
    test, Main_DOODZ.c:830) accepts it; relative tolerance 1e-8 otherwise.
    Loading is elastic, tau_II = 2 G t to first order, so yielding
    (C cos phi = 0.866) starts near step 44."""
    import mdz
    g = mdz.Grid(N, N, -0.5, 0.5, -0.5, 0.5).set_bc_pureshear(1.0)
    x, z = seed_markers(g, nm, nm, 0.5, seed)
    ph = np.zeros(len(x), np.int32)
    rng = np.random.default_rng(seed + 1)
    phases = [dict(cstv=1, eta0=1e3, mu=1.0, bet=1e-2, C=1.0, phi=np.pi / 6, psi=0.0, rho=1.0, Slim=1e10,
                   eta_vp=0.05, n_vp=1.0, gs_ref=1.0, pls_start=0.0, pls_end=1.0)]
    mat = mdz.Materials.from_phases(phases)
    prm = mdz.RheoParams.make(dt=1e-2, iselastic=1, step=1, eta_avg=0)
    model = mdz.Model.make(prm, newton=1, nit_max=10, rel_tol=1e-8, abs_tol=1e-14, lin_rtol=1e-6, line_search=1,
                           reseed=1, min_part_cell=16, direct_neighbour=0, ispureshear_ale=1)
    u, v = pure_shear_velocity(g, 1.0)
    m = _markers_dict(x, z, ph, cmul=1.0 + noise * rng.standard_normal(len(x)))
    return dict(name="vep", grid=g, markers=m, mat=mat, model=model, u=u, v=v, p=np.zeros(g.size(1)), eps_bg=1.0)


def config_lithosphere(Nx=1025, Nz=513, nm=4, seed=12345, precision=64, learned=0):
    """Layered lithosphere over 1000 x 400 km: upper crust 0-20 km, lower crust
    20-35 km, mantle lithosphere 35-120 km, asthenosphere; each phase with
    dislocation creep (n in [3.0, 3.5], A and Q log-uniform from the seed),
    diffusion creep, Maxwell elasticity and Drucker-Prager plasticity; linear
    geotherm 0 -> 1330 C at 120 km then adiabatic (0.3 K/km); 1 cm/yr
    extension (pure-shear walls); gravity.  Non-dimensionalised with Scales()."""
    import mdz
    sc = Scales()
    L = sc.L
    g = mdz.Grid(Nx, Nz, -500e3 / L, 500e3 / L, -400e3 / L, 0.0).set_bc_pureshear(0.0)
    Vext = 0.01 / (365.25 * 24 * 3600)               # 1 cm/yr in m/s
    eps = -2 * 0.5 * Vext / 1000e3                   # extension: u = -x eps > 0 on the east wall
    g.set_bc_pureshear(eps / sc.E)
    x, z = seed_markers(g, nm, nm, 0.5, seed)
    depth = -z * L                                   # m
    ph = np.where(depth < 20e3, 0, np.where(depth < 35e3, 1, np.where(depth < 120e3, 2, 3))).astype(np.int32)
    T = np.where(depth < 120e3, 273.15 + 1330.0 * depth / 120e3, 273.15 + 1330.0 + 0.3e-3 * (depth - 120e3))
    rng = np.random.default_rng(seed)
    R = 8.314510

    def logu(a, b):
        return float(np.exp(rng.uniform(np.log(a), np.log(b))))
    # (A range Pa^-n s^-1, Q range J/mol, diffusion A, Q), per phase
    specs = [((1e-28, 1e-25), (135e3, 225e3), 1e-19, 200e3, 2700.0),
             ((1e-26, 1e-23), (200e3, 300e3), 1e-20, 250e3, 2900.0),
             ((1e-17, 1e-15), (480e3, 540e3), 1e-15, 375e3, 3300.0),
             ((1e-16, 1e-14), (430e3, 480e3), 1e-14, 335e3, 3300.0)]
    phases = []
    S, t = sc.S, sc.t
    for (Ar, Qr, Ad, Qd, rho) in specs:
        n = float(rng.uniform(3.0, 3.5))
        A = logu(*Ar)
        Q = logu(*Qr)
        phases.append(dict(
            pwlv=1, npwl=n, Apwl=A * S ** n * t, Qpwl=Q, Vpwl=0.0, mpwl=0.0, rpwl=0.0, fpwl=1.0, apwl=0.0, Fpwl=1.0,
            pref_pwl=1.0, linv=1, nlin=1.0, Alin=Ad * S * t, Qlin=Qd, Vlin=0.0, mlin=0.0, rlin=0.0, flin=1.0,
            alin=0.0, Flin=1.0, mu=3e10 / S, bet=1e-11 * S, C=1e7 / S, phi=np.pi / 6, psi=0.0, rho=rho, Slim=1e90,
            eta_vp=1e21 / sc.eta, n_vp=1.0, gs_ref=1.0, pls_start=0.0, pls_end=1.0))
    mat = mdz.Materials.from_phases(phases, R=R)
    # visco-elasto-plastic (Maxwell elasticity, G = 30 GPa, dt = 10 kyr); the
    # viscosity limiter's tangent is the derivative of the limited law
    prm = mdz.RheoParams.make(dt=1e4 * 365.25 * 24 * 3600 / t, iselastic=1, step=1, eta_avg=0,
                              mineta=1e19 / sc.eta, maxeta=1e24 / sc.eta, scale_T=1.0, scale_E=sc.E,
                              scale_S=sc.S, scale_eta=sc.eta, scale_L=sc.L, clamp_tangent=1)
    # Picard iterations until resx or resz dropped tenfold, then Newton
    # (Picard2Newton of the reference); 30 iterations at most
    # (no line search: the reference's default, line_search = 0; each defect
    # solve asks only for the reduction the non-linear iteration can use; the
    # FP32 form also evaluates the local rheology of the first two non-linear
    # iterations in FP32; once the residual is below 1e-2 of its first value
    # the multigrid hierarchy of the previous solve is kept; markers are
    # reseeded after every advection, CountPartCell with RESEED = 1 and the
    # reference's defaults Reseed = 1, min_part_cell = 16, DirectNeighbour = 0:
    # the extension's inflow through the bottom wall empties the lowest cells
    # of markers within a few tens of steps otherwise)
    model = mdz.Model.make(prm, gz=-9.81 * L / S, newton=1, nit_max=30, rel_tol=1e-8, lin_rtol=1e-5,
                           line_search=0, precision=precision, learned_guess=learned, picard2newton=1,
                           pic2newt_cond=1e-1, nit_pic_max=10, newton_maxit=200, adaptive_lin_tol=1,
                           fp32_rheology_its=2 if precision == 32 else 0, mg_reuse_below=1e-2,
                           reseed=1, min_part_cell=16, direct_neighbour=0)
    u, v = pure_shear_velocity(g, eps / sc.E)
    m = _markers_dict(x, z, ph, T=T)
    # initial pressure: lithostatic column of the layered densities (the
    # reference starts from ComputeLithostaticPressure as well)
    zc = g.zc
    dz = g.dz
    rho_of = lambda d: np.where(d < 20e3, specs[0][4], np.where(d < 35e3, specs[1][4], specs[2][4]))
    rho_c = rho_of(-zc * L)
    col = np.cumsum((rho_c * (-model.gz) * dz)[::-1])[::-1] - 0.5 * rho_c * (-model.gz) * dz
    p0 = np.repeat(col[:, None], g.ncx, axis=1).ravel()
    # markers start at the lithostatic pressure of their depth (the reference
    # interpolates p_lith to them, Main_DOODZ.c:297)
    m["P"] = np.interp(z, zc, col)
    return dict(name="lithosphere", grid=g, markers=m, mat=mat, model=model, u=u, v=v, p=p0, scales=sc)


def config_shear_band(N=2049, nm=4, seed=12345, noise=0.01, precision=64, learned=0):
    """Shear-band localisation: VEP pure shear with cohesion softening linearly
    from 1 to 0.5 over accumulated plastic strain 0-1, 1 % seeded cohesion
    noise, 16 markers per cell, box deforming with the flow.

    The time step is the Courant step of the walls (Courant number 0.5 at
    |v| = 0.5: dt = dx), the reference's default criterion (Courant = 0.5,
    EvaluateCourantCriterion): with the deforming box each step loses the
    markers of a band 0.5 dt |v| wide at the inflowing walls (the midpoint
    stage of RogerGuntherII leaves the box), which the reseeding refills only
    while the band is at most two quarter cells (dt <= 4 dx); the 1e-2 step
    of the 401 x 401 model is twenty times that at 2049 x 2049.  The shear
    modulus is 100 so that the elastic loading, 2 G dt per step, reaches the
    yield stress (C cos phi = 0.87) after some nine steps and leaves forty for
    yielding, softening and localisation."""
    cfg = config_vep(N=N, nm=nm, seed=seed, noise=noise)
    import mdz
    g = cfg["grid"]
    phases = [dict(cstv=1, eta0=1e3, mu=100.0, bet=1e-2, C=1.0, C_end=0.5, coh_soft=1, phi=np.pi / 6, psi=0.0,
                   rho=1.0, Slim=1e10, eta_vp=0.05, n_vp=1.0, gs_ref=1.0, pls_start=0.0, pls_end=1.0)]
    cfg["mat"] = mdz.Materials.from_phases(phases)
    cfg["model"].rheo.dt = min(g.dx, g.dz) * 0.5 / 0.5
    cfg["model"].softening = 1
    cfg["model"].nit_max = 15
    cfg["model"].precision = precision
    cfg["model"].learned_guess = learned
    cfg["name"] = "shear_band"
    return cfg


# ranges of the learned guess's training tuples for the lithosphere model:
# log10 strain rate [1/s], T [K], P [Pa], log10 dt [s]
LO_LITHO, HI_LITHO = [-18.0, 273.0, 0.0, 9.0], [-12.0, 1800.0, 15e9, 12.0]


def train_guess(ctx, cfg, steps=3000, n=1 << 20, batch=65536, seed=1, lo=LO_LITHO, hi=HI_LITHO):
    """The learned local-rheology start of a configuration: n tuples drawn
    over [lo, hi] and labelled by the plain local solve of the model's
    materials on the device, then `steps` Adam steps; returns the final loss."""
    ctx.mlp_init(seed)
    ctx.mlp_generate(cfg["mat"], cfg["model"].rheo, n, seed, lo, hi)
    return ctx.mlp_train(steps, batch, 2e-3)


def marker_capacity(cfg):
    """Marker slots of a run: twice the seeded markers.  Reseeding adds one
    marker to every quarter cell that holds fewer than min_part_cell / 4 and
    never removes any, so a quarter cell that a marker leaves gets a new one
    while the cell the marker entered keeps it: the count creeps up over the
    steps (by about a quarter over the first 25 steps of the 1025 x 513
    lithosphere model) before the quarter cells hold enough spare markers.
    Markers that leave the box free their slots for the next pass."""
    g = cfg["grid"]
    n = len(cfg["markers"]["x"])
    return 2 * n + 4 * g.ncx * g.ncz


def renew_bcs(cfg):
    """The setup's SetBCs for the next step: with a deforming box
    (ispureshear_ale) the pure-shear Dirichlet values follow the moved walls.
    Returns True when they changed."""
    if not cfg["model"].ispureshear_ale:
        return False
    cfg["grid"].set_bc_pureshear(cfg["eps_bg"])
    return True


def time_step(ctx, cfg):
    """One time step of a configuration on a context from load_context: the
    library's step, then the setup's boundary values for the next one."""
    rep = ctx.time_step(cfg["mat"], cfg["model"])
    if renew_bcs(cfg):
        ctx.set_boundary_values(cfg["grid"])
    return rep


def load_context(cfg, max_markers=None):
    """Context with the configuration's markers, attributes and initial fields
    resident; room for max_markers markers (default: marker_capacity)."""
    import mdz
    g, m = cfg["grid"], cfg["markers"]
    ctx = mdz.Context(g, cfg["mat"].n_phases, max_markers or marker_capacity(cfg))
    ctx.set_markers(m["x"], m["z"], m["phase"])
    for attr, key in ((mdz.M_SXXD, "sxxd"), (mdz.M_SZZD, "szzd"), (mdz.M_SXZ, "sxz"), (mdz.M_STRAIN_PL, "strain_pl"),
                      (mdz.M_STRAIN, "strain"), (mdz.M_T, "T"), (mdz.M_CMUL, "cmul"), (mdz.M_P, "P")):
        ctx.set_marker_attr(attr, m[key])
    f = mdz.GridFields(g, cfg["mat"].n_phases)
    f["u"], f["v"], f["p"] = cfg["u"], cfg["v"], cfg["p"]
    s = f.struct()
    for name in mdz.FIELD_NAMES:
        if name not in ("u", "v", "p"):
            setattr(s, name, None)
    ctx._check(ctx.L.mdz_sync_fields(ctx.h, mdz.C.byref(s), 1))
    return ctx
