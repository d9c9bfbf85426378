/*
 * Harness around the reference's OWN hot-path C functions (MDOODZ 6.0,
 * compiled in place from the reference SOURCE directory by oracle/Makefile,
 * target `ref`).  It builds the reference's `grid`, `markers`, `params`,
 * `mat_prop` and `scale` structures from plain arrays and exposes a handful of
 * extern "C" entry points that Python (ctypes) calls to produce golden
 * vectors.  Nothing here re-implements an algorithm: every number this harness
 * returns is computed by the reference's own functions.
 *
 * Test infrastructure only: the resulting library lives in oracle/_ref/ and is
 * loaded only by tests/golden/make_golden.py and the oracle self-checks.
 *
 * Reference entry points driven from here (paths inside the reference repo):
 *   SOURCE/GridRoutines.c:230        SetGridCoordinates
 *   SOURCE/GridRoutines.c:481        GridIndices
 *   SOURCE/MemoryAllocFree.c:182,333 PartAlloc, GridAlloc
 *   SOURCE/ParticleRoutines.c:3226   P2Mastah
 *   SOURCE/ParticleRoutines.c:4485   CountPartCell_Old
 *   SOURCE/ParticleRoutines.c:2439   Interp_Grid2P
 *   SOURCE/ParticleRoutines.c:2612   Interp_Grid2P_centroids2
 *   SOURCE/AdvectionRoutines.c:569   RogerGuntherII
 *   SOURCE/RheologyDensity.c:1902    StrainRateComponents
 *   SOURCE/RheologyDensity.c:961     NonNewtonianViscosityGrid
 *   SOURCE/RheologyDensity.c:713     RheologicalOperators
 *   SOURCE/StokesRoutines.c:922      EvaluateRHS
 *   SOURCE/StokesRoutines.c:1134     EvalNumberOfEquations
 *   SOURCE/StokesRoutines.c:839      EvaluateStokesResidualDecoupled
 *   SOURCE/StokesAssemblyDecoupled.c:1573 BuildStokesOperatorDecoupled
 *   SOURCE/StokesAssemblyDecoupled.c:3834 BuildJacobianOperatorDecoupled
 *   SOURCE/RheologyParticles.c:1124  UpdateParticleStress
 *   SOURCE/ParticleRoutines.c:3543   CountPartCell (RESEED = 1: marker reseeding)
 *   SOURCE/RheologyParticles.c:191   AccumulatedStrainII
 *   SOURCE/RheologyParticles.c:1004  UpdateParticlePressure
 *   SOURCE/RheologyDensity.c:1422    CohesionFrictionDilationGrid
 *   SOURCE/RheologyDensity.c:1666    ShearModCompExpGrid
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <omp.h>
#include "header_MDOODZ.h"

/* Reference functions used here whose prototypes are not in its header. */
void CountPartCell_Old(markers *, grid *, params, surface, int, scale);
void Interp_Grid2P_centroids2(markers, DoodzFP *, grid *, double *, double *, double *, int, int, char *, params *);
void BuildStokesOperatorDecoupled(grid *, params, int, double *, double *, double *, double *, SparseMat *, SparseMat *,
                                  SparseMat *, SparseMat *, SparseMat *, int);
void BuildJacobianOperatorDecoupled(grid *, params, int, double *, double *, double *, double *, SparseMat *, SparseMat *,
                                    SparseMat *, SparseMat *, SparseMat *, int);
void EvaluateStokesResidualDecoupled(SparseMat *, SparseMat *, SparseMat *, SparseMat *, SparseMat *, Nparams *, grid *,
                                     params, scale, int);

static params   g_model;
static grid     g_mesh;
static mat_prop g_mat;
static scale    g_scale;
static markers  g_parts;
static Nparams  g_nmodel;
static int      g_have_grid = 0, g_have_parts = 0, g_have_eqn = 0;
static SparseMat g_S, g_SA, g_SB, g_SC, g_SD;     /* Picard blocks    */
static SparseMat g_J, g_JA, g_JB, g_JC, g_JD;     /* Jacobian blocks  */
static int g_have_picard = 0, g_have_jac = 0;

/* ------------------------------------------------------------------------ */
int ref_setup(int Nx, int Nz, double xmin, double xmax, double zmin, double zmax, int nphases) {
    memset(&g_model, 0, sizeof g_model);
    memset(&g_mesh, 0, sizeof g_mesh);
    memset(&g_mat, 0, sizeof g_mat);
    memset(&g_nmodel, 0, sizeof g_nmodel);
    g_scale.eta = g_scale.L = g_scale.V = g_scale.T = g_scale.t = 1.0;
    g_scale.a = g_scale.E = g_scale.S = g_scale.m = g_scale.rho = 1.0;
    g_scale.F = g_scale.J = g_scale.W = g_scale.Cv = g_scale.rhoE = g_scale.k = 1.0;
    g_model.Nx = Nx; g_model.Nz = Nz; g_model.Nt = 1;
    g_model.xmin = xmin; g_model.xmax = xmax; g_model.zmin = zmin; g_model.zmax = zmax;
    g_model.xmin0 = xmin; g_model.xmax0 = xmax; g_model.zmin0 = zmin; g_model.zmax0 = zmax;
    g_model.Nb_phases = nphases; g_mat.Nb_phases = nphases;
    g_model.itp_stencil = 1; g_model.mineta = 1e-100; g_model.maxeta = 1e100;
    g_model.decoupled_solve = 1; g_model.step = 1; g_model.loc_iter = 1;
    g_mat.R = Rg;
    GridAlloc(&g_mesh, &g_model);
    SetGridCoordinates(&g_mesh, &g_model, Nx, Nz);
    GridIndices(&g_mesh);
    g_have_grid = 1;
    return 0;
}

/* Pure-shear, free-slip box: the BC tags of the reference's pure-shear setup
 * (shear_style = 0 branch of SetBCs, SOURCE/set_Shear_VEVP.c:177-265), with
 * every centroid and vertex an inner node. */
int ref_set_bc_pureshear(double EpsBG) {
    int Nx = g_mesh.Nx, Nz = g_mesh.Nz, k, l, c;
    for (l = 0; l < Nz + 1; l++)
        for (k = 0; k < Nx; k++) {
            c = k + l * Nx;
            g_mesh.BCu.type[c] = -1; g_mesh.BCu.val[c] = 0.0;
            if (k == 0 || k == Nx - 1) { g_mesh.BCu.type[c] = 0; g_mesh.BCu.val[c] = -g_mesh.xg_coord[k] * EpsBG; }
            if (l == 0 || l == Nz) { g_mesh.BCu.type[c] = 13; g_mesh.BCu.val[c] = 0.0; }
        }
    for (l = 0; l < Nz; l++)
        for (k = 0; k < Nx + 1; k++) {
            c = k + l * (Nx + 1);
            g_mesh.BCv.type[c] = -1; g_mesh.BCv.val[c] = 0.0;
            if (l == 0 || l == Nz - 1) { g_mesh.BCv.type[c] = 0; g_mesh.BCv.val[c] = g_mesh.zg_coord[l] * EpsBG; }
            if (k == 0 || k == Nx) { g_mesh.BCv.type[c] = 13; g_mesh.BCv.val[c] = 0.0; }
        }
    for (c = 0; c < (Nx - 1) * (Nz - 1); c++) { g_mesh.BCp.type[c] = -1; g_mesh.BCp.val[c] = 0.0; g_mesh.BCt.type[c] = -1; }
    for (c = 0; c < Nx * Nz; c++) { g_mesh.BCg.type[c] = -1; }
    g_model.EpsBG = EpsBG;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Scalar model / scaling parameters by name.                               */
int ref_set_param(const char *name, double v) {
#define P_D(f) if (!strcmp(name, #f)) { g_model.f = v; return 0; }
#define P_I(f) if (!strcmp(name, #f)) { g_model.f = (int)v; return 0; }
    P_D(dt) P_D(mineta) P_D(maxeta) P_D(gx) P_D(gz) P_D(EpsBG)
    P_I(iselastic) P_I(step) P_I(eta_avg) P_I(itp_stencil) P_I(compressible) P_I(Newton)
    P_I(isperiodic_x) P_I(StressUpdate) P_I(StressRotation) P_I(subgrid_diff) P_I(ConservInterp)
    P_I(free_surf) P_I(aniso) P_I(loc_iter) P_I(Plith_trick)
#undef P_D
#undef P_I
    if (!strcmp(name, "scale_eta")) { g_scale.eta = v; return 0; }
    if (!strcmp(name, "scale_L")) { g_scale.L = v; return 0; }
    if (!strcmp(name, "scale_T")) { g_scale.T = v; return 0; }
    if (!strcmp(name, "scale_E")) { g_scale.E = v; return 0; }
    if (!strcmp(name, "scale_S")) { g_scale.S = v; return 0; }
    if (!strcmp(name, "R")) { g_mat.R = v; return 0; }
    return -1;
}

/* Per-phase material property by name (mat_prop, SOURCE/header_MDOODZ.h:46-63). */
int ref_set_mat(const char *name, int p, double v) {
#define M_D(f) if (!strcmp(name, #f)) { g_mat.f[p] = v; return 0; }
#define M_I(f) if (!strcmp(name, #f)) { g_mat.f[p] = (int)v; return 0; }
    M_D(eta0) M_D(rho) M_D(mu) M_D(C) M_D(phi) M_D(psi) M_D(Slim) M_D(n) M_D(A) M_D(Ea) M_D(Va) M_D(alp) M_D(bet)
    M_D(tpwl) M_D(Qpwl) M_D(Vpwl) M_D(npwl) M_D(mpwl) M_D(Apwl) M_D(apwl) M_D(fpwl) M_D(rpwl) M_D(Fpwl) M_D(pref_pwl)
    M_D(tlin) M_D(Qlin) M_D(Vlin) M_D(nlin) M_D(mlin) M_D(Alin) M_D(alin) M_D(flin) M_D(rlin) M_D(Flin)
    M_D(gs_ref) M_D(C_end) M_D(phi_end) M_D(psi_end) M_D(pls_start) M_D(pls_end) M_D(eta_vp) M_D(n_vp)
    M_D(Qexp) M_D(Sexp) M_D(Eexp) M_D(Gexp) M_D(nexp)
    M_D(Qgbs) M_D(Vgbs) M_D(ngbs) M_D(mgbs) M_D(Agbs) M_D(agbs) M_D(fgbs) M_D(rgbs) M_D(Fgbs)
    M_I(cstv) M_I(pwlv) M_I(linv) M_I(expv) M_I(gbsv) M_I(gs) M_I(is_tensile)
    M_I(coh_soft) M_I(phi_soft) M_I(psi_soft)
#undef M_D
#undef M_I
    return -1;
}

/* ------------------------------------------------------------------------ */
/* Grid fields by name: the returned pointer aliases the reference's array.   */
double *ref_field(const char *name) {
#define F(f) if (!strcmp(name, #f)) return g_mesh.f;
    F(u_in) F(v_in) F(p_in) F(p_corr) F(div_u) F(div_u_s) F(exxd) F(ezzd) F(exz) F(exz_n) F(exxd_s) F(ezzd_s)
    F(sxxd) F(szzd) F(sxz) F(sxz_n) F(sxxd0) F(szzd0) F(sxz0) F(sxxd0_s) F(szzd0_s) F(sxz0_n)
    F(eta_n) F(eta_s) F(eta_phys_n) F(eta_phys_s) F(VE_n) F(VE_s) F(mu_n) F(mu_s) F(T) F(T_s) F(P_s)
    F(d0_n) F(d0_s) F(phi0_n) F(phi0_s) F(X0_n) F(X0_s) F(strain_n) F(strain_s) F(p0_n) F(p0_s)
    F(bet_n) F(bet_s) F(rho_n) F(rho_s) F(C_n) F(C_s) F(fric_n) F(fric_s) F(dil_n) F(dil_s)
    F(eII_el) F(eII_pl) F(eII_pwl) F(eII_lin) F(eII_cst) F(eII_exp) F(eII_gbs) F(exx_el) F(ezz_el) F(exz_el) F(exx_diss) F(ezz_diss) F(exz_diss)
    F(d_n) F(OverS_n) F(OverS_s) F(X_n) F(X_s) F(div_u_el) F(div_u_pl) F(div_u_r) F(Wtot) F(Wel) F(Wdiss)
    F(D11_n) F(D12_n) F(D13_n) F(D14_n) F(D21_n) F(D22_n) F(D23_n) F(D24_n) F(D31_s) F(D32_s) F(D33_s) F(D34_s)
    F(detadexx_n) F(detadezz_n) F(detadgxz_n) F(detadp_n) F(ddivpdexx_n) F(ddivpdezz_n) F(ddivpdgxz_n) F(ddivpdp_n)
    F(detadexx_s) F(detadezz_s) F(detadgxz_s) F(detadp_s)
    F(roger_x) F(roger_z) F(rhs_p) F(ru) F(rv) F(rp) F(gx) F(gz)
    F(xg_coord) F(zg_coord) F(xc_coord) F(zc_coord) F(xvz_coord) F(zvx_coord) F(dp) F(p_lith) F(p_lith0)
    F(kx) F(kz) F(Cv) F(Qr) F(dT) F(alp)
#undef F
    if (!strcmp(name, "BCu_val")) return g_mesh.BCu.val;
    if (!strcmp(name, "BCv_val")) return g_mesh.BCv.val;
    return NULL;
}

char *ref_tags(const char *name) {
    if (!strcmp(name, "BCu")) return g_mesh.BCu.type;
    if (!strcmp(name, "BCv")) return g_mesh.BCv.type;
    if (!strcmp(name, "BCp")) return g_mesh.BCp.type;
    if (!strcmp(name, "BCg")) return g_mesh.BCg.type;
    return NULL;
}

double *ref_phase_perc(int centroid, int p) {
    return centroid ? g_mesh.phase_perc_n[p] : g_mesh.phase_perc_s[p];
}
int *ref_count_array(int centroid) { return centroid ? g_mesh.nb_part_cell : g_mesh.nb_part_vert; }
double ref_dx(void) { return g_mesh.dx; }
double ref_dz(void) { return g_mesh.dz; }

/* ------------------------------------------------------------------------ */
int ref_set_markers(int n, const double *x, const double *z, const int *phase) {
    if (g_have_parts) PartFree(&g_parts, &g_model);
    memset(&g_parts, 0, sizeof g_parts);
    g_parts.Nb_part = n; g_parts.Nb_part_max = n > 0 ? n : 1;
    PartAlloc(&g_parts, &g_model);
    memcpy(g_parts.x, x, sizeof(double) * n);
    memcpy(g_parts.z, z, sizeof(double) * n);
    memcpy(g_parts.phase, phase, sizeof(int) * n);
    g_have_parts = 1;
    return 0;
}

/* Markers with room for cap of them (reseeding writes new markers up to cap). */
int ref_set_markers_cap(int n, int cap, const double *x, const double *z, const int *phase) {
    if (g_have_parts) PartFree(&g_parts, &g_model);
    memset(&g_parts, 0, sizeof g_parts);
    g_parts.Nb_part = n; g_parts.Nb_part_max = cap > n ? cap : (n > 0 ? n : 1);
    PartAlloc(&g_parts, &g_model);
    memcpy(g_parts.x, x, sizeof(double) * n);
    memcpy(g_parts.z, z, sizeof(double) * n);
    memcpy(g_parts.phase, phase, sizeof(int) * n);
    g_have_parts = 1;
    return 0;
}

/* CountPartCell with RESEED = 1 on ONE OpenMP thread: the reference splits the
 * domain into per-thread x-slabs whose overlap decides which markers a new one
 * may copy from, so only the one-thread result is thread-count independent.
 * No free surface, no sedimentation, no finite strain / P-T recording /
 * anisotropy.  Returns the new Nb_part. */
int ref_reseed(int direct_neighbour, int min_part_cell) {
    surface topo, topo_ini;
    memset(&topo, 0, sizeof topo);
    memset(&topo_ini, 0, sizeof topo_ini);
    g_model.DirectNeighbour = direct_neighbour;
    g_model.free_surf = 0; g_model.surf_processes = 0; g_model.fstrain = 0; g_model.rec_T_P_x_z = 0;
    g_model.aniso = 0; g_model.isperiodic_x = 0;
    g_parts.min_part_cell = min_part_cell;
    const int nt = omp_get_max_threads();
    omp_set_num_threads(1);
    CountPartCell(&g_parts, &g_mesh, g_model, topo, topo_ini, 1, g_scale);
    omp_set_num_threads(nt);
    return g_parts.Nb_part;
}

double *ref_marker_field(const char *name) {
#define F(f) if (!strcmp(name, #f)) return g_parts.f;
    F(x) F(z) F(Vx) F(Vz) F(P) F(sxxd) F(szzd) F(sxz) F(strain) F(strain_pl) F(T) F(d) F(phi) F(X)
#undef F
    return NULL;
}
int *ref_marker_phase(void) { return g_parts.phase; }

static char *node_tags(int centroid) {
    if (centroid == 1) return g_mesh.BCp.type;
    if (centroid == 0) return g_mesh.BCg.type;
    if (centroid == -1) return g_mesh.BCu.type;
    return g_mesh.BCv.type;
}

/* P2Mastah with a per-phase (flag 0) or per-marker (flag 1) property. */
int ref_p2g(const double *prop_values, double *out, int flag, int avg, int prop, int centroid, int itp_stencil) {
    P2Mastah(&g_model, g_parts, (DoodzFP *)prop_values, &g_mesh, out, node_tags(centroid), flag, avg, prop, centroid,
             itp_stencil);
    return 0;
}

int ref_count_old(void) {
    surface topo;
    memset(&topo, 0, sizeof topo);
    CountPartCell_Old(&g_parts, &g_mesh, g_model, topo, 0, g_scale);
    return 0;
}

/* Grid -> marker, vertex-type node set (Interp_Grid2P) or extended-centroid frame
 * (Interp_Grid2P_centroids2).  which: 0 vertices, 1 centroids (extended frame). */
int ref_g2p(double *node_field, double *out, int which) {
    int Nx = g_mesh.Nx, Nz = g_mesh.Nz;
    if (which == 0)
        Interp_Grid2P(g_parts, out, &g_mesh, node_field, g_mesh.xg_coord, g_mesh.zg_coord, Nx, Nz, g_mesh.BCg.type);
    else
        Interp_Grid2P_centroids2(g_parts, out, &g_mesh, node_field, g_mesh.xvz_coord, g_mesh.zvx_coord, Nx - 1, Nz - 1,
                                 g_mesh.BCp.type, &g_model);
    return 0;
}

int ref_rk4(void) {
    RogerGuntherII(&g_parts, g_model, g_mesh, 0, g_scale);
    return 0;
}

/* Scaling factors by name (the breakpoint writer and loader scale with them). */
int ref_set_scale(const char *name, double v) {
#define S_D(f) if (!strcmp(name, #f)) { g_scale.f = v; return 0; }
    S_D(L) S_D(V) S_D(S) S_D(T) S_D(t) S_D(E) S_D(rho) S_D(eta) S_D(rhoE)
#undef S_D
    return -1;
}

/* MakeBreakpointParticles (SOURCE/InputOutput.c:515-903) of the harness state
 * into BreakpointXXXXX.dat in the working directory (delete_breakpoints = -1;
 * no free surface, so the topography arguments are not read). */
int ref_make_breakpoint(void) {
    markers chain, chain_ini;
    surface topo, topo_ini;
    memset(&chain, 0, sizeof chain); memset(&chain_ini, 0, sizeof chain_ini);
    memset(&topo, 0, sizeof topo); memset(&topo_ini, 0, sizeof topo_ini);
    if (!g_have_grid || !g_have_parts) return -1;
    g_model.delete_breakpoints = -1;
    MakeBreakpointParticles(&g_parts, &g_mesh, &chain, &chain_ini, g_model, &topo, &topo_ini, g_scale);
    return 0;
}

/* LoadBreakpointParticles (SOURCE/InputOutput.c:160-514) of BreakpointXXXXX.dat
 * into the harness state; returns the loaded Nb_part. */
int ref_load_breakpoint(void) {
    markers chain, chain_ini;
    surface topo, topo_ini;
    memset(&chain, 0, sizeof chain); memset(&chain_ini, 0, sizeof chain_ini);
    memset(&topo, 0, sizeof topo); memset(&topo_ini, 0, sizeof topo_ini);
    if (!g_have_grid || !g_have_parts) return -1;
    g_model.delete_breakpoints = -1;
    LoadBreakpointParticles(&g_parts, &g_mesh, &chain, &chain_ini, &g_model, &topo, &topo_ini, g_scale);
    return g_parts.Nb_part;
}

/* Model scalars the breakpoint loader sets. */
double ref_get_model(const char *name) {
    if (!strcmp(name, "dt")) return g_model.dt;
    if (!strcmp(name, "time")) return g_model.time;
    if (!strcmp(name, "xmin")) return g_model.xmin;
    if (!strcmp(name, "xmax")) return g_model.xmax;
    if (!strcmp(name, "zmin")) return g_model.zmin;
    if (!strcmp(name, "zmax")) return g_model.zmax;
    return 0.0;
}

/* Closest-marker phase map on the visualisation grid of res_fact times the
 * computational resolution, built and filled as WriteOutputHDF5 does
 * (HDF5Output.c:266-297: lines by accumulation from the first grid line,
 * Interp_Phase2VizGrid); compo holds (nxviz-1)*(nzviz-1) chars, xviz / zviz
 * the nxviz / nzviz lines. */
int ref_phase_viz(int res_fact, char *compo, double *xviz, double *zviz) {
    const int nxviz = res_fact * (g_mesh.Nx - 1) + 1, nzviz = res_fact * (g_mesh.Nz - 1) + 1;
    xviz[0] = g_mesh.xg_coord[0];
    zviz[0] = g_mesh.zg_coord[0];
    for (int k = 1; k < nxviz; k++) xviz[k] = xviz[k - 1] + g_mesh.dx / res_fact;
    for (int k = 1; k < nzviz; k++) zviz[k] = zviz[k - 1] + g_mesh.dz / res_fact;
    surface topo;
    memset(&topo, 0, sizeof topo);
    Interp_Phase2VizGrid(g_parts, g_parts.phase, &g_mesh, compo, xviz, zviz, nxviz, nzviz, g_model, topo);
    return 0;
}

/* ------------------------------------------------------------------------ */
int ref_strain_rates(void) { StrainRateComponents(&g_mesh, g_scale, &g_model); return 0; }
int ref_viscosity_grid(void) { NonNewtonianViscosityGrid(&g_mesh, &g_mat, &g_model, g_nmodel, &g_scale); return 0; }
int ref_rheo_operators(int jacobian) { RheologicalOperators(&g_mesh, &g_model, &g_scale, jacobian); return 0; }
int ref_rhs(void) { EvaluateRHS(&g_mesh, g_model, g_scale, g_mat.rho[0]); return 0; }
int ref_accumulated_strain(void) {
    AccumulatedStrainII(&g_mesh, g_scale, g_model, &g_parts, g_mesh.xc_coord, g_mesh.zc_coord, g_mesh.Nx - 1,
                        g_mesh.Nz - 1, g_mesh.BCp.type);
    return 0;
}
int ref_update_particle_stress(void) { UpdateParticleStress(&g_mesh, &g_parts, &g_model, &g_mat, &g_scale); return 0; }
/* ShearModCompExpGrid and CohesionFrictionDilationGrid from the phase
 * fractions already on the grid and the markers' strain_pl. */
int ref_shear_mod_grid(void) { ShearModCompExpGrid(&g_mesh, g_mat, g_model, g_scale); return 0; }
int ref_cohesion_grid(void) { CohesionFrictionDilationGrid(&g_mesh, &g_parts, g_mat, g_model, g_scale); return 0; }
/* UpdateParticlePressure (no subgrid diffusion when subgrid_diff < 2) from
 * p_in, p0_n and, with Plith_trick = 1, p_lith and p_lith0. */
int ref_update_particle_pressure(void) { UpdateParticlePressure(&g_mesh, g_scale, g_model, &g_parts, &g_mat); return 0; }

static void free_blocks(SparseMat *A, SparseMat *B, SparseMat *C, SparseMat *D) {
    FreeMat(A); FreeMat(B); FreeMat(C); FreeMat(D);
}

int ref_setup_equations(void) {
    if (g_have_eqn) return 0;
    EvalNumberOfEquations(&g_mesh, &g_S);
    SAlloc(&g_S, g_S.neq);
    g_SA.neq = g_SB.neq = g_S.neq_mom; g_SC.neq = g_SD.neq = g_S.neq_cont;
    SAlloc(&g_SA, g_S.neq_mom); SAlloc(&g_SB, g_S.neq_mom); SAlloc(&g_SC, g_S.neq_cont); SAlloc(&g_SD, g_S.neq_cont);
    g_J = g_S;
    g_JA.neq = g_JB.neq = g_S.neq_mom; g_JC.neq = g_JD.neq = g_S.neq_cont;
    SAlloc(&g_JA, g_S.neq_mom); SAlloc(&g_JB, g_S.neq_mom); SAlloc(&g_JC, g_S.neq_cont); SAlloc(&g_JD, g_S.neq_cont);
    g_have_eqn = 1;
    return 0;
}

int ref_neq(int which) { return which == 0 ? g_S.neq_mom : (which == 1 ? g_S.neq_cont : g_S.neq); }
int *ref_eqn(int which) { return which == 0 ? g_S.eqn_u : (which == 1 ? g_S.eqn_v : g_S.eqn_p); }

/* Non-linear residual in the reference's decoupled form (momentum F of length
 * neq_mom, continuity F of length neq_cont) plus its three norms. */
int ref_residual(double *norms3) {
    ref_setup_equations();
    g_nmodel.nit = 0;
    EvaluateStokesResidualDecoupled(&g_S, &g_SA, &g_SB, &g_SC, &g_SD, &g_nmodel, &g_mesh, g_model, g_scale, 1);
    norms3[0] = g_nmodel.resx; norms3[1] = g_nmodel.resz; norms3[2] = g_nmodel.resp;
    return 0;
}
double *ref_residual_vec(int which) { return which == 0 ? g_SA.F : g_SC.F; }
double *ref_rhs_vec(int which) { return which == 0 ? g_SA.b : g_SC.b; }

/* Assemble the Picard blocks (jacobian = 0) or the Newton Jacobian blocks
 * (jacobian = 1); blocks are then read with ref_block(). */
int ref_assemble(int jacobian) {
    ref_setup_equations();
    if (!jacobian) {
        if (g_have_picard) free_blocks(&g_SA, &g_SB, &g_SC, &g_SD);
        BuildStokesOperatorDecoupled(&g_mesh, g_model, 0, g_mesh.p_corr, g_mesh.p_in, g_mesh.u_in, g_mesh.v_in, &g_S,
                                     &g_SA, &g_SB, &g_SC, &g_SD, 1);
        g_have_picard = 1;
    } else {
        if (g_have_jac) free_blocks(&g_JA, &g_JB, &g_JC, &g_JD);
        BuildJacobianOperatorDecoupled(&g_mesh, g_model, 0, g_mesh.p_corr, g_mesh.p_in, g_mesh.u_in, g_mesh.v_in, &g_J,
                                       &g_JA, &g_JB, &g_JC, &g_JD, 1);
        g_have_jac = 1;
    }
    return 0;
}

/* CSR of block b (0 A=uu, 1 B=up, 2 C=pu, 3 D=pp) of the Picard (0) or
 * Jacobian (1) operator: row pointer (neq+1), columns and values. */
int ref_block(int jacobian, int b, int **Ic, int **J, double **A, double **bbc) {
    SparseMat *M = jacobian ? (b == 0 ? &g_JA : b == 1 ? &g_JB : b == 2 ? &g_JC : &g_JD)
                            : (b == 0 ? &g_SA : b == 1 ? &g_SB : b == 2 ? &g_SC : &g_SD);
    *Ic = M->Ic; *J = M->J; *A = M->A; *bbc = M->bbc;
    return M->neq;
}


/* ------------------------------------------------------------------------ */
/* Energy equation.  ThermalSolver.c (the CHOLMOD factorisation and solve of
 * EnergyDirectSolve) is not built; these stand-ins keep a copy of the matrix
 * the reference assembled and of its right-hand side, and solve the system by
 * dense Gaussian elimination with partial pivoting (fixture sizes, a few
 * hundred unknowns), so that EnergyDirectSolve runs to its end.  Test
 * infrastructure only. */
static int g_en_n = 0, g_en_nnz = 0;
static int *g_en_ia = NULL, *g_en_ja = NULL;
static double *g_en_a = NULL, *g_en_b = NULL, *g_en_x = NULL;
static cholmod_factor g_en_factor;

int cholmod_start(cholmod_common *c) { (void)c; return 1; }
int cholmod_finish(cholmod_common *c) { (void)c; return 1; }
int cholmod_free_factor(cholmod_factor **f, cholmod_common *c) { (void)f; (void)c; return 1; }
cs_di *cs_spfree(cs_di *A) { (void)A; return NULL; }
cs_di *TransposeA(cholmod_common *c, double *A, int *Ic, int *J, int neq, int nnz) {
    (void)c; (void)A; (void)Ic; (void)J; (void)neq; (void)nnz;
    return NULL;   /* used by the polar mode only */
}

cholmod_factor *FactorEnergyCHOLMOD(cholmod_common *c, cs_di *At, double *a, int *ia, int *ja, int n, int nnz,
                                    int polar_mode) {
    (void)c; (void)At; (void)polar_mode;
    free(g_en_ia); free(g_en_ja); free(g_en_a);
    g_en_n = n; g_en_nnz = nnz;
    g_en_ia = malloc(sizeof(int) * (n + 1));
    g_en_ja = malloc(sizeof(int) * (nnz > 0 ? nnz : 1));
    g_en_a = malloc(sizeof(double) * (nnz > 0 ? nnz : 1));
    memcpy(g_en_ia, ia, sizeof(int) * (n + 1));
    memcpy(g_en_ja, ja, sizeof(int) * nnz);
    memcpy(g_en_a, a, sizeof(double) * nnz);
    return &g_en_factor;
}

void SolveEnergyCHOLMOD(cholmod_common *c, cs_di *At, cholmod_factor *F, double *x, double *b, int n, int nnz,
                        int polar_mode) {
    (void)c; (void)At; (void)F; (void)nnz; (void)polar_mode;
    int i, j, k;
    free(g_en_b); free(g_en_x);
    g_en_b = malloc(sizeof(double) * n);
    g_en_x = malloc(sizeof(double) * n);
    memcpy(g_en_b, b, sizeof(double) * n);
    double *M = calloc((size_t)n * (n + 1), sizeof(double));
    for (i = 0; i < n; i++) {
        for (k = g_en_ia[i]; k < g_en_ia[i + 1]; k++) M[(size_t)i * (n + 1) + g_en_ja[k]] += g_en_a[k];
        M[(size_t)i * (n + 1) + n] = b[i];
    }
    for (j = 0; j < n; j++) {
        int piv = j;
        for (i = j + 1; i < n; i++)
            if (fabs(M[(size_t)i * (n + 1) + j]) > fabs(M[(size_t)piv * (n + 1) + j])) piv = i;
        if (piv != j)
            for (k = 0; k <= n; k++) {
                double t = M[(size_t)j * (n + 1) + k];
                M[(size_t)j * (n + 1) + k] = M[(size_t)piv * (n + 1) + k];
                M[(size_t)piv * (n + 1) + k] = t;
            }
        for (i = j + 1; i < n; i++) {
            double f = M[(size_t)i * (n + 1) + j] / M[(size_t)j * (n + 1) + j];
            if (f == 0.0) continue;
            for (k = j; k <= n; k++) M[(size_t)i * (n + 1) + k] -= f * M[(size_t)j * (n + 1) + k];
        }
    }
    for (i = n - 1; i >= 0; i--) {
        double s = M[(size_t)i * (n + 1) + n];
        for (k = i + 1; k < n; k++) s -= M[(size_t)i * (n + 1) + k] * x[k];
        x[i] = s / M[(size_t)i * (n + 1) + i];
    }
    memcpy(g_en_x, x, sizeof(double) * n);
    free(M);
}

/* One implicit energy step (EnergyDirectSolve, ThermalRoutines.c:72-551,
 * nit = 1) on the harness grid: mesh T, rho_n, Cv, Qr, kx, kz, Wdiss, alp,
 * BCt. */
int ref_energy_solve(double dt, int shear_heating, int adiab_heating) {
    EnergyDirectSolve(&g_mesh, g_model, g_mesh.T, g_mesh.dT, NULL, g_mesh.T, &g_parts, dt, shear_heating,
                      adiab_heating, g_scale, 1);
    return 0;
}

/* The last assembled energy system: n rows, CSR (ia, ja, a), right-hand side
 * b (b + bbc as solved) and solution x. */
int ref_energy_system(int **ia, int **ja, double **a, double **b, double **x) {
    *ia = g_en_ia; *ja = g_en_ja; *a = g_en_a; *b = g_en_b; *x = g_en_x;
    return g_en_n;
}

/* Thermal boundary arrays (BCT BCt): tags "type" (centroids), "typW",
 * "typE" (Nz-1), "typS", "typN" (Nx-1); values "valW" ... "valN". */
char *ref_bct_tags(const char *name) {
    if (!strcmp(name, "type")) return g_mesh.BCt.type;
    if (!strcmp(name, "typW")) return g_mesh.BCt.typW;
    if (!strcmp(name, "typE")) return g_mesh.BCt.typE;
    if (!strcmp(name, "typS")) return g_mesh.BCt.typS;
    if (!strcmp(name, "typN")) return g_mesh.BCt.typN;
    return NULL;
}
double *ref_bct_vals(const char *name) {
    if (!strcmp(name, "valW")) return g_mesh.BCt.valW;
    if (!strcmp(name, "valE")) return g_mesh.BCt.valE;
    if (!strcmp(name, "valS")) return g_mesh.BCt.valS;
    if (!strcmp(name, "valN")) return g_mesh.BCt.valN;
    return NULL;
}
