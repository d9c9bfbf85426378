/*
 * Reference-signature drop-ins: the MDOODZ 6.0 functions of the per-time-step
 * path, with the names and argument lists of SOURCE/header_MDOODZ.h, each
 * computed on the GPU through the library's C ABI (include/mdoodz_gpu.h).  A
 * reference build links this file (and libmdoodz_gb300.so) in place of the
 * reference's own definitions of these functions; Main_DOODZ.c and the
 * reference's structures stay as they are.
 *
 *   P2Mastah                      SOURCE/header_MDOODZ.h:345
 *   CountPartCell                 :430
 *   StrainRateComponents          :417
 *   NonNewtonianViscosityGrid     :416
 *   RheologicalOperators          :580
 *   UpdateNonLinearity            :414
 *   BuildStokesOperatorDecoupled  :474
 *   BuildJacobianOperatorDecoupled:491
 *   EvaluateStokesResidualDecoupled:473
 *   SolveStokesDefectDecoupled    :476
 *   LineSearchDecoupled           :472
 *   Interp_Grid2P                 :340
 *   Interp_Grid2P_centroids2      :592
 *   RogerGuntherII                :567
 *   UpdateParticleStress          :409
 *   AccumulatedStrainII           :568
 * plus mdz_gpu_init / mdz_gpu_finalize / mdz_gpu_last_status /
 * mdz_gpu_sync_to_host (include/mdoodz_refshim.h).
 *
 * Compiled against the reference's header (-DMDZ_WITH_REFERENCE_HEADER and its
 * include path) in a reference build, or against include/mdoodz_ref_types.h,
 * the generated layout view of the same structures.
 *
 * State: one library context for the grid given to mdz_gpu_init (or to the
 * first drop-in called), kept until mdz_gpu_finalize.  The markers are the
 * caller's: each call that reads them uploads positions and phases (and the
 * attributes it updates) and writes back what the reference function writes.
 * Matrix-free: the Build*Operator*(Assemble = 1) calls assemble nothing and
 * only record which operator the next defect solve uses; the CSR blocks of the
 * SparseMat arguments are never read.  Errors: the reference prints and
 * exit()s; these print the library's message and exit(1) at the same points,
 * and mdz_gpu_last_status() gives the last status.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "mdoodz_gpu.h"
#ifdef MDZ_WITH_REFERENCE_HEADER
#include "header_MDOODZ.h"
#else
#include "mdoodz_ref_types.h"
#endif
#include "mdoodz_refshim.h"

/* BC tags are plain char in the reference's structures: signed on x86-64,
 * unsigned on AArch64, so every comparison reads them as signed char. */
#define TAG(t) ((signed char)(t))

static mdz_ctx *g_ctx = NULL;
static mdz_grid_desc g_desc;         /* the grid of the context (the caller's arrays) */
static int g_nph = 0;
static long long g_cap = 0;
static int g_status = 0;
static int g_jacobian = 0;           /* operator of the next defect solve (Build*Operator*) */
static int g_precision = 64;         /* MDZ_REFSHIM_PRECISION = 32: FP32-refined defect solves */
static double *g_pp = NULL;          /* contiguous phase fractions (n_phases x nodes) */
static size_t g_pp_n = 0;

static void check(mdz_status s, const char *where) {
    g_status = (int)s;
    if (s == MDZ_OK) return;
    fprintf(stderr, "%s (GPU): %s\n", where, g_ctx ? mdz_last_error(g_ctx) : "no context");
    exit(1);
}

static double *pp_buffer(size_t n) {
    if (n > g_pp_n) {
        free(g_pp);
        g_pp = (double *)malloc(sizeof(double) * n);
        if (!g_pp) { fprintf(stderr, "mdz_refshim: out of host memory\n"); exit(1); }
        g_pp_n = n;
    }
    return g_pp;
}

int mdz_gpu_init(const params *model, const grid *mesh, const markers *particles) {
    if (g_ctx) return 0;
    if (!model || !mesh) return (int)MDZ_ERR_ARG;
    mdz_grid_desc d;
    memset(&d, 0, sizeof d);
    d.Nx = mesh->Nx; d.Nz = mesh->Nz; d.dx = mesh->dx; d.dz = mesh->dz;
    d.xmin = model->xmin; d.xmax = model->xmax; d.zmin = model->zmin; d.zmax = model->zmax;
    d.xg = mesh->xg_coord; d.zg = mesh->zg_coord; d.xc = mesh->xc_coord; d.zc = mesh->zc_coord;
    d.xvz = mesh->xvz_coord; d.zvx = mesh->zvx_coord;
    d.BCu_type = (const signed char *)mesh->BCu.type; d.BCv_type = (const signed char *)mesh->BCv.type;
    d.BCp_type = (const signed char *)mesh->BCp.type; d.BCg_type = (const signed char *)mesh->BCg.type;
    d.BCu_val = mesh->BCu.val; d.BCv_val = mesh->BCv.val;
    d.isperiodic_x = model->isperiodic_x;
    const char *prec = getenv("MDZ_REFSHIM_PRECISION");
    g_precision = prec && atoi(prec) == 32 ? 32 : 64;
    long long cap = particles ? (particles->Nb_part_max > particles->Nb_part ? particles->Nb_part_max
                                                                              : particles->Nb_part) : 1;
    g_status = (int)mdz_create(&g_ctx, &d, model->Nb_phases, cap);
    if (g_status == 0) { g_desc = d; g_nph = model->Nb_phases; g_cap = cap; }
    return g_status;
}

void mdz_gpu_finalize(void) {
    if (g_ctx) mdz_destroy(g_ctx);
    g_ctx = NULL;
    free(g_pp);
    g_pp = NULL;
    g_pp_n = 0;
}

int mdz_gpu_last_status(void) { return g_status; }

int mdz_gpu_sync_to_host(unsigned int fieldmask) {
    (void)fieldmask;   /* every drop-in returns with its outputs in the caller's arrays */
    return g_ctx ? (int)mdz_sync(g_ctx) : 0;
}

static void ensure(const params *model, const grid *mesh, const markers *particles) {
    if (!g_ctx && mdz_gpu_init(model, mesh, particles) != 0) {
        fprintf(stderr, "mdz_refshim: no usable GPU context (status %d)%s\n", g_status,
                model ? "" : ": call mdz_gpu_init first");
        exit(1);
    }
}

/* a context with room for n markers: a larger marker set than the context was
 * made for replaces it (the drop-ins keep no device state between calls that
 * the next call does not upload again) */
static void ensure_capacity(long long n) {
    if (n <= g_cap) return;
    mdz_destroy(g_ctx);
    g_ctx = NULL;
    long long cap = 2 * n;
    g_status = (int)mdz_create(&g_ctx, &g_desc, g_nph, cap);
    if (g_status != 0) { fprintf(stderr, "mdz_refshim: context for %lld markers refused\n", cap); exit(1); }
    g_cap = cap;
}

static void put_markers(const markers *p) {
    ensure_capacity(p->Nb_part_max > p->Nb_part ? p->Nb_part_max : p->Nb_part);
    check(mdz_set_markers(g_ctx, p->Nb_part, p->x, p->z, p->phase), "markers");
}

static void put_attrs(const markers *p, int with_strain, int with_stress, int with_P) {
    const int n = p->Nb_part;
    if (with_stress) {
        check(mdz_set_marker_attr(g_ctx, MDZ_M_SXXD, n, p->sxxd), "markers");
        check(mdz_set_marker_attr(g_ctx, MDZ_M_SZZD, n, p->szzd), "markers");
        check(mdz_set_marker_attr(g_ctx, MDZ_M_SXZ, n, p->sxz), "markers");
    }
    if (with_strain) {
        check(mdz_set_marker_attr(g_ctx, MDZ_M_STRAIN, n, p->strain), "markers");
        check(mdz_set_marker_attr(g_ctx, MDZ_M_STRAIN_PL, n, p->strain_pl), "markers");
    }
    if (with_P && p->P) check(mdz_set_marker_attr(g_ctx, MDZ_M_P, n, p->P), "markers");
}

static void get_attr(int attr, int n, double *dst) {
    if (dst) check(mdz_get_marker_attr(g_ctx, attr, n, dst), "markers");
}

/* ---- marker -> grid ------------------------------------------------------ */

void P2Mastah(params *model, markers particles, DoodzFP *mat_prop, grid *mesh, double *NodeField, char *NodeType,
              int flag, int avg, int prop, int centroid, int itp_stencil) {
    ensure(model, mesh, &particles);
    put_markers(&particles);
    const int nph = model->Nb_phases;
    if (prop == 1) {
        const size_t nn = centroid == 1 ? (size_t)(mesh->Nx - 1) * (mesh->Nz - 1) : (size_t)mesh->Nx * mesh->Nz;
        double *pp = pp_buffer(nn * (size_t)nph);
        check(mdz_P2Mastah(g_ctx, mat_prop, NodeField, (const signed char *)NodeType, flag, avg, 1, centroid,
                           itp_stencil, pp), "P2Mastah");
        double **dst = centroid == 1 ? mesh->phase_perc_n : mesh->phase_perc_s;
        for (int p = 0; p < nph; p++) memcpy(dst[p], pp + (size_t)p * nn, sizeof(double) * nn);
        return;
    }
    check(mdz_P2Mastah(g_ctx, mat_prop, NodeField, (const signed char *)NodeType, flag, avg, 0, centroid,
                       itp_stencil, NULL), "P2Mastah");
}

/* CountPartCell with RESEED = 1: reseeding of the caller's markers (their
 * count grows; the new markers are written into the caller's arrays).  With
 * RESEED = 0: the per-cell and per-vertex marker counts. */
void CountPartCell(markers *particles, grid *mesh, params model, surface topo, surface topo_ini, int reseed,
                   scale scaling) {
    (void)topo; (void)topo_ini; (void)scaling;
    ensure(&model, mesh, particles);
    put_markers(particles);
    if (!reseed) {
        check(mdz_count_markers(g_ctx, mesh->nb_part_cell, mesh->nb_part_vert, NULL, NULL), "CountPartCell");
        return;
    }
    check(mdz_set_marker_velocity(g_ctx, particles->Nb_part, particles->Vx, particles->Vz), "CountPartCell");
    put_attrs(particles, 1, 1, 1);
    if (particles->T) check(mdz_set_marker_attr(g_ctx, MDZ_M_T, particles->Nb_part, particles->T), "CountPartCell");
    int added = 0;
    check(mdz_CountPartCell(g_ctx, 1, particles->min_part_cell, model.DirectNeighbour, mesh->T, mesh->sxxd,
                            mesh->szzd, mesh->sxz, mesh->p_in, &added), "CountPartCell");
    const int n = mdz_marker_count(g_ctx);
    check(mdz_get_markers(g_ctx, n, particles->x, particles->z, particles->phase, particles->Vx, particles->Vz),
          "CountPartCell");
    get_attr(MDZ_M_SXXD, n, particles->sxxd);
    get_attr(MDZ_M_SZZD, n, particles->szzd);
    get_attr(MDZ_M_SXZ, n, particles->sxz);
    get_attr(MDZ_M_STRAIN, n, particles->strain);
    get_attr(MDZ_M_STRAIN_PL, n, particles->strain_pl);
    get_attr(MDZ_M_T, n, particles->T);
    get_attr(MDZ_M_P, n, particles->P);
    particles->Nb_part = n;
}

/* ---- grid fields --------------------------------------------------------- */

/* The library's field view of the caller's grid: every member names the
 * reference array of the same meaning (u, v, p are u_in, v_in, p_in).  The
 * phase fractions are contiguous copies (the reference keeps one array per
 * phase). */
static void fields_of(grid *m, mdz_fields *f, int nph, int with_pp) {
    memset(f, 0, sizeof *f);
    f->u = m->u_in; f->v = m->v_in; f->p = m->p_in; f->p_corr = m->p_corr;
    f->div_u = m->div_u; f->div_u_s = m->div_u_s; f->exxd = m->exxd; f->ezzd = m->ezzd; f->exz = m->exz;
    f->exz_n = m->exz_n; f->exxd_s = m->exxd_s; f->ezzd_s = m->ezzd_s;
    f->sxxd0 = m->sxxd0; f->szzd0 = m->szzd0; f->sxz0 = m->sxz0; f->sxxd0_s = m->sxxd0_s; f->szzd0_s = m->szzd0_s;
    f->sxz0_n = m->sxz0_n; f->mu_n = m->mu_n; f->mu_s = m->mu_s; f->T = m->T; f->T_s = m->T_s; f->P_s = m->P_s;
    f->d0_n = m->d0_n; f->d0_s = m->d0_s; f->phi0_n = m->phi0_n; f->phi0_s = m->phi0_s; f->X0_n = m->X0_n;
    f->X0_s = m->X0_s; f->strain_n = m->strain_n; f->strain_s = m->strain_s; f->dil_n = m->dil_n;
    f->dil_s = m->dil_s; f->fric_n = m->fric_n; f->fric_s = m->fric_s; f->C_n = m->C_n; f->C_s = m->C_s;
    f->p0_n = m->p0_n; f->p0_s = m->p0_s; f->bet_n = m->bet_n; f->bet_s = m->bet_s; f->rho_n = m->rho_n;
    f->rho_s = m->rho_s; f->eta_n = m->eta_n; f->eta_s = m->eta_s; f->eta_phys_n = m->eta_phys_n;
    f->eta_phys_s = m->eta_phys_s; f->VE_n = m->VE_n; f->VE_s = m->VE_s; f->sxxd = m->sxxd; f->szzd = m->szzd;
    f->sxz = m->sxz; f->sxz_n = m->sxz_n; f->eII_el = m->eII_el; f->eII_pl = m->eII_pl; f->eII_pwl = m->eII_pwl;
    f->eII_exp = m->eII_exp; f->eII_gbs = m->eII_gbs;
    f->eII_lin = m->eII_lin; f->eII_cst = m->eII_cst; f->d_n = m->d_n; f->exx_el = m->exx_el;
    f->ezz_el = m->ezz_el; f->exz_el = m->exz_el; f->exx_diss = m->exx_diss; f->ezz_diss = m->ezz_diss;
    f->exz_diss = m->exz_diss; f->detadexx_n = m->detadexx_n; f->detadezz_n = m->detadezz_n;
    f->detadgxz_n = m->detadgxz_n; f->detadp_n = m->detadp_n; f->ddivpdexx_n = m->ddivpdexx_n;
    f->ddivpdezz_n = m->ddivpdezz_n; f->ddivpdgxz_n = m->ddivpdgxz_n; f->ddivpdp_n = m->ddivpdp_n;
    f->detadexx_s = m->detadexx_s; f->detadezz_s = m->detadezz_s; f->detadgxz_s = m->detadgxz_s;
    f->detadp_s = m->detadp_s; f->div_u_el = m->div_u_el; f->div_u_pl = m->div_u_pl; f->div_u_r = m->div_u_r;
    f->Wtot = m->Wtot; f->Wel = m->Wel; f->Wdiss = m->Wdiss; f->X_n = m->X_n; f->X_s = m->X_s;
    f->OverS_n = m->OverS_n; f->OverS_s = m->OverS_s;
    f->D11_n = m->D11_n; f->D12_n = m->D12_n; f->D13_n = m->D13_n; f->D14_n = m->D14_n;
    f->D21_n = m->D21_n; f->D22_n = m->D22_n; f->D23_n = m->D23_n; f->D24_n = m->D24_n;
    f->D31_s = m->D31_s; f->D32_s = m->D32_s; f->D33_s = m->D33_s; f->D34_s = m->D34_s;
    f->roger_x = m->roger_x; f->roger_z = m->roger_z; f->rhs_p = m->rhs_p; f->gx = m->gx; f->gz = m->gz;
    f->ru = m->ru; f->rv = m->rv; f->rp = m->rp;
    if (with_pp) {
        const size_t nc = (size_t)(m->Nx - 1) * (m->Nz - 1), nv = (size_t)m->Nx * m->Nz;
        double *pp = pp_buffer((nc + nv) * (size_t)nph);
        for (int p = 0; p < nph; p++) {
            memcpy(pp + (size_t)p * nc, m->phase_perc_n[p], sizeof(double) * nc);
            memcpy(pp + (size_t)nph * nc + (size_t)p * nv, m->phase_perc_s[p], sizeof(double) * nv);
        }
        f->phase_perc_n = pp;
        f->phase_perc_s = pp + (size_t)nph * nc;
    }
}

/* Only the members named stay set (mdz_sync-style uploads copy every non-NULL
 * member, so each drop-in passes exactly the arrays its reference function
 * reads or writes). */
static void keep_only(mdz_fields *f, const char *names) {
    mdz_fields all = *f;
    memset(f, 0, sizeof *f);
#define KEEP(n) if (strstr(names, " " #n " ")) f->n = all.n;
    KEEP(u) KEEP(v) KEEP(p) KEEP(p_corr) KEEP(div_u) KEEP(div_u_s) KEEP(exxd) KEEP(ezzd) KEEP(exz) KEEP(exz_n)
    KEEP(exxd_s) KEEP(ezzd_s) KEEP(sxxd0) KEEP(szzd0) KEEP(sxz0) KEEP(sxxd0_s) KEEP(szzd0_s) KEEP(sxz0_n) KEEP(mu_n)
    KEEP(mu_s) KEEP(T) KEEP(T_s) KEEP(P_s) KEEP(d0_n) KEEP(d0_s) KEEP(phi0_n) KEEP(phi0_s) KEEP(X0_n) KEEP(X0_s)
    KEEP(strain_n) KEEP(strain_s) KEEP(dil_n) KEEP(dil_s) KEEP(fric_n) KEEP(fric_s) KEEP(C_n) KEEP(C_s) KEEP(p0_n)
    KEEP(p0_s) KEEP(bet_n) KEEP(bet_s) KEEP(rho_n) KEEP(rho_s) KEEP(phase_perc_n) KEEP(phase_perc_s) KEEP(eta_n)
    KEEP(eta_s) KEEP(eta_phys_n) KEEP(eta_phys_s) KEEP(VE_n) KEEP(VE_s) KEEP(sxxd) KEEP(szzd) KEEP(sxz) KEEP(sxz_n)
    KEEP(eII_el) KEEP(eII_pl) KEEP(eII_pwl) KEEP(eII_lin) KEEP(eII_cst) KEEP(eII_exp) KEEP(eII_gbs) KEEP(d_n) KEEP(exx_el) KEEP(ezz_el)
    KEEP(exz_el) KEEP(exx_diss) KEEP(ezz_diss) KEEP(exz_diss) KEEP(detadexx_n) KEEP(detadezz_n) KEEP(detadgxz_n)
    KEEP(detadp_n) KEEP(ddivpdexx_n) KEEP(ddivpdezz_n) KEEP(ddivpdgxz_n) KEEP(ddivpdp_n) KEEP(detadexx_s)
    KEEP(detadezz_s) KEEP(detadgxz_s) KEEP(detadp_s) KEEP(div_u_el) KEEP(div_u_pl) KEEP(div_u_r) KEEP(Wtot)
    KEEP(Wel) KEEP(Wdiss) KEEP(X_n) KEEP(X_s) KEEP(OverS_n) KEEP(OverS_s) KEEP(D11_n) KEEP(D12_n) KEEP(D13_n)
    KEEP(D14_n) KEEP(D21_n) KEEP(D22_n) KEEP(D23_n) KEEP(D24_n) KEEP(D31_s) KEEP(D32_s) KEEP(D33_s) KEEP(D34_s)
    KEEP(roger_x) KEEP(roger_z) KEEP(rhs_p) KEEP(gx) KEEP(gz) KEEP(ru) KEEP(rv) KEEP(rp)
#undef KEEP
}

static void materials_of(const mat_prop *mp, int nph, mdz_materials *m) {
    memset(m, 0, sizeof *m);
    m->n_phases = nph;
    m->R = mp->R;
    for (int p = 0; p < nph && p < MDZ_MAX_PHASES; p++) {
        m->cstv[p] = mp->cstv[p]; m->pwlv[p] = mp->pwlv[p]; m->linv[p] = mp->linv[p]; m->expv[p] = mp->expv[p];
        m->gbsv[p] = mp->gbsv[p]; m->gs[p] = mp->gs[p]; m->is_tensile[p] = mp->is_tensile[p];
        m->reac_soft[p] = mp->reac_soft[p]; m->phase_mix[p] = mp->phase_mix[p];
        m->eta0[p] = mp->eta0[p]; m->rho[p] = mp->rho[p]; m->alp[p] = mp->alp[p]; m->gs_ref[p] = mp->gs_ref[p];
        m->Slim[p] = mp->Slim[p]; m->eta_vp[p] = mp->eta_vp[p]; m->n_vp[p] = mp->n_vp[p];
        m->npwl[p] = mp->npwl[p]; m->Apwl[p] = mp->Apwl[p]; m->Qpwl[p] = mp->Qpwl[p]; m->Vpwl[p] = mp->Vpwl[p];
        m->mpwl[p] = mp->mpwl[p]; m->rpwl[p] = mp->rpwl[p]; m->fpwl[p] = mp->fpwl[p]; m->apwl[p] = mp->apwl[p];
        m->Fpwl[p] = mp->Fpwl[p]; m->pref_pwl[p] = mp->pref_pwl[p];
        m->nlin[p] = mp->nlin[p]; m->Alin[p] = mp->Alin[p]; m->Qlin[p] = mp->Qlin[p]; m->Vlin[p] = mp->Vlin[p];
        m->mlin[p] = mp->mlin[p]; m->rlin[p] = mp->rlin[p]; m->flin[p] = mp->flin[p]; m->alin[p] = mp->alin[p];
        m->Flin[p] = mp->Flin[p];
        m->mu[p] = mp->mu[p]; m->bet[p] = mp->bet[p]; m->C[p] = mp->C[p]; m->phi[p] = mp->phi[p];
        m->psi[p] = mp->psi[p]; m->C_end[p] = mp->C_end[p]; m->phi_end[p] = mp->phi_end[p];
        m->psi_end[p] = mp->psi_end[p]; m->pls_start[p] = mp->pls_start[p]; m->pls_end[p] = mp->pls_end[p];
        m->coh_soft[p] = mp->coh_soft[p]; m->phi_soft[p] = mp->phi_soft[p]; m->psi_soft[p] = mp->psi_soft[p];
        m->Qexp[p] = mp->Qexp[p]; m->Sexp[p] = mp->Sexp[p]; m->Eexp[p] = mp->Eexp[p]; m->Gexp[p] = mp->Gexp[p];
        m->nexp[p] = mp->nexp[p];
        m->ngbs[p] = mp->ngbs[p]; m->Agbs[p] = mp->Agbs[p]; m->Qgbs[p] = mp->Qgbs[p]; m->Vgbs[p] = mp->Vgbs[p];
        m->mgbs[p] = mp->mgbs[p]; m->rgbs[p] = mp->rgbs[p]; m->fgbs[p] = mp->fgbs[p]; m->agbs[p] = mp->agbs[p];
        m->Fgbs[p] = mp->Fgbs[p];
    }
}

static void rheo_of(const params *model, const scale *sc, mdz_rheo_params *r) {
    memset(r, 0, sizeof *r);
    r->dt = model->dt; r->iselastic = model->iselastic; r->step = model->step; r->eta_avg = model->eta_avg;
    r->mineta = model->mineta; r->maxeta = model->maxeta;
    r->scale_T = sc->T; r->scale_E = sc->E; r->scale_S = sc->S; r->scale_eta = sc->eta; r->scale_L = sc->L;
    r->clamp_tangent = 0;   /* the reference's tangent */
}

void StrainRateComponents(grid *mesh, scale scaling, params *model) {
    (void)scaling;
    ensure(model, mesh, NULL);
    mdz_fields f;
    fields_of(mesh, &f, model->Nb_phases, 0);
    keep_only(&f, " u v div_u exxd ezzd exz exz_n exxd_s ezzd_s ");
    check(mdz_StrainRateComponents(g_ctx, &f), "StrainRateComponents");
}

void NonNewtonianViscosityGrid(grid *mesh, mat_prop *materials, params *model, Nparams Nmodel, scale *scaling) {
    (void)Nmodel;
    ensure(model, mesh, NULL);
    mdz_materials m;
    mdz_rheo_params r;
    materials_of(materials, model->Nb_phases, &m);
    rheo_of(model, scaling, &r);
    mdz_fields f;
    fields_of(mesh, &f, model->Nb_phases, 1);
    int not_conv = 0;
    check(mdz_NonNewtonianViscosityGrid(g_ctx, &m, &r, &f, &not_conv), "NonNewtonianViscosityGrid");
    if (not_conv) { fprintf(stderr, "Visco-Elastic iterations failed!\n"); exit(0); }
}

void RheologicalOperators(grid *mesh, params *model, scale *scaling, int Jacobian) {
    ensure(model, mesh, NULL);
    mdz_rheo_params r;
    rheo_of(model, scaling, &r);
    mdz_fields f;
    fields_of(mesh, &f, model->Nb_phases, 0);   /* every field: the tangent reads many of them */
    check(mdz_RheologicalOperators(g_ctx, &r, &f, Jacobian), "RheologicalOperators");
}

static void evaluate_rhs(grid *mesh, params *model, scale *scaling) {
    mdz_rheo_params r;
    rheo_of(model, scaling, &r);
    mdz_fields f;
    fields_of(mesh, &f, model->Nb_phases, 0);
    check(mdz_EvaluateRHS(g_ctx, &r, model->gx, model->gz, &f), "EvaluateRHS");
}

void UpdateNonLinearity(grid *mesh, markers *particles, markers *topo_chain, surface *topo, mat_prop materials,
                        params *model, Nparams *Nmodel, scale scaling, int mode, double h_contin) {
    (void)particles; (void)topo_chain; (void)topo; (void)mode; (void)h_contin;
    StrainRateComponents(mesh, scaling, model);
    NonNewtonianViscosityGrid(mesh, &materials, model, *Nmodel, &scaling);
    evaluate_rhs(mesh, model, &scaling);
    RheologicalOperators(mesh, model, &scaling, 0);
}

/* ---- decoupled Stokes ---------------------------------------------------- */

/* F (equation numbering of StokesA / StokesC) from the grid-layout rows. */
static void rows_to_eqn(const grid *m, const SparseMat *S, const double *ru, const double *rv, const double *rp,
                        double *Fm, double *Fc) {
    const int nu = m->Nx * (m->Nz + 1), nv = (m->Nx + 1) * m->Nz, np = (m->Nx - 1) * (m->Nz - 1);
    for (int c = 0; c < nu; c++) if (S->eqn_u[c] >= 0 && TAG(m->BCu.type[c]) == -1) Fm[S->eqn_u[c]] = ru[c];
    for (int c = 0; c < nv; c++) if (S->eqn_v[c] >= 0 && TAG(m->BCv.type[c]) == -1) Fm[S->eqn_v[c]] = rv[c];
    for (int c = 0; c < np; c++)
        if (S->eqn_p[c] >= 0 && TAG(m->BCp.type[c]) == -1) Fc[S->eqn_p[c] - S->neq_mom] = rp[c];
}

/* Assemble = 1 records the operator for the next defect solve (matrix-free);
 * Assemble = 0 evaluates the residual rows into StokesA->F / StokesC->F. */
static void build_operator(grid *mesh, params model, SparseMat *Stokes, SparseMat *StokesA, SparseMat *StokesC,
                           int Assemble, int jacobian) {
    ensure(&model, mesh, NULL);
    if (Assemble == 1) { g_jacobian = jacobian; return; }
    mdz_fields f;
    fields_of(mesh, &f, model.Nb_phases, 0);
    keep_only(&f, " u v p_corr D11_n D22_n D33_s roger_x roger_z rhs_p ru rv rp eta_n eta_s ");
    double norms[3];
    check(mdz_EvaluateStokesResidualDecoupled(g_ctx, &f, norms), "BuildStokesOperatorDecoupled");
    rows_to_eqn(mesh, Stokes, mesh->ru, mesh->rv, mesh->rp, StokesA->F, StokesC->F);
}

void BuildStokesOperatorDecoupled(grid *mesh, params model, int lev, double *p_corr, double *p, double *u,
                                  double *v, SparseMat *Stokes, SparseMat *StokesA, SparseMat *StokesB,
                                  SparseMat *StokesC, SparseMat *StokesD, int Assemble) {
    (void)lev; (void)p_corr; (void)p; (void)u; (void)v; (void)StokesB; (void)StokesD;
    build_operator(mesh, model, Stokes, StokesA, StokesC, Assemble, 0);
}

void BuildJacobianOperatorDecoupled(grid *mesh, params model, int lev, double *p_corr, double *p, double *u,
                                    double *v, SparseMat *Stokes, SparseMat *StokesA, SparseMat *StokesB,
                                    SparseMat *StokesC, SparseMat *StokesD, int Assemble) {
    (void)lev; (void)p_corr; (void)p; (void)u; (void)v; (void)StokesB; (void)StokesD;
    build_operator(mesh, model, Stokes, StokesA, StokesC, Assemble, 1);
}

void EvaluateStokesResidualDecoupled(SparseMat *Stokes, SparseMat *StokesA, SparseMat *StokesB, SparseMat *StokesC,
                                     SparseMat *StokesD, Nparams *Nmodel, grid *mesh, params model, scale scaling,
                                     int quiet) {
    (void)StokesB; (void)StokesD; (void)scaling; (void)quiet;
    ensure(&model, mesh, NULL);
    mdz_fields f;
    fields_of(mesh, &f, model.Nb_phases, 0);
    keep_only(&f, " u v p_corr D11_n D22_n D33_s roger_x roger_z rhs_p ru rv rp eta_n eta_s ");
    double norms[3];
    check(mdz_EvaluateStokesResidualDecoupled(g_ctx, &f, norms), "EvaluateStokesResidualDecoupled");
    rows_to_eqn(mesh, Stokes, mesh->ru, mesh->rv, mesh->rp, StokesA->F, StokesC->F);
    Nmodel->resx = norms[0];
    Nmodel->resz = norms[1];
    Nmodel->resp = norms[2];
}

/* ExtractSolutions2 (SOURCE/StokesRoutines.c:187-234) on grid-layout
 * corrections: x <- x + alpha dx on the equation nodes, then the Dirichlet
 * values and free-slip mirrors (ApplyBC). */
static void extract(grid *m, const params *model, const double *du, const double *dv, const double *dp,
                    double alpha) {
    const int Nx = m->Nx, Nz = m->Nz, nu = Nx * (Nz + 1), nv = (Nx + 1) * Nz, np = (Nx - 1) * (Nz - 1);
    (void)model;
    for (int c = 0; c < nu; c++) if (TAG(m->BCu.type[c]) == -1) m->u_in[c] += alpha * du[c];
    for (int c = 0; c < nv; c++) if (TAG(m->BCv.type[c]) == -1) m->v_in[c] += alpha * dv[c];
    for (int c = 0; c < np; c++) if (TAG(m->BCp.type[c]) == -1) m->p_in[c] += alpha * dp[c];
    for (int c = 0; c < nu; c++) if (TAG(m->BCu.type[c]) == 0) m->u_in[c] = m->BCu.val[c];
    for (int c = 0; c < nv; c++) if (TAG(m->BCv.type[c]) == 0) m->v_in[c] = m->BCv.val[c];
    for (int k = 0; k < Nx; k++) {
        if (TAG(m->BCu.type[k]) == 13) m->u_in[k] = m->u_in[k + Nx];
        if (TAG(m->BCu.type[k + Nz * Nx]) == 13) m->u_in[k + Nz * Nx] = m->u_in[k + (Nz - 1) * Nx];
    }
    for (int l = 0; l < Nz; l++) {
        if (TAG(m->BCv.type[l * (Nx + 1)]) == 13) m->v_in[l * (Nx + 1)] = m->v_in[l * (Nx + 1) + 1];
        if (TAG(m->BCv.type[l * (Nx + 1) + Nx]) == 13) m->v_in[l * (Nx + 1) + Nx] = m->v_in[l * (Nx + 1) + Nx - 1];
    }
}

static double *g_dx = NULL;   /* the last defect solve's correction (u | v | p grid layout) */
static size_t g_dx_n = 0;

static double *solve_defect(grid *mesh, params *model, SparseMat *Stokes, SparseMat *StokesA, SparseMat *StokesC) {
    const int Nx = mesh->Nx, Nz = mesh->Nz, nu = Nx * (Nz + 1), nv = (Nx + 1) * Nz, np = (Nx - 1) * (Nz - 1);
    const size_t n = (size_t)nu + nv + np;
    if (n * 2 > g_dx_n) {
        free(g_dx);
        g_dx = (double *)calloc(n * 2, sizeof(double));
        if (!g_dx) { fprintf(stderr, "mdz_refshim: out of host memory\n"); exit(1); }
        g_dx_n = n * 2;
    }
    double *F = g_dx + n, *dx = g_dx;
    memset(F, 0, sizeof(double) * n);
    /* F from the equation-numbered StokesA->F / StokesC->F */
    for (int c = 0; c < nu; c++) if (Stokes->eqn_u[c] >= 0 && TAG(mesh->BCu.type[c]) == -1) F[c] = StokesA->F[Stokes->eqn_u[c]];
    for (int c = 0; c < nv; c++)
        if (Stokes->eqn_v[c] >= 0 && TAG(mesh->BCv.type[c]) == -1) F[nu + c] = StokesA->F[Stokes->eqn_v[c]];
    for (int c = 0; c < np; c++)
        if (Stokes->eqn_p[c] >= 0 && TAG(mesh->BCp.type[c]) == -1)
            F[nu + nv + c] = StokesC->F[Stokes->eqn_p[c] - Stokes->neq_mom];
    mdz_fields f;
    fields_of(mesh, &f, model->Nb_phases, 0);
    keep_only(&f, " eta_n eta_s D11_n D12_n D13_n D14_n D21_n D22_n D23_n D24_n D31_s D32_s D33_s D34_s ");
    int its = 0;
    double rel = 0.0, rtol = model->rel_tol_KSP > 0.0 ? model->rel_tol_KSP : 1e-10;
    check(mdz_SolveStokesDefect(g_ctx, &f, g_jacobian, g_precision, rtol, 1000, F, F + nu, F + nu + nv, dx,
                                dx + nu, dx + nu + nv, &its, &rel), "SolveStokesDefectDecoupled");
    return dx;
}

/* LineSearchDecoupled (SOURCE/StokesRoutines.c:396-626): six trial steps
 * alpha in [amin, amax] (Newton: [-1, -line_search_min], Picard: [-2.5, 0]),
 * each followed by UpdateNonLinearity and the residual; the step of least
 * total residual, else the reference's fall-backs on the x / z residuals. */
static double line_search(grid *mesh, params *model, Nparams *Nmodel, SparseMat *Stokes, SparseMat *StokesA,
                          SparseMat *StokesB, SparseMat *StokesC, SparseMat *StokesD, mat_prop materials,
                          scale scaling, const double *dx) {
    const int Nx = mesh->Nx, Nz = mesh->Nz, nu = Nx * (Nz + 1), nv = (Nx + 1) * Nz, np = (Nx - 1) * (Nz - 1);
    double *u0 = (double *)malloc(sizeof(double) * ((size_t)nu + nv + np));
    if (!u0) { fprintf(stderr, "mdz_refshim: out of host memory\n"); exit(1); }
    memcpy(u0, mesh->u_in, sizeof(double) * nu);
    memcpy(u0 + nu, mesh->v_in, sizeof(double) * nv);
    memcpy(u0 + nu + nv, mesh->p_in, sizeof(double) * np);
    const double r0x = Nmodel->resx, r0z = Nmodel->resz, r0p = Nmodel->resp;
    const int ntry = 6;
    const double amin = model->Newton ? -1.0 : -2.5, amax = model->Newton ? -model->line_search_min : 0.0;
    const double da = fabs(amax - amin) / (ntry - 1);
    double a = amax, av[6], rx[6], rz[6], best = 1e300;
    int ib = 0;
    for (int k = 0; k < ntry; k++) {
        if (k > 0) a -= da;
        av[k] = a;
        memcpy(mesh->u_in, u0, sizeof(double) * nu);
        memcpy(mesh->v_in, u0 + nu, sizeof(double) * nv);
        memcpy(mesh->p_in, u0 + nu + nv, sizeof(double) * np);
        extract(mesh, model, dx, dx + nu, dx + nu + nv, a);
        UpdateNonLinearity(mesh, NULL, NULL, NULL, materials, model, Nmodel, scaling, 0, 0.0);
        EvaluateStokesResidualDecoupled(Stokes, StokesA, StokesB, StokesC, StokesD, Nmodel, mesh, *model, scaling, 1);
        rx[k] = Nmodel->resx; rz[k] = Nmodel->resz;
        const double t = sqrt(Nmodel->resx * Nmodel->resx + Nmodel->resz * Nmodel->resz +
                              Nmodel->resp * Nmodel->resp);
        if (t < best) { best = t; ib = k; }
    }
    int ok = best < sqrt(r0x * r0x + r0z * r0z + r0p * r0p);
    if (!ok) {
        int ixz = 0, ix = 0, iz = 0;
        for (int k = 1; k < ntry; k++) {
            if (hypot(rx[k], rz[k]) < hypot(rx[ixz], rz[ixz])) ixz = k;
            if (rx[k] < rx[ix]) ix = k;
            if (rz[k] < rz[iz]) iz = k;
        }
        if (rx[ixz] < r0x && rz[ixz] < r0z) { ok = 1; ib = ixz; }
        else if (rx[ix] < r0x) { ok = 1; ib = ix; }
        else if (rz[iz] < r0z) { ok = 1; ib = iz; }
    }
    memcpy(mesh->u_in, u0, sizeof(double) * nu);
    memcpy(mesh->v_in, u0 + nu, sizeof(double) * nv);
    memcpy(mesh->p_in, u0 + nu + nv, sizeof(double) * np);
    Nmodel->resx = r0x; Nmodel->resz = r0z; Nmodel->resp = r0p;
    free(u0);
    if (!ok || fabs(av[ib]) < 1e-13) { Nmodel->stagnated = 1; return 0.0; }
    return av[ib];
}

double LineSearchDecoupled(SparseMat *Stokes, SparseMat *StokesA, SparseMat *StokesB, SparseMat *StokesC,
                           SparseMat *StokesD, double *sol, grid *mesh, params *model, Nparams *Nmodel,
                           markers *particles, markers *topo_chain, surface *topo, mat_prop materials,
                           scale scaling) {
    (void)particles; (void)topo_chain; (void)topo;
    ensure(model, mesh, NULL);
    /* sol: the correction in the reference's equation numbering */
    const int Nx = mesh->Nx, Nz = mesh->Nz, nu = Nx * (Nz + 1), nv = (Nx + 1) * Nz, np = (Nx - 1) * (Nz - 1);
    double *dx = (double *)calloc((size_t)nu + nv + np, sizeof(double));
    if (!dx) { fprintf(stderr, "mdz_refshim: out of host memory\n"); exit(1); }
    for (int c = 0; c < nu; c++) if (Stokes->eqn_u[c] >= 0 && TAG(mesh->BCu.type[c]) == -1) dx[c] = sol[Stokes->eqn_u[c]];
    for (int c = 0; c < nv; c++)
        if (Stokes->eqn_v[c] >= 0 && TAG(mesh->BCv.type[c]) == -1) dx[nu + c] = sol[Stokes->eqn_v[c]];
    for (int c = 0; c < np; c++)
        if (Stokes->eqn_p[c] >= 0 && TAG(mesh->BCp.type[c]) == -1) dx[nu + nv + c] = sol[Stokes->eqn_p[c]];
    const double a = line_search(mesh, model, Nmodel, Stokes, StokesA, StokesB, StokesC, StokesD, materials, scaling,
                                 dx);
    free(dx);
    return a;
}

void SolveStokesDefectDecoupled(SparseMat *StokesA, SparseMat *StokesB, SparseMat *StokesC, SparseMat *StokesD,
                                SparseMat *Stokes, DirectSolver *PardisoStokes, Nparams *Nmodel, grid *mesh,
                                params *model, markers *particles, markers *topo_chain, surface *topo,
                                mat_prop materials, scale scaling, SparseMat *JacobA, SparseMat *JacobB,
                                SparseMat *JacobC) {
    (void)PardisoStokes; (void)particles; (void)topo_chain; (void)topo; (void)JacobA; (void)JacobB; (void)JacobC;
    ensure(model, mesh, NULL);
    double *dx = solve_defect(mesh, model, Stokes, StokesA, StokesC);
    const int Nx = mesh->Nx, Nz = mesh->Nz, nu = Nx * (Nz + 1), nv = (Nx + 1) * Nz;
    double alpha = -1.0;
    if (model->line_search == 1)
        alpha = line_search(mesh, model, Nmodel, Stokes, StokesA, StokesB, StokesC, StokesD, materials, scaling, dx);
    extract(mesh, model, dx, dx + nu, dx + nu + nv, alpha);
}

/* ---- grid -> markers and advection ---------------------------------------- */

static int node_set_of(const grid *m, const double *X, const double *Z) {
    if (X == m->xg_coord && Z == m->zg_coord) return 0;
    if (X == m->xg_coord && Z == m->zvx_coord) return -1;
    if (X == m->xvz_coord && Z == m->zg_coord) return -2;
    return 9;
}

void Interp_Grid2P(markers particles, DoodzFP *PartField, grid *mesh, double *NodeField, double *X_vect,
                   double *Z_vect, int Nx, int Nz, char *tag) {
    (void)Nx; (void)Nz; (void)tag;
    ensure(NULL, mesh, &particles);
    const int set = node_set_of(mesh, X_vect, Z_vect);
    if (set == 9) { fprintf(stderr, "Interp_Grid2P (GPU): coordinate lines of no known node set\n"); exit(1); }
    put_markers(&particles);
    check(mdz_Interp_Grid2P(g_ctx, NodeField, set, PartField), "Interp_Grid2P");
}

void Interp_Grid2P_centroids2(markers particles, DoodzFP *PartField, grid *mesh, double *NodeField,
                              double *X_vect, double *Z_vect, int Nx, int Nz, char *tag, params *model) {
    (void)X_vect; (void)Z_vect; (void)Nx; (void)Nz; (void)tag;
    ensure(model, mesh, &particles);
    put_markers(&particles);
    check(mdz_Interp_Grid2P(g_ctx, NodeField, 1, PartField), "Interp_Grid2P_centroids2");
}

void RogerGuntherII(markers *particles, params model, grid mesh, int precise, scale scaling) {
    (void)precise; (void)scaling;
    ensure(&model, &mesh, particles);
    put_markers(particles);
    check(mdz_RogerGuntherII(g_ctx, mesh.u_in, mesh.v_in, model.dt), "RogerGuntherII");
    check(mdz_get_markers(g_ctx, particles->Nb_part, particles->x, particles->z, particles->phase, particles->Vx,
                          particles->Vz), "RogerGuntherII");
}

void UpdateParticleStress(grid *mesh, markers *particles, params *model, mat_prop *materials, scale *scaling) {
    (void)materials; (void)scaling;
    ensure(model, mesh, particles);
    put_markers(particles);
    put_attrs(particles, 0, 1, 0);
    mdz_fields f;
    fields_of(mesh, &f, model->Nb_phases, 0);
    keep_only(&f, " sxxd szzd sxz sxxd0 szzd0 sxz0 ");
    check(mdz_UpdateParticleStress(g_ctx, &f), "UpdateParticleStress");
    const int n = particles->Nb_part;
    get_attr(MDZ_M_SXXD, n, particles->sxxd);
    get_attr(MDZ_M_SZZD, n, particles->szzd);
    get_attr(MDZ_M_SXZ, n, particles->sxz);
}

void AccumulatedStrainII(grid *mesh, scale scaling, params model, markers *particles, double *X_vect,
                         double *Z_vect, int Nx, int Nz, char *tag) {
    (void)scaling; (void)X_vect; (void)Z_vect; (void)Nx; (void)Nz; (void)tag;
    ensure(&model, mesh, particles);
    put_markers(particles);
    put_attrs(particles, 1, 0, 0);
    mdz_fields f;
    fields_of(mesh, &f, model.Nb_phases, 0);
    keep_only(&f, " eII_pl eII_pwl eII_lin eII_el eII_cst ");
    check(mdz_AccumulatedStrainII(g_ctx, &f, model.dt), "AccumulatedStrainII");
    const int n = particles->Nb_part;
    get_attr(MDZ_M_STRAIN, n, particles->strain);
    get_attr(MDZ_M_STRAIN_PL, n, particles->strain_pl);
}
