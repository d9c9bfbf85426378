/*
 * CPU oracle, part 2 (test infrastructure only): strain rates, local
 * visco-elasto-plastic rheology, rheological operators and the RHS, restated
 * from MDOODZ 6.0 for the isotropic, incompressible, non-reactive subset.
 * Line references are to the reference's SOURCE/ directory.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "mdz_oracle.h"

#define ZEROC 273.15

/* ------------------------------------------------------------------------ */
/* InterpCentroidsToVerticesDouble, non-periodic (GridRoutines.c:106-198):
 * pad the centroid array by one ring repeating its edge (corners repeat the
 * diagonal neighbour), then average the four centroids around each vertex. */
int orc_c2v(const mdz_grid_desc *g, const double *cen, double *ver) {
    int ncx = g->Nx - 1, ncz = g->Nz - 1, W = ncx + 2, k, l;
    double *t = calloc((size_t)W * (ncz + 2), sizeof(double));
    if (!t) return -1;
    for (l = 0; l < ncz; l++)
        for (k = 0; k < ncx; k++) t[(k + 1) + (l + 1) * W] = cen[k + l * ncx];
    for (k = 1; k < ncx + 1; k++) { t[k] = t[k + W]; t[k + (ncz + 1) * W] = t[k + ncz * W]; }
    for (l = 1; l < ncz + 1; l++) { t[l * W] = t[1 + l * W]; t[ncx + 1 + l * W] = t[ncx + l * W]; }
    t[0] = t[1 + W];
    t[ncx + 1] = t[ncx + W];
    t[(ncz + 1) * W] = t[1 + ncz * W];
    t[ncx + 1 + (ncz + 1) * W] = t[ncx + ncz * W];
    for (k = 0; k < g->Nx; k++)
        for (l = 0; l < g->Nz; l++) {
            int c1 = k + l * g->Nx, c0 = k + (l + 1) * W + 1;
            ver[c1] = 0.0;
            if (g->BCg_type[c1] != 30) ver[c1] = 0.25 * (t[c0 - 1 - W] + t[c0 - W] + t[c0 - 1] + t[c0]);
        }
    free(t);
    return 0;
}

/* InterpVerticesToCentroidsDouble (GridRoutines.c:204-228). */
int orc_v2c(const mdz_grid_desc *g, double *cen, const double *ver) {
    int ncx = g->Nx - 1, ncz = g->Nz - 1, Nx = g->Nx;
    for (int k = 0; k < ncx; k++)
        for (int l = 0; l < ncz; l++) {
            int c0 = k + l * ncx, c1 = k + l * Nx;
            if (g->BCp_type[c0] != 30 && g->BCp_type[c0] != 31)
                cen[c0] = 0.25 * (ver[c1] + ver[c1 + 1] + ver[c1 + Nx] + ver[c1 + 1 + Nx]);
        }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* StrainRateComponents (RheologyDensity.c:1902-1984). */
int orc_strain_rates(const mdz_grid_desc *g, mdz_fields *f) {
    int Nx = g->Nx, Nz = g->Nz, ncx = Nx - 1, ncz = Nz - 1, k, l;
    double dx = g->dx, dz = g->dz;
    const double *u = f->u, *v = f->v;
    for (l = 0; l < ncz; l++)
        for (k = 0; k < ncx; k++) {
            int c0 = k + l * ncx, c1 = k + l * Nx, c2 = k + l * (Nx + 1);
            if (g->BCp_type[c0] != 30 && g->BCp_type[c0] != 31) {
                f->div_u[c0] = (u[c1 + 1 + Nx] - u[c1 + Nx]) / dx + (v[c2 + Nx + 1 + 1] - v[c2 + 1]) / dz;
                f->exxd[c0] = (u[c1 + 1 + Nx] - u[c1 + Nx]) / dx - 1.0 / 3.0 * f->div_u[c0];
                f->ezzd[c0] = (v[c2 + 1 + (Nx + 1)] - v[c2 + 1]) / dz - 1.0 / 3.0 * f->div_u[c0];
            } else {
                f->div_u[c0] = f->exxd[c0] = f->ezzd[c0] = 0.0;
            }
        }
    for (l = 0; l < Nz; l++)
        for (k = 0; k < Nx; k++) {
            int c1 = k + l * Nx, c2 = k + l * (Nx + 1);
            f->exz[c1] = 0.0;
            if (g->BCg_type[c1] != 30) {
                if (g->BCu_type[c1] != 30 && g->BCu_type[c1 + Nx] != 30) f->exz[c1] += 0.5 * (u[c1 + Nx] - u[c1]) / dz;
                if (g->BCv_type[c2] != 30 && g->BCv_type[c2 + 1] != 30) f->exz[c1] += 0.5 * (v[c2 + 1] - v[c2]) / dx;
            }
        }
    for (l = 0; l < ncz; l++)
        for (k = 0; k < ncx; k++) {
            int c0 = k + l * ncx, c1 = k + l * Nx;
            double s = 0.0;
            f->exz_n[c0] = 0.0;
            if (g->BCp_type[c0] != 30 && g->BCp_type[c0] != 31) {
                if (g->BCg_type[c1] != 30) { f->exz_n[c0] += f->exz[c1]; s++; }
                if (g->BCg_type[c1 + 1] != 30) { f->exz_n[c0] += f->exz[c1 + 1]; s++; }
                if (g->BCg_type[c1 + Nx] != 30) { f->exz_n[c0] += f->exz[c1 + Nx]; s++; }
                if (g->BCg_type[c1 + Nx + 1] != 30) { f->exz_n[c0] += f->exz[c1 + Nx + 1]; s++; }
                if (s > 0) f->exz_n[c0] /= s;
            }
        }
    orc_c2v(g, f->exxd, f->exxd_s);
    orc_c2v(g, f->ezzd, f->ezzd_s);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Outputs of one local solve (the pointer arguments of Viscosity()). */
typedef struct {
    double eta, txx, tzz, txz, etaVE, VEcoeff, Eii_el, Eii_pl, Eii_pwl, Eii_lin, Eii_cst, Eii_exp, Eii_gbs;
    double Exx_el, Ezz_el, Exz_el, Exx_diss, Ezz_diss, Exz_diss, d1;
    double detadexx, detadezz, detadexz, detadp, X1, OverS;
    double ddivpdexx, ddivpdezz, ddivpdexz, ddivpdp, Pcorr, drhodp, rho, div_el, div_pl, div_r;
    int ve_fail, vp_fail;
} visc_out;

static double dmin(double a, double b) { return a <= b ? a : b; }

/* Viscosity (RheologyDensity.c:44-707) for constant, dislocation, diffusion
 * and Peierls creep, grain-boundary sliding, elasticity and Drucker-Prager /
 * von Mises plasticity with the tension cut-off. */
static void orc_visc(int p, double G, double T, double P, double d, double phi, double X0, double Exx, double Ezz,
                     double Exz, double Gxx, double Gzz, double Gxz, double Txx0, double Tzz0, double Txz0,
                     const mdz_materials *m, const mdz_rheo_params *prm, double dil, double fric, double C, double P0,
                     double beta, visc_out *o) {
    double R = m->R, dt = prm->dt, minEta = prm->mineta, maxEta = prm->maxeta;
    int nitmax = 20, it, elastic = prm->iselastic;
    int constant = m->cstv[p] != 0, dislocation = m->pwlv[p] != 0, diffusion = m->linv[p] != 0;
    /* :135-141 (Peierls tested before the 0 C clamp) */
    int peierls = m->expv[p] != 0 && T < (1200.0 + ZEROC) / prm->scale_T, gbs = m->gbsv[p] != 0;
    double Ea_gbs = m->Qgbs[p], Va_gbs = m->Vgbs[p], n_gbs = m->ngbs[p], m_gbs = m->mgbs[p], r_gbs = m->rgbs[p];
    double A_gbs = m->Agbs[p], f_gbs = m->fgbs[p], a_gbs = m->agbs[p], F_gbs = m->Fgbs[p];
    double B_gbs = 0, C_gbs = 0, eta_gbs = 0, Eii_gbs = 0;
    double Ea_exp = m->Qexp[p], S_exp = m->Sexp[p], E_exp = m->Eexp[p], gamma = m->Gexp[p], n_exp = m->nexp[p];
    double ST = 0, B_exp = 0, C_exp = 0, F_exp = 0, eta_exp = 0, Eii_exp = 0;
    double Exx_exp = 0, Ezz_exp = 0, Exz_exp = 0;
    int tens = 0;
    double dsin_dildExx = 0.0, dsin_dildEzz = 0.0, dsin_dildExz = 0.0, dsin_dildP = 0.0;
    double tol = 1.0e-11, res = 0.0, res0 = 0.0, dfdeta, Txx, Tzz, Txz, Tii, ieta_sum;
    double Tii0 = sqrt(Txx0 * Txx0 + Txz0 * Txz0);
    double eta_up, eta_lo, eta_ve, eta_pwl = 0.0, eta_lin = 0.0, eta_el, eta_cst = 0.0, eta_vep = 0.0;
    double Eii, Gii, f_ani, K = 1.0 / beta;
    double Ea_pwl = m->Qpwl[p], Va_pwl = m->Vpwl[p], n_pwl = m->npwl[p], m_pwl = m->mpwl[p], r_pwl = m->rpwl[p];
    double A_pwl = m->Apwl[p], f_pwl = m->fpwl[p], a_pwl = m->apwl[p], F_pwl = m->Fpwl[p], pre = m->pref_pwl[p];
    double Ea_lin = m->Qlin[p], Va_lin = m->Vlin[p], n_lin = m->nlin[p], m_lin = m->mlin[p], r_lin = m->rlin[p];
    double A_lin = m->Alin[p], f_lin = m->flin[p], a_lin = m->alin[p], F_lin = m->Flin[p];
    double B_pwl = 0, B_lin = 0, C_pwl = 0, C_lin = 0, dCpwldP = 0, dClindP = 0;
    double eta_vp0 = m->eta_vp[p], n_vp = m->n_vp[p], eta_vp = 0.0;
    double Exx_lin = 0, Ezz_lin = 0, Exz_lin = 0, Exx_cst = 0, Ezz_cst = 0, Exz_cst = 0;
    double Exx_pl, Ezz_pl, Exz_pl, Exx_pwl, Ezz_pwl, Exz_pwl;
    double detadTxx, detadTzz, detadTxz, dve_dExx, dve_dEzz, dve_dExz, dve_dP, deta, dummy, Jii;
    double gdot = 0.0, dQdtxx = 0, dQdtzz = 0, dQdtxz = 0, dQdP = 0, Tyield, F_trial, F_trial0, divp = 0.0, Pc = P;
    double dlamdExx = 0, dlamdEzz = 0, dlamdExz = 0, dlamdP = 0;
    double dvep_dExx = 0, dvep_dEzz = 0, dvep_dExz = 0, dvep_dP = 0;
    int is_pl = 0;
    double Eii_pwl = 0, Eii_lin = 0, Eii_cst = 0;

    memset(o, 0, sizeof *o);
    /* invariants :106-115 */
    double Eyy = -(Exx + Ezz), Gyy = -(Gxx + Gzz);
    Eii = sqrt(1.0 / 2.0 * (Exx * Exx + Ezz * Ezz + Eyy * Eyy) + Exz * Exz);
    Gii = sqrt(1.0 / 2.0 * (Gxx * Gxx + Gzz * Gzz + Gyy * Gyy) + Gxz * Gxz);
    if (Eii * prm->scale_E < 1e-30) Eii = 1e-30 / prm->scale_E;
    if (Gii * prm->scale_E < 1e-30) Gii = 1e-30 / prm->scale_E;
    f_ani = Gii / Eii;
    o->Pcorr = P;
    if (prm->step == 0) elastic = 0;                                   /* :147 */
    o->d1 = m->gs_ref[p];
    if (elastic == 0) { G = 1e1; K = 1e1; dil = 0.0; }                 /* :156 */
    if (T < ZEROC / prm->scale_T) T = ZEROC / prm->scale_T;
    /* precomputations :164-181 */
    if (dislocation) {
        B_pwl = pre * F_pwl * pow(A_pwl, -1.0 / n_pwl) * exp((Ea_pwl + P * Va_pwl) / R / n_pwl / T) *
                pow(d, m_pwl / n_pwl) * pow(f_pwl, -r_pwl / n_pwl) * exp(-a_pwl * phi / n_pwl);
        C_pwl = pow(2.0 * f_ani * B_pwl, -n_pwl);
        dCpwldP = -C_pwl * Va_pwl / R / T;
    }
    if (diffusion) {
        B_lin = F_lin * pow(A_lin, -1.0 / n_lin) * exp((Ea_lin + P * Va_lin) / R / n_lin / T) *
                pow(f_lin, -r_lin / n_lin) * exp(-a_lin * phi / n_lin);
        C_lin = pow(2.0 * f_ani * B_lin, -n_lin);
        dClindP = -C_lin * Va_lin / R / T;
    }
    if (gbs) {
        B_gbs = F_gbs * pow(A_gbs, -1.0 / n_gbs) * exp((Ea_gbs + P * Va_gbs) / R / n_gbs / T) * pow(d, m_gbs / n_gbs) *
                pow(f_gbs, -r_gbs / n_gbs) * exp(-a_gbs * phi / n_gbs);
        C_gbs = pow(2.0 * f_ani * B_gbs, -n_gbs);
    }
    if (peierls) {   /* :181-199, the "new" form */
        ST = Ea_exp / R / T * 2.0 * gamma * (1 - gamma);
        double Arr_exp = exp(-Ea_exp / R / T * pow(1.0 - gamma, 2.0));
        F_exp = pow(pow(2.0, 1.0 - ST - n_exp) / pow(sqrt(3.0), ST + n_exp + 1.0), 1.0 / (ST + n_exp));
        B_exp = F_exp * (pow(gamma * S_exp, ST / (ST + n_exp)) / pow(E_exp * Arr_exp, 1.0 / (ST + n_exp)));
        C_exp = pow(2.0 * f_ani * B_exp, -(ST + n_exp));
    }
    /* yield :214-225 */
    double cos_fric = cos(fric), sin_fric = sin(fric), sin_dil = sin(dil);
    Tyield = C * cos_fric + P * sin_fric;
    if (m->Slim[p] < Tyield) { sin_fric = 0.0; cos_fric = 1.0; sin_dil = 0.0; C = m->Slim[p]; Tyield = m->Slim[p]; }
    {   /* tension cut-off :204-213 */
        double P_tens = -25e6 / prm->scale_S;
        double sin_fric_tens = -C * cos_fric / P_tens;
        if (C * cos_fric + P * sin_fric_tens < Tyield && m->is_tensile[p] == 1) {
            sin_fric = sin_fric_tens;
            Tyield = C * cos_fric + P * sin_fric_tens;
            tens = 1;
        }
    }
    o->X1 = X0;
    /* isolated viscosities :320-330 */
    eta_el = G * dt;
    if (constant) eta_cst = m->eta0[p];
    if (dislocation) eta_pwl = B_pwl * pow(Eii, 1.0 / n_pwl - 1.0);
    if (diffusion) eta_lin = B_lin * pow(Eii, 1.0 / n_lin - 1.0) * pow(d, m_lin / n_lin);
    if (gbs) eta_gbs = B_gbs * pow(Eii, 1.0 / n_gbs - 1.0);
    if (peierls) eta_exp = B_exp * pow(Eii, 1.0 / (ST + n_exp) - 1.0);
    /* bounds :340-378 */
    eta_up = 1.0e100 / prm->scale_eta;
    ieta_sum = 0.0;
    if (constant) { eta_up = dmin(eta_up, eta_cst); ieta_sum += 1.0 / eta_cst; }
    if (dislocation) { eta_up = dmin(eta_up, eta_pwl); ieta_sum += 1.0 / eta_pwl; }
    if (elastic) { eta_up = dmin(eta_up, eta_el); ieta_sum += 1.0 / eta_el; }
    if (peierls) { eta_up = dmin(eta_up, eta_exp); ieta_sum += 1.0 / eta_exp; }
    if (diffusion) { eta_up = dmin(eta_up, eta_lin); ieta_sum += 1.0 / eta_lin; }
    if (gbs) { eta_up = dmin(eta_up, eta_gbs); ieta_sum += 1.0 / eta_gbs; }
    eta_lo = 1.0 / ieta_sum;
    (void)eta_lo;
    /* local Newton on eta_ve :384-415 */
    eta_ve = eta_up;
    for (it = 0; it < nitmax; it++) {
        Tii = 2.0 * f_ani * eta_ve * Eii;
        if (constant) Eii_cst = Tii / f_ani / 2.0 / eta_cst;
        if (dislocation) Eii_pwl = C_pwl * pow(Tii, n_pwl);
        if (gbs) Eii_gbs = C_gbs * pow(Tii, n_gbs);
        if (peierls) Eii_exp = C_exp * pow(Tii, ST + n_exp);
        if (diffusion) Eii_lin = C_lin * pow(Tii, n_lin) * pow(o->d1, -m_lin);
        double Eii_vis = Eii_pwl + Eii_exp + Eii_lin + Eii_gbs + Eii_cst;
        double r = Eii - elastic * Tii / (2.0 * eta_el) - Eii_vis;
        res = fabs(r / Eii);
        if (it == 0) res0 = res;
        if (res < tol / 100) break;
        dfdeta = 0.0;
        if (elastic) dfdeta += -Eii / eta_el;
        if (peierls) dfdeta += -Eii_exp * (ST + n_exp) / eta_ve;
        if (diffusion) dfdeta += -Eii_lin * n_lin / eta_ve;
        if (dislocation) dfdeta += -Eii_pwl * n_pwl / eta_ve;
        if (constant) dfdeta += -Eii / eta_cst;
        eta_ve -= r / dfdeta;
    }
    (void)res0;
    if (it == nitmax - 1 && res > tol) o->ve_fail = 1;                  /* :417 (the reference exits) */
    /* stresses :421-425 */
    Tii = 2.0 * eta_ve * f_ani * Eii;
    Txx = Gxx * Tii / f_ani / Eii;
    double Tyy = Gxx * Tii / f_ani / Eii;
    Tzz = Gzz * Tii / f_ani / Eii;
    Txz = Gxz * Tii / f_ani / Eii;
    if (dislocation) eta_pwl = pow(2.0 * C_pwl, -1.0) * pow(Tii, 1.0 - n_pwl);
    if (diffusion) eta_lin = B_lin * pow(Eii_lin, 1.0 / n_lin - 1.0) * pow(o->d1, m_lin / n_lin);
    if (diffusion) { Exx_lin = Txx / 2.0 / eta_lin; Ezz_lin = Tzz / 2.0 / eta_lin; Exz_lin = Txz / 2.0 / eta_lin; }
    if (peierls) eta_exp = B_exp * pow(Eii_exp, 1.0 / (ST + n_exp) - 1.0);
    if (peierls) { Exx_exp = Txx / 2.0 / eta_exp; Ezz_exp = Tzz / 2.0 / eta_exp; Exz_exp = Txz / 2.0 / eta_exp; }
    if (constant) { Exx_cst = Txx / 2.0 / eta_cst; Ezz_cst = Tzz / 2.0 / eta_cst; Exz_cst = Txz / 2.0 / eta_cst; }
    /* VE tangent :449-471 */
    deta = 0.0;
    if (dislocation) deta += -C_pwl * pow(Tii, n_pwl - 3.0) * (n_pwl - 1.0);
    if (peierls) deta += -C_exp * pow(Tii, n_exp + ST - 3.0) * (n_exp + ST - 1.0);
    if (diffusion) deta += -C_lin * pow(Tii, n_lin - 3.0) * (n_lin - 1.0) * pow(o->d1, -m_lin);
    detadTxx = deta * (2.0 * Txx + Tzz) * pow(eta_ve, 2.0);
    detadTzz = deta * (2.0 * Tzz + Txx) * pow(eta_ve, 2.0);
    detadTxz = 2.0 * deta * Txz * pow(eta_ve, 2.0);
    double den = 1.0 - 2.0 * (detadTxx * Exx + detadTzz * Ezz + detadTxz * Exz);
    dve_dExx = detadTxx * 2.0 * eta_ve / den;
    dve_dEzz = detadTzz * 2.0 * eta_ve / den;
    dve_dExz = detadTxz * 2.0 * eta_ve / den;
    dummy = 0.0;
    Jii = Tii * Tii;
    if (dislocation) dummy += -2.0 * pow(Jii, (1.0 / 2.0) * n_pwl - 1.0 / 2.0) * dCpwldP;
    if (diffusion) dummy += -2.0 * pow(Jii, (1.0 / 2.0) * n_lin - 1.0 / 2.0) * pow(d, -m_lin) * dClindP;
    dve_dP = pow(eta_ve, 2) * dummy;
    /* plasticity :482-560 */
    F_trial = Tii - Tyield;
    if (tens == 1) {   /* :456-465 */
        eta_vp = eta_vp0 * pow(Eii, 1.0 / n_vp - 1);
        double Pc_chk = -(C * cos_fric) / (-Tii / P + sin_fric);
        sin_dil = (P * eta_ve + P * eta_vp - Pc_chk * eta_ve - Pc_chk * eta_vp) /
                  (K * dt * (C * cos_fric + Pc_chk * sin_fric - Tii));
    }
    if (F_trial > 1e-17) {
        is_pl = 1;
        eta_vp = eta_vp0 * pow(Eii, 1.0 / n_vp - 1);
        gdot = F_trial / (eta_ve + eta_vp + K * dt * sin_fric * sin_dil);
        dQdtxx = Txx / 2.0 / Tii;
        dQdtzz = Tzz / 2.0 / Tii;
        dQdtxz = Txz / 1.0 / Tii;
        dQdP = -sin_dil;
        res0 = F_trial;
        F_trial0 = F_trial;
        for (it = 0; it < nitmax; it++) {
            dQdP = -sin_dil;
            divp = -gdot * dQdP;
            Pc = P + K * dt * divp;
            eta_vp = eta_vp0 * pow(fabs(gdot), 1.0 / n_vp - 1.0);
            Tyield = C * cos_fric + Pc * sin_fric + gdot * eta_vp;
            F_trial = Tii - eta_ve * gdot - Tyield;
            res = fabs(F_trial);
            if (res < tol || res / F_trial0 < tol) break;
            double dFdgdot = -eta_ve - eta_vp / n_vp - K * dt * sin_fric * sin_dil;
            gdot -= F_trial / dFdgdot;
        }
        if (it == nitmax - 1 && (res > tol || res / F_trial0 > tol)) o->vp_fail = 1;   /* :529 */
        Txx = 2.0 * eta_ve * (Exx - gdot * dQdtxx);
        Tzz = 2.0 * eta_ve * (Ezz - gdot * dQdtzz);
        Tyy = -(Txx + Tzz);
        Txz = 2.0 * eta_ve * (Exz - gdot * dQdtxz / 2.0);
        Tii = sqrt(0.5 * (pow(Txx, 2.0) + pow(Tzz, 2.0) + pow(Tyy, 2.0)) + pow(Txz, 2.0));
        eta_vep = Tii / (2.0 * Eii);
        o->Eii_pl = gdot / 2.0;
        Tii = 2.0 * eta_vep * Eii;
        o->OverS = eta_vp * gdot;
        o->Pcorr = Pc;
    }
    (void)Tyy;
    /* VEP tangent :573-603 */
    if (is_pl) {
        if (tens == 1) {   /* :578-587 */
            double dEii_dExx = (2.0 * Exx + Ezz) / 2.0 / Eii;
            double dEii_dEzz = (2.0 * Ezz + Exx) / 2.0 / Eii;
            double dEii_dExz = Exz / 1.0 / Eii;
            double A = 2 * Eii * eta_ve - P * sin_fric;
            double den = K * dt * A * (C * P * cos_fric * sin_fric + (C * cos_fric - 2 * Eii * eta_ve) * A);
            dsin_dildExx = (2 * K * dt * sin_dil * (Eii * dve_dExx + dEii_dExx * eta_ve) * (C * P * cos_fric * sin_fric + pow(A, 2)) +
                            P * (-C * cos_fric * dve_dExx * A + 2 * C * cos_fric * (eta_ve + eta_vp) * (Eii * dve_dExx + dEii_dExx * eta_ve) +
                                 dve_dExx * pow(A, 2))) / den;
            dsin_dildEzz = (2 * K * dt * sin_dil * (Eii * dve_dEzz + dEii_dEzz * eta_ve) * (C * P * cos_fric * sin_fric + pow(A, 2)) +
                            P * (-C * cos_fric * dve_dEzz * A + 2 * C * cos_fric * (eta_ve + eta_vp) * (Eii * dve_dEzz + dEii_dEzz * eta_ve) +
                                 dve_dEzz * pow(A, 2))) / den;
            dsin_dildExz = (2 * K * dt * sin_dil * (Eii * dve_dExz + dEii_dExz * eta_ve) * (C * P * cos_fric * sin_fric + pow(A, 2)) +
                            P * (-C * cos_fric * dve_dExz * A + 2 * C * cos_fric * (eta_ve + eta_vp) * (Eii * dve_dExz + dEii_dExz * eta_ve) +
                                 dve_dExz * pow(A, 2))) / den;
            dsin_dildP = (2 * C * Eii * cos_fric * (eta_ve + eta_vp) * (P * dve_dP - eta_ve) - C * P * cos_fric * dve_dP * A +
                          2 * Eii * K * dt * sin_dil * (C * cos_fric * sin_fric * (P * dve_dP - eta_ve) + dve_dP * pow(A, 2)) +
                          pow(A, 2) * (P * dve_dP + eta_ve + eta_vp)) / den;
        }
        double dFdExx = (2.0 * Exx + Ezz) * eta_ve / Eii + 2.0 * Eii * dve_dExx;
        double dFdEzz = (2.0 * Ezz + Exx) * eta_ve / Eii + 2.0 * Eii * dve_dEzz;
        double dFdExz = 2.0 * Exz * eta_ve / Eii + 2.0 * Eii * dve_dExz;
        double dFdP = -sin_fric + 2.0 * Eii * dve_dP;
        double gg = 1.0 / (eta_ve + eta_vp / n_vp + K * dt * sin_fric * sin_dil);
        dlamdExx = gg * (dFdExx - gdot * (dve_dExx + K * dt * sin_fric * dsin_dildExx));
        dlamdEzz = gg * (dFdEzz - gdot * (dve_dEzz + K * dt * sin_fric * dsin_dildEzz));
        dlamdExz = gg * (dFdExz - gdot * (dve_dExz + K * dt * sin_fric * dsin_dildExz));
        dlamdP = gg * (dFdP - gdot * (dve_dP + K * dt * sin_fric * dsin_dildP));
        double dvp_dExx = eta_vp / gdot * dlamdExx * (1.0 / n_vp - 1.0);
        double dvp_dEzz = eta_vp / gdot * dlamdEzz * (1.0 / n_vp - 1.0);
        double dvp_dExz = eta_vp / gdot * dlamdExz * (1.0 / n_vp - 1.0);
        double dvp_dP = eta_vp / gdot * dlamdP * (1.0 / n_vp - 1.0);
        double a = eta_vp + K * dt * sin_fric * sin_dil;
        dvep_dExx = -0.5 * (2.0 * Exx + Ezz) * Tyield / (2.0 * pow(Eii, 3.0)) +
                    (a * dlamdExx + gdot * dvp_dExx + gdot * K * dt * sin_fric * dsin_dildExx) / (2.0 * Eii);
        dvep_dEzz = -0.5 * (2.0 * Ezz + Exx) * Tyield / (2.0 * pow(Eii, 3.0)) +
                    (a * dlamdEzz + gdot * dvp_dEzz + gdot * K * dt * sin_fric * dsin_dildEzz) / (2.0 * Eii);
        dvep_dExz = -Exz * Tyield / (2.0 * pow(Eii, 3.0)) +
                    (a * dlamdExz + gdot * dvp_dExz + gdot * K * dt * sin_fric * dsin_dildExz) / (2.0 * Eii);
        dvep_dP = (sin_fric + a * dlamdP + gdot * dvp_dP + gdot * K * dt * sin_fric * dsin_dildP) / (2.0 * Eii);
    }
    /* density :632-640 (non-reactive branch) */
    o->rho = m->rho[p] * exp(1.0 / K * Pc - m->alp[p] * T);
    o->drhodp = o->rho / K;
    /* outputs :657-707 */
    double inv_eta_diss = 0.0;
    if (peierls) inv_eta_diss += 1.0 / eta_exp;
    if (dislocation) inv_eta_diss += 1.0 / eta_pwl;
    if (diffusion) inv_eta_diss += 1.0 / eta_lin;
    if (constant) inv_eta_diss += 1.0 / eta_cst;
    if (is_pl == 0) {
        o->detadexx = dve_dExx; o->detadezz = dve_dEzz; o->detadexz = dve_dExz; o->detadp = dve_dP;
        o->etaVE = eta_ve;
        o->ddivpdexx = o->ddivpdezz = o->ddivpdexz = 0.0;
        o->ddivpdp = 0.0;
    } else {
        o->detadexx = dvep_dExx; o->detadezz = dvep_dEzz; o->detadexz = dvep_dExz; o->detadp = dvep_dP;
        o->etaVE = eta_vep;
        o->ddivpdexx = -dQdP * dlamdExx + gdot * dsin_dildExx;
        o->ddivpdezz = -dQdP * dlamdEzz + gdot * dsin_dildEzz;
        o->ddivpdexz = -dQdP * dlamdExz + gdot * dsin_dildExz;
        o->ddivpdp = -dQdP * dlamdP + gdot * dsin_dildP + 0.0;
        inv_eta_diss += 1.0 / eta_vep;
    }
    eta_pwl = pow(2.0 * C_pwl, -1.0) * pow(Tii, 1.0 - n_pwl);
    o->Exx_el = (double)elastic * (Txx - Txx0) / 2.0 / eta_el;
    o->Ezz_el = (double)elastic * (Tzz - Tzz0) / 2.0 / eta_el;
    o->Exz_el = (double)elastic * (Txz - Txz0) / 2.0 / eta_el;
    Exx_pl = gdot * dQdtxx; Ezz_pl = gdot * dQdtzz; Exz_pl = gdot * dQdtxz / 2.0;
    Exx_pwl = Txx / 2.0 / eta_pwl; Ezz_pwl = Tzz / 2.0 / eta_pwl; Exz_pwl = Txz / 2.0 / eta_pwl;
    o->Exx_diss = Exx_pl + Exx_lin + Exx_pwl + Exx_exp + 0.0 + Exx_cst;   /* Exx_gbs stays 0 (:678) */
    o->Ezz_diss = Ezz_pl + Ezz_lin + Ezz_pwl + Ezz_exp + 0.0 + Ezz_cst;
    o->Exz_diss = Exz_pl + Exz_lin + Exz_pwl + Exz_exp + 0.0 + Exz_cst;
    o->Eii_el = (double)elastic * fabs(Tii - Tii0) / 2.0 / eta_el;
    o->Eii_pwl = Tii / 2.0 / eta_pwl;
    o->Eii_lin = Eii_lin;
    o->Eii_cst = Eii_cst;
    o->Eii_exp = Eii_exp;
    o->Eii_gbs = Eii_gbs;
    o->div_pl = divp;
    o->div_el = -(Pc - P0) / (K * dt);
    o->div_r = 0.0;
    double eta = 1.0 / inv_eta_diss;
    o->VEcoeff = eta_ve / eta_el;
    if (elastic == 0) o->VEcoeff = 0.0;
    if (prm->step == 0) o->etaVE = eta;
    o->txx = Txx; o->tzz = Tzz; o->txz = Txz;
    if (eta > maxEta) eta = maxEta;
    if (eta < minEta) eta = minEta;
    {
        const int clamped = o->etaVE > maxEta || o->etaVE < minEta;
        if (o->etaVE > maxEta) o->etaVE = maxEta;
        if (o->etaVE < minEta) o->etaVE = minEta;
        /* optional (not in the reference): tangent of the limited law */
        if (clamped && prm->clamp_tangent) {
            o->detadexx = 0.0; o->detadezz = 0.0; o->detadexz = 0.0; o->detadp = 0.0;
        }
    }
    o->eta = eta;
}

/* Effective strain rates entering the local solve, isotropic form of the
 * elastic-stress correction (RheologyDensity.c:1060-1094 / 1275-1306):
 * returns Exx, Ezz, Exz and the G-tensor (Gxx, Gzz, Gxz). */
static void eff_rates(double exx, double ezz, double exz, double sxx0, double szz0, double sxz0, double etae,
                      double *E) {
    /* ani = d0 = d1 = 0 */
    double Da11 = 2.0 - 2.0 * 0.0 * 0.0, Da12 = 2.0 * 0.0 * 0.0, Da13 = 2.0 * 0.0 * 0.0;
    double Da22 = 2.0 - 2.0 * 0.0 * 0.0, Da23 = -2.0 * 0.0 * 0.0, Da33 = 1.0 + 2.0 * 0.0 * (0.0 - 0.5);
    double a11 = Da33 * Da22 - pow(Da23, 2), a12 = Da13 * Da23 - Da33 * Da12, a13 = Da12 * Da23 - Da13 * Da22;
    double a22 = Da33 * Da11 - pow(Da13, 2), a23 = Da12 * Da13 - Da11 * Da23, a33 = Da11 * Da22 - pow(Da12, 2);
    double det = (Da11 * a11) + (Da12 * a12) + (Da13 * a13);
    double i11 = a11 / det, i12 = a12 / det, i13 = a13 / det, i22 = a22 / det, i23 = a23 / det, i33 = a33 / det;
    double Exx = exx + (i11 * sxx0 + i12 * szz0 + i13 * sxz0) / etae;
    double Ezz = ezz + (i12 * sxx0 + i22 * szz0 + i23 * sxz0) / etae;
    double Exz = exz + (i13 * sxx0 + i23 * szz0 + i33 * sxz0) / 2.0 / etae;
    double gxz = 2.0 * exz + (i13 * sxx0 + i23 * szz0 + i33 * sxz0) / etae;
    E[0] = Exx; E[1] = Ezz; E[2] = Exz;
    E[3] = Exx * (1.0 - 0.0 * 0.0) + Ezz * 0.0 * 0.0 + gxz * 0.0 * 0.0;
    E[4] = Ezz * (1.0 - 0.0 * 0.0) + Exx * 0.0 * 0.0 - gxz * 0.0 * 0.0;
    E[5] = Exx * 0.0 * 0.0 - Exx * 0.0 * 0.0 + gxz * (0.0 * (0.0 - 0.5) + 0.5);
}

#define SETF(ptr, idx, val) do { if (ptr) (ptr)[idx] = (val); } while (0)

int orc_viscosity_grid(const mdz_grid_desc *g, const mdz_materials *mat, const mdz_rheo_params *prm, mdz_fields *f,
                       int *not_conv) {
    int Nx = g->Nx, Nz = g->Nz, ncx = Nx - 1, ncz = Nz - 1, nph = mat->n_phases, avg = prm->eta_avg;
    int nc = ncx * ncz, nv = Nx * Nz, c, p, ve_fail = 0, vp_fail = 0;
    orc_c2v(g, f->div_u, f->div_u_s);                                 /* :979-983 */
    orc_c2v(g, f->T, f->T_s);
    orc_c2v(g, f->p, f->P_s);
    orc_c2v(g, f->d0_n, f->d0_s);
    orc_c2v(g, f->phi0_n, f->phi0_s);
    /* centroids :987-1240 (nodes are independent: the threads' results are
     * those of the serial loop, bit for bit) */
#pragma omp parallel for private(p) reduction(+ : ve_fail, vp_fail) schedule(dynamic, 256)
    for (c = 0; c < nc; c++) {
        double eexp = 0, egbs = 0;
        double eta = 0, eta_phys = 0, VE = 0, sxx = 0, szz = 0, sxz = 0, eel = 0, epl = 0, epwl = 0, elin = 0,
               ecst = 0, dn = 0, xel = 0, xdi = 0, zel = 0, zdi = 0, dexx = 0, dezz = 0, dgxz = 0, dp = 0,
               vxx = 0, vzz = 0, vxz = 0, vp = 0, pc = 0, del = 0, dpl = 0, dr = 0, Wt = 0, We = 0, Wd = 0, X = 0,
               OS = 0;
        if (g->BCp_type[c] != 30 && g->BCp_type[c] != 31) {
            double etae = prm->iselastic == 1 ? prm->dt * f->mu_n[c] : 1.0, E[6];
            eff_rates(f->exxd[c], f->ezzd[c], f->exz_n[c], f->sxxd0[c], f->szzd0[c], f->sxz0_n[c], etae, E);
            for (p = 0; p < nph; p++) {
                double w = f->phase_perc_n[(size_t)p * nc + c];
                if (!(fabs(w) > 1.0e-13)) continue;
                visc_out o;
                orc_visc(p, f->mu_n[c], f->T[c], f->p[c], f->d0_n[c], f->phi0_n[c], f->X0_n ? f->X0_n[c] : 0.0, E[0],
                         E[1], E[2], E[3], E[4], E[5], f->sxxd0[c], f->szzd0[c], f->sxz0_n[c], mat, prm, f->dil_n[c],
                         f->fric_n[c], f->C_n[c], f->p0_n ? f->p0_n[c] : 0.0, f->bet_n[c], &o);
                ve_fail += o.ve_fail; vp_fail += o.vp_fail;
                if (avg == 0) {
                    eta += w * o.etaVE; eta_phys += w * o.eta; dexx += w * o.detadexx; dezz += w * o.detadezz;
                    dgxz += w * o.detadexz / 2.0; dp += w * o.detadp;
                }
                if (avg == 0 || avg == 2) { sxx += w * o.txx; szz += w * o.tzz; sxz += w * o.txz; }
                VE += w * o.VEcoeff; eel += w * o.Eii_el; epl += w * o.Eii_pl; epwl += w * o.Eii_pwl;
                elin += w * o.Eii_lin; ecst += w * o.Eii_cst; dn += w * 1.0 / o.d1;
                eexp += w * o.Eii_exp; egbs += w * o.Eii_gbs;
                xel += w * o.Exx_el; xdi += w * o.Exx_diss; zel += w * o.Ezz_el; zdi += w * o.Ezz_diss;
                Wt += w * (o.txx * f->exxd[c] + o.tzz * f->ezzd[c] + (o.txx + o.tzz) * (f->exxd[c] + f->ezzd[c]) +
                           2.0 * o.txz * f->exz_n[c]);
                Wd += w * (o.txx * o.Exx_diss + o.tzz * o.Ezz_diss + (o.txx + o.tzz) * (o.Exx_diss + o.Ezz_diss) +
                           2.0 * o.txz * o.Exz_diss);
                We += w * (o.txx * o.Exx_el + o.tzz * o.Ezz_el + (o.txx + o.tzz) * (o.Exx_el + o.Ezz_el) +
                           2.0 * o.txz * o.Exz_el);
                vxx += w * o.ddivpdexx; vzz += w * o.ddivpdezz; vxz += w * o.ddivpdexz / 2.0; vp += w * o.ddivpdp;
                pc += w * o.Pcorr; del += w * o.div_el; dpl += w * o.div_pl; dr += w * o.div_r;
                X += w * o.X1; OS += w * o.OverS;
                if (avg == 1) {
                    sxx += w * 1.0 / o.txx; szz += w * 1.0 / o.tzz; sxz += w * 1.0 / o.txz;
                    eta += w * 1.0 / o.etaVE; eta_phys += w * 1.0 / o.eta;
                    dexx += w * o.detadexx / pow(o.etaVE, 2.0); dezz += w * o.detadezz / pow(o.etaVE, 2.0);
                    dgxz += w * o.detadexz / 2.0 / pow(o.etaVE, 2.0); dp += w * o.detadp / pow(o.etaVE, 2.0);
                }
                if (avg == 2) {
                    eta += w * log(o.etaVE); eta_phys += w * log(o.eta);
                    dexx += w * o.detadexx / o.etaVE; dezz += w * o.detadezz / o.etaVE;
                    dgxz += w * o.detadexz / 2.0 / o.etaVE; dp += w * o.detadp / o.etaVE;
                }
            }
            dn = 1.0 / dn;
            if (avg == 1) {
                sxx = 1.0 / sxx; szz = 1.0 / szz; sxz = 1.0 / sxz; eta = 1.0 / eta; eta_phys = 1.0 / eta_phys;
                dexx *= pow(eta, 2.0); dezz *= pow(eta, 2.0); dgxz *= pow(eta, 2.0); dp *= pow(eta, 2.0);
            }
            if (avg == 2) {
                eta = exp(eta); eta_phys = exp(eta_phys);
                dexx *= eta; dezz *= eta; dgxz *= eta; dp *= eta;
            }
        }
        SETF(f->eta_n, c, eta); SETF(f->eta_phys_n, c, eta_phys); SETF(f->VE_n, c, VE);
        SETF(f->sxxd, c, sxx); SETF(f->szzd, c, szz); SETF(f->sxz_n, c, sxz);
        SETF(f->eII_el, c, eel); SETF(f->eII_pl, c, epl); SETF(f->eII_pwl, c, epwl); SETF(f->eII_lin, c, elin);
        SETF(f->eII_cst, c, ecst); SETF(f->d_n, c, dn); SETF(f->eII_exp, c, eexp); SETF(f->eII_gbs, c, egbs);
        SETF(f->exx_el, c, xel); SETF(f->exx_diss, c, xdi); SETF(f->ezz_el, c, zel); SETF(f->ezz_diss, c, zdi);
        SETF(f->detadexx_n, c, dexx); SETF(f->detadezz_n, c, dezz); SETF(f->detadgxz_n, c, dgxz);
        SETF(f->detadp_n, c, dp);
        SETF(f->ddivpdexx_n, c, vxx); SETF(f->ddivpdezz_n, c, vzz); SETF(f->ddivpdgxz_n, c, vxz);
        SETF(f->ddivpdp_n, c, vp);
        SETF(f->p_corr, c, pc); SETF(f->div_u_el, c, del); SETF(f->div_u_pl, c, dpl); SETF(f->div_u_r, c, dr);
        SETF(f->Wtot, c, Wt); SETF(f->Wel, c, We); SETF(f->Wdiss, c, Wd); SETF(f->X_n, c, X);
        SETF(f->OverS_n, c, OS);
    }
    /* vertices :1246-1410 */
#pragma omp parallel for private(p) reduction(+ : ve_fail, vp_fail) schedule(dynamic, 256)
    for (c = 0; c < nv; c++) {
        double VE = 0, sxz = 0, eta_phys = 0, eta = 0, zel = 0, zdi = 0, dexx = 0, dezz = 0, dgxz = 0, dp = 0, X = 0,
               OS = 0;
        if (g->BCg_type[c] != 30) {
            double etae = prm->iselastic == 1 ? prm->dt * f->mu_s[c] : 1.0, E[6];
            eff_rates(f->exxd_s[c], f->ezzd_s[c], f->exz[c], f->sxxd0_s[c], f->szzd0_s[c], f->sxz0[c], etae, E);
            for (p = 0; p < nph; p++) {
                double w = f->phase_perc_s[(size_t)p * nv + c];
                if (!(fabs(w) > 1.0e-13)) continue;
                visc_out o;
                orc_visc(p, f->mu_s[c], f->T_s[c], f->P_s[c], f->d0_s[c], f->phi0_s[c], f->X0_s ? f->X0_s[c] : 0.0,
                         E[0], E[1], E[2], E[3], E[4], E[5], f->sxxd0_s[c], f->szzd0_s[c], f->sxz0[c], mat, prm,
                         f->dil_s[c], f->fric_s[c], f->C_s[c], f->p0_s ? f->p0_s[c] : 0.0, f->bet_s[c], &o);
                ve_fail += o.ve_fail; vp_fail += o.vp_fail;
                if (avg == 0) {
                    eta += w * o.etaVE; eta_phys += w * o.eta; dexx += w * o.detadexx; dezz += w * o.detadezz;
                    dgxz += w * o.detadexz / 2.0; dp += w * o.detadp;
                }
                if (avg == 0 || avg == 2) sxz += w * o.txz;
                VE += w * o.VEcoeff; zel += w * o.Exz_el; zdi += w * o.Exz_diss; OS += w * o.OverS; X += w * o.X1;
                if (avg == 1) {
                    sxz += w * 1.0 / o.txz; eta += w * 1.0 / o.etaVE; eta_phys += w * 1.0 / o.eta;
                    dexx += w * o.detadexx / pow(o.etaVE, 2.0); dezz += w * o.detadezz / pow(o.etaVE, 2.0);
                    dgxz += w * o.detadexz / 2.0 / pow(o.etaVE, 2.0); dp += w * o.detadp / pow(o.etaVE, 2.0);
                }
                if (avg == 2) {
                    eta += w * log(o.etaVE); eta_phys += w * log(o.eta);
                    dexx += w * o.detadexx / o.etaVE; dezz += w * o.detadezz / o.etaVE;
                    dgxz += w * o.detadexz / 2.0 / o.etaVE; dp += w * o.detadp / o.etaVE;
                }
            }
            if (avg == 1) {
                sxz = 1.0 / sxz; eta = 1.0 / eta; eta_phys = 1.0 / eta_phys;
                dexx *= pow(eta, 2.0); dezz *= pow(eta, 2.0); dgxz *= pow(eta, 2.0); dp *= pow(eta, 2.0);
            }
            if (avg == 2) {
                eta = exp(eta); eta_phys = exp(eta_phys);
                dexx *= eta; dezz *= eta; dgxz *= eta; dp *= eta;
            }
        }
        SETF(f->VE_s, c, VE); SETF(f->sxz, c, sxz); SETF(f->eta_phys_s, c, eta_phys); SETF(f->eta_s, c, eta);
        SETF(f->exz_el, c, zel); SETF(f->exz_diss, c, zdi);
        SETF(f->detadexx_s, c, dexx); SETF(f->detadezz_s, c, dezz); SETF(f->detadgxz_s, c, dgxz);
        SETF(f->detadp_s, c, dp); SETF(f->X_s, c, X); SETF(f->OverS_s, c, OS);
    }
    if (not_conv) { not_conv[0] = ve_fail; not_conv[1] = vp_fail; }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* RheologicalOperators, isotropic (RheologyDensity.c:713-954). */
int orc_rheo_operators(const mdz_grid_desc *g, const mdz_rheo_params *prm, mdz_fields *f, int jacobian) {
    int Nx = g->Nx, Nz = g->Nz, nc = (Nx - 1) * (Nz - 1), nv = Nx * Nz, k;
    for (k = 0; k < nc; k++) {
        double d11 = 0, d12 = 0, d13 = 0, d14 = 0, d21 = 0, d22 = 0, d23 = 0, d24 = 0;
        if (g->BCp_type[k] != 30 && g->BCp_type[k] != 31) {
            double eta = f->eta_n[k];
            if (!jacobian) {
                d11 = 2.0 * eta - 2.0 * 0.0 * 0.0 * eta; d12 = 2.0 * 0.0 * 0.0 * eta; d13 = 2.0 * 0.0 * 0.0 * eta;
                d21 = 2.0 * 0.0 * 0.0 * eta; d22 = 2.0 * eta - 2.0 * 0.0 * 0.0 * eta; d23 = -2.0 * 0.0 * 0.0 * eta;
            } else {
                double etae = prm->iselastic == 1 ? prm->dt * f->mu_n[k] : 1.0, E[6], K = 0.0, dt = prm->dt;
                eff_rates(f->exxd[k], f->ezzd[k], f->exz_n[k], f->sxxd0[k], f->szzd0[k], f->sxz0_n[k], etae, E);
                double Gxx = E[3], Gzz = E[4];
                d11 = 2.0 * eta - 2.0 * 0.0 * 0.0 * eta + 2.0 * f->detadexx_n[k] * Gxx - K * dt * f->ddivpdexx_n[k];
                d12 = 2.0 * 0.0 * 0.0 * eta + 2.0 * f->detadezz_n[k] * Gxx - K * dt * f->ddivpdezz_n[k];
                d13 = 2.0 * 0.0 * 0.0 * eta + 2.0 * f->detadgxz_n[k] * Gxx - K * dt * f->ddivpdgxz_n[k];
                d14 = 2.0 * f->detadp_n[k] * E[0] - K * dt * f->ddivpdp_n[k];
                d21 = 2.0 * 0.0 * 0.0 * eta + 2.0 * f->detadexx_n[k] * Gzz - K * dt * f->ddivpdexx_n[k];
                d22 = 2.0 * eta - 2.0 * 0.0 * 0.0 * eta + 2.0 * f->detadezz_n[k] * Gzz - K * dt * f->ddivpdezz_n[k];
                d23 = -2.0 * 0.0 * 0.0 * eta + 2.0 * f->detadgxz_n[k] * Gzz - K * dt * f->ddivpdgxz_n[k];
                d24 = 2.0 * f->detadp_n[k] * E[1] - K * dt * f->ddivpdp_n[k];
            }
        }
        f->D11_n[k] = d11; f->D12_n[k] = d12; f->D13_n[k] = d13; f->D14_n[k] = d14;
        f->D21_n[k] = d21; f->D22_n[k] = d22; f->D23_n[k] = d23; f->D24_n[k] = d24;
    }
    for (k = 0; k < nv; k++) {
        double d31 = 0, d32 = 0, d33 = 0, d34 = 0;
        if (g->BCg_type[k] != 30) {
            double eta = f->eta_s[k];
            if (!jacobian) {
                d31 = 2.0 * 0.0 * 0.0 * eta; d32 = -2.0 * 0.0 * 0.0 * eta; d33 = eta + 2.0 * 0.0 * (0.0 - 0.5) * eta;
            } else {
                double etae = prm->iselastic == 1 ? prm->dt * f->mu_s[k] : 1.0, E[6];
                eff_rates(f->exxd_s[k], f->ezzd_s[k], f->exz[k], f->sxxd0_s[k], f->szzd0_s[k], f->sxz0[k], etae, E);
                double Gxz = E[5];
                d31 = 2.0 * 0.0 * 0.0 * eta + 2.0 * f->detadexx_s[k] * Gxz;
                d32 = -2.0 * 0.0 * 0.0 * eta + 2.0 * f->detadezz_s[k] * Gxz;
                d33 = eta + 2.0 * 0.0 * (0.0 - 0.5) * eta + 2.0 * f->detadgxz_s[k] * Gxz;
                d34 = 2.0 * f->detadp_s[k] * E[2];
            }
        }
        f->D31_s[k] = d31; f->D32_s[k] = d32; f->D33_s[k] = d33; f->D34_s[k] = d34;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* EvaluateRHS (StokesRoutines.c:922-1133), incompressible, non-polar. */
int orc_rhs(const mdz_grid_desc *g, const mdz_rheo_params *prm, double gx, double gz, mdz_fields *f) {
    int Nx = g->Nx, Nz = g->Nz, NzVx = Nz + 1, NxVz = Nx + 1, ncx = Nx - 1, k, l;
    double dx = g->dx, dz = g->dz, dt = prm->dt;
    for (l = 0; l < NzVx; l++)
        for (k = 0; k < Nx; k++) {
            int c = k + l * Nx, c2 = k + (l - 1) * ncx;
            double r = 0.0;
            if (f->gx) f->gx[c] = gx;
            if (l > 0 && l < NzVx - 1) {
                signed char t = g->BCu_type[c];
                if (t == -1 || t == 2 || t == -2) {
                    int iPrW = c2 - 1, iPrE = c2, ixyN = c, ixyS = c - Nx, iVxS = c - Nx, iVxN = c + Nx;
                    double inW = 0, inE = 0, inS = 0, inN = 0;
                    if (k > 0 && g->BCp_type[iPrW] == -1) inW = 1.0;
                    if (k < Nx - 1 && g->BCp_type[iPrE] == -1) inE = 1.0;
                    if (g->BCg_type[ixyS] != 30 && g->BCu_type[iVxS] != 13) inS = 1.0;
                    if (g->BCg_type[ixyN] != 30 && g->BCu_type[iVxN] != 13) inN = 1.0;
                    double rhoVx = 0.5 * (f->rho_s[ixyS] + f->rho_s[ixyN]);
                    r = -gx * rhoVx;
                    if (prm->iselastic == 1 && k > 0 && k < Nx - 1) {
                        if (inE) r -= 1.0 / dx * (f->eta_n[iPrE] / (f->mu_n[iPrE] * dt) * f->sxxd0[iPrE]);
                        if (inW) r -= 1.0 / dx * (-f->eta_n[iPrW] / (f->mu_n[iPrW] * dt) * f->sxxd0[iPrW]);
                        if (inN) r -= 1.0 / dz * (f->eta_s[ixyN] / (f->mu_s[ixyN] * dt) * f->sxz0[ixyN]);
                        if (inS) r -= 1.0 / dz * (-f->eta_s[ixyS] / (f->mu_s[ixyS] * dt) * f->sxz0[ixyS]);
                    }
                }
            }
            f->roger_x[c] = -r;
        }
    for (l = 0; l < Nz; l++)
        for (k = 0; k < NxVz; k++) {
            int c = k + l * NxVz, c1 = k + l * Nx - 1, c2 = k - 1 + (l - 1) * ncx;
            double r = 0.0;
            if (f->gz) f->gz[c] = gz;
            if (k > 0 && k < NxVz - 1 && g->BCv_type[c] == -1) {
                int iPrS = c2, iPrN = c2 + ncx, ixyE = c1 + 1, ixyW = c1, iVyW = c - 1, iVyE = c + 1;
                double inS = 0, inN = 0, inW = 0, inE = 0;
                if (l > 0 && g->BCp_type[iPrS] == -1) inS = 1.0;
                if (l < Nz - 1 && g->BCp_type[iPrN] == -1) inN = 1.0;
                if (g->BCg_type[ixyW] != 30 && g->BCv_type[iVyW] != 13) inW = 1.0;
                if (g->BCg_type[ixyE] != 30 && g->BCv_type[iVyE] != 13) inE = 1.0;
                double rhoVz = 0.5 * ((l > 0 ? f->rho_n[iPrS] : 0.0) + (l < Nz - 1 ? f->rho_n[iPrN] : 0.0));
                r = -gz * rhoVz;
                if (prm->iselastic == 1 && l > 0 && l < Nz - 1) {
                    if (inN) r -= 1.0 / dz * (f->eta_n[iPrN] / (f->mu_n[iPrN] * dt) * (f->szzd0[iPrN]));
                    if (inS) r -= 1.0 / dz * (-f->eta_n[iPrS] / (f->mu_n[iPrS] * dt) * (f->szzd0[iPrS]));
                    if (inE) r -= 1.0 / dx * (f->eta_s[ixyE] / (f->mu_s[ixyE] * dt) * f->sxz0[ixyE]);
                    if (inW) r -= 1.0 / dx * (-f->eta_s[ixyW] / (f->mu_s[ixyW] * dt) * f->sxz0[ixyW]);
                }
            }
            f->roger_z[c] = -r;
        }
    for (k = 0; k < ncx * (Nz - 1); k++)
        if (g->BCp_type[k] != 30 && g->BCp_type[k] != 31) f->rhs_p[k] = 0.0;
    return 0;
}
