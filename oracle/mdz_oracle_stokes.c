/*
 * CPU oracle, part 3 (test infrastructure only): the decoupled Stokes
 * residual and the linear Picard / Newton operators, restated from MDOODZ 6.0
 * (SOURCE/StokesAssemblyDecoupled.c) for inner equations with Dirichlet and
 * free-slip boundaries.
 *
 * Picard rows are written in the reference's coefficient form
 * (Xmomentum_InnerNodesDecoupled :109-234, Zmomentum_InnerNodesDecoupled
 * :796-1167, Continuity_InnerNodesDecoupled :62-103).  Newton rows
 * (Xjacobian/Zjacobian_InnerNodesDecoupled3 :3034-3833) are evaluated by first
 * forming the strain rates of the whole input field and then, row by row,
 * the flag-weighted averages and tangent stresses the reference's
 * coefficients encode.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "mdz_oracle.h"

#define IN(b) ((b) ? 1.0 : 0.0)

/* Picard x-momentum row (k, l): returns the row value before the RHS. */
static double picard_x(const mdz_grid_desc *g, const mdz_fields *f, const double *u, const double *v,
                       const double *p, int k, int l) {
    int nx = g->Nx, ncx = nx - 1, nxvz = nx + 1;
    int c1 = k + l * nx, c2 = k - 1 + (l - 1) * ncx, c3 = k + l * nxvz;
    int iVxC = c1, iVxW = c1 - 1, iVxE = c1 + 1, iVxS = c1 - nx, iVxN = c1 + nx;
    int iVzSW = c3 - nxvz, iVzSE = c3 - nxvz + 1, iVzNW = c3, iVzNE = c3 + 1, iPrW = c2, iPrE = c2 + 1;
    int ixyN = c1, ixyS = c1 - nx;
    double D11E = f->D11_n[iPrE], D11W = f->D11_n[iPrW], D33N = f->D33_s[ixyN], D33S = f->D33_s[ixyS];
    double inW = IN(g->BCp_type[iPrW] == -1), inE = IN(g->BCp_type[iPrE] == -1);
    double inS = IN(g->BCg_type[ixyS] != 30 && g->BCu_type[ixyS] != 13);
    double inN = IN(g->BCg_type[c1] != 30 && g->BCu_type[c1 + nx] != 13);
    double dx = g->dx, dz = g->dz, comp = 1.0;
    double uW = D11W * inW * ((1.0 / 3.0) * comp / dx - 1.0 / dx) / dx;
    double uC = -(-D33N * inN / dz - D33S * inS / dz) / dz -
                (D11E * inE * ((1.0 / 3.0) * comp / dx - 1 / dx) - D11W * inW * (-1.0 / 3.0 * comp / dx + 1.0 / dx)) / dx;
    double uE = -D11E * inE * (-1.0 / 3.0 * comp / dx + 1.0 / dx) / dx;
    double uS = -D33S * inS / pow(dz, 2.0), uN = -D33N * inN / pow(dz, 2.0);
    double vSW = (1.0 / 3.0) * D11W * comp * inW / (dx * dz) - D33S * inS / (dx * dz);
    double vSE = -1.0 / 3.0 * D11E * comp * inE / (dx * dz) + D33S * inS / (dx * dz);
    double vNW = -1.0 / 3.0 * D11W * comp * inW / (dx * dz) + D33N * inN / (dx * dz);
    double vNE = (1.0 / 3.0) * D11E * comp * inE / (dx * dz) - D33N * inN / (dx * dz);
    double pW = 0, pE = 0;
    if (g->BCp_type[iPrE] != 30 && g->BCp_type[iPrW] != 30) { pW = -1.0 / dx; pE = 1.0 / dx; }
    double F = uC * u[iVxC] + pW * p[iPrW] + pE * p[iPrE];
    F += vSE * v[iVzSE] + vSW * v[iVzSW] + vNE * v[iVzNE] + vNW * v[iVzNW];
    F += uS * u[iVxS] + uN * u[iVxN] + uW * u[iVxW] + uE * u[iVxE];
    return F;
}

static double picard_z(const mdz_grid_desc *g, const mdz_fields *f, const double *u, const double *v,
                       const double *p, int k, int l) {
    int nx = g->Nx, ncx = nx - 1, nxvz = nx + 1;
    int c3 = k + l * nxvz, c1 = k + l * nx, c2 = k - 1 + (l - 1) * ncx;
    double D22S = f->D22_n[c2], D22N = f->D22_n[c2 + ncx], D33E = f->D33_s[c1], D33W = f->D33_s[c1 - 1];
    double inS = 0, inN = 0;
    if (g->BCv_type[c3 - nxvz] != 30 && g->BCv_type[c3 + nxvz] != 30) { inS = 1; inN = 1; }
    if (g->BCp_type[c2] == -1) inS = 1;
    if (g->BCp_type[c2 + ncx] == -1) inN = 1;
    double inW = IN(g->BCg_type[c1 - 1] != 30 && g->BCv_type[c3 - 1] != 13);
    double inE = IN(g->BCg_type[c1] != 30 && g->BCv_type[c3 + 1] != 13);
    double dx = g->dx, dz = g->dz, comp = 1.0;
    double vW = -D33W * inW / pow(dx, 2);
    double vC = -(D22N * inN * ((1.0 / 3.0) * comp / dz - 1 / dz) - D22S * inS * (-1.0 / 3.0 * comp / dz + 1.0 / dz)) / dz -
                (-D33E * inE / dx - D33W * inW / dx) / dx;
    double vE = -D33E * inE / pow(dx, 2);
    double vS = D22S * inS * ((1.0 / 3.0) * comp / dz - 1 / dz) / dz;
    double vN = -D22N * inN * (-1.0 / 3.0 * comp / dz + 1.0 / dz) / dz;
    double uSW = (1.0 / 3.0) * D22S * comp * inS / (dx * dz) - D33W * inW / (dx * dz);
    double uSE = -1.0 / 3.0 * D22S * comp * inS / (dx * dz) + D33E * inE / (dx * dz);
    double uNW = -1.0 / 3.0 * D22N * comp * inN / (dx * dz) + D33W * inW / (dx * dz);
    double uNE = (1.0 / 3.0) * D22N * comp * inN / (dx * dz) - D33E * inE / (dx * dz);
    double pS = 0, pN = 0;
    if (g->BCp_type[c2] != 30 && g->BCp_type[c2 + ncx] != 30) { pS = -1.0 / dz; pN = 1.0 / dz; }
    double F = vC * v[c3] + pS * p[c2] + pN * p[c2 + ncx];
    F += vS * v[c3 - nxvz] + vW * v[c3 - 1] + vE * v[c3 + 1] + vN * v[c3 + nxvz];
    F += uSW * u[c1 - 1] + uSE * u[c1] + uNW * u[c1 + nx - 1] + uNE * u[c1 + nx];
    return F;
}

static double cont_row(const mdz_grid_desc *g, const double *u, const double *v, int k, int l) {
    int nx = g->Nx, nxvz = nx + 1, c1 = k + (l + 1) * nx, c3 = k + l * nxvz + 1;
    double uW = 0, uE = 0, vS = 0, vN = 0;
    if (g->BCu_type[c1] != 13) uW = -1.0 / g->dx;
    if (g->BCu_type[c1 + 1] != 13) uE = 1.0 / g->dx;
    if (g->BCv_type[c3] != 13) vS = -1.0 / g->dz;
    if (g->BCv_type[c3 + nxvz] != 13) vN = 1.0 / g->dz;
    return uW * u[c1] + uE * u[c1 + 1] + vS * v[c3] + vN * v[c3 + nxvz];
}

/* Newton rows: strain rates of the input first (exx', ezz' per centroid, gxz per vertex). */
typedef struct { double *exx, *ezz, *gxz; const double *v; } rates_t;

static rates_t rates(const mdz_grid_desc *g, const double *u, const double *v) {
    int nx = g->Nx, nz = g->Nz, ncx = nx - 1, ncz = nz - 1, nxvz = nx + 1;
    rates_t r;
    r.exx = calloc((size_t)ncx * ncz, sizeof(double));
    r.ezz = calloc((size_t)ncx * ncz, sizeof(double));
    r.gxz = calloc((size_t)nx * nz, sizeof(double));
    r.v = v;
    for (int l = 0; l < ncz; l++)
        for (int k = 0; k < ncx; k++) {
            int cu = k + (l + 1) * nx, cv = k + 1 + l * nxvz;
            double dudx = (u[cu + 1] - u[cu]) / g->dx, dvdz = (v[cv + nxvz] - v[cv]) / g->dz;
            r.exx[k + l * ncx] = dudx - (dudx + dvdz) / 3.0;
            r.ezz[k + l * ncx] = dvdz - (dudx + dvdz) / 3.0;
        }
    for (int l = 0; l < nz; l++)
        for (int k = 0; k < nx; k++) {
            int cu = k + l * nx, cv = k + l * nxvz;
            r.gxz[k + l * nx] = (u[cu + nx] - u[cu]) / g->dz + (v[cv + 1] - v[cv]) / g->dx;
        }
    return r;
}

static double wnorm(double s) { return s > 1.0 ? 1.0 / s : s; }

static double newton_x(const mdz_grid_desc *g, const mdz_fields *f, const rates_t *R, const double *p, int k, int l) {
    int nx = g->Nx, ncx = nx - 1, nzvx = g->Nz + 1;
    int c1 = k + l * nx, c2 = k - 1 + (l - 1) * ncx;
    int W = c2, E = c2 + 1, N = c1, S = c1 - nx;
    double inW = IN(g->BCp_type[W] == -1), inE = IN(g->BCp_type[E] == -1);
    double inS = IN(g->BCg_type[S] != 30 && g->BCu_type[c1 - nx] != 13);
    double inN = IN(g->BCg_type[N] != 30 && g->BCu_type[c1 + nx] != 13);
    double inSWc = 0, inSEc = 0, inNWc = 0, inNEc = 0;
    if (l > 1) { inSWc = IN(g->BCp_type[W - ncx] == -1); inSEc = IN(g->BCp_type[E - ncx] == -1); }
    if (l < nzvx - 2) { inNWc = IN(g->BCp_type[W + ncx] == -1); inNEc = IN(g->BCp_type[E + ncx] == -1); }
    double inSWv = IN(g->BCg_type[S - 1] != 30), inNWv = IN(g->BCg_type[N - 1] != 30);
    double inSEv = IN(g->BCg_type[S + 1] != 30), inNEv = IN(g->BCg_type[N + 1] != 30);
    double wE = wnorm(inN + inS + inNEv + inSEv), wW = wnorm(inN + inS + inNWv + inSWv);
    double wS = wnorm(inW + inE + inSWc + inSEc), wN = wnorm(inW + inE + inNWc + inNEc);
    const double *gx = R->gxz, *ex = R->exx, *ez = R->ezz;
    double gE = wE * (inN * gx[N] + inS * gx[S] + inNEv * gx[N + 1] + inSEv * gx[S + 1]);
    double gW = wW * (inN * gx[N] + inS * gx[S] + inNWv * gx[N - 1] + inSWv * gx[S - 1]);
#define CV(arr, idx, flag) ((flag) != 0.0 ? (arr)[idx] : 0.0)
    double TxxE = f->D11_n[E] * ex[E] + f->D12_n[E] * ez[E] + f->D13_n[E] * gE + f->D14_n[E] * p[E];
    double TxxW = f->D11_n[W] * ex[W] + f->D12_n[W] * ez[W] + f->D13_n[W] * gW + f->D14_n[W] * p[W];
    double exS = wS * (inW * ex[W] + inE * ex[E] + inSWc * CV(ex, W - ncx, inSWc) + inSEc * CV(ex, E - ncx, inSEc));
    double ezS = wS * (inW * ez[W] + inE * ez[E] + inSWc * CV(ez, W - ncx, inSWc) + inSEc * CV(ez, E - ncx, inSEc));
    double pS = wS * (inW * p[W] + inE * p[E] + inSWc * CV(p, W - ncx, inSWc) + inSEc * CV(p, E - ncx, inSEc));
    double exN = wN * (inW * ex[W] + inE * ex[E] + inNWc * CV(ex, W + ncx, inNWc) + inNEc * CV(ex, E + ncx, inNEc));
    double ezN = wN * (inW * ez[W] + inE * ez[E] + inNWc * CV(ez, W + ncx, inNWc) + inNEc * CV(ez, E + ncx, inNEc));
    double pN = wN * (inW * p[W] + inE * p[E] + inNWc * CV(p, W + ncx, inNWc) + inNEc * CV(p, E + ncx, inNEc));
    double TxzS = f->D31_s[S] * exS + f->D32_s[S] * ezS + f->D33_s[S] * gx[S] + f->D34_s[S] * pS;
    double TxzN = f->D31_s[N] * exN + f->D32_s[N] * ezN + f->D33_s[N] * gx[N] + f->D34_s[N] * pN;
    return -(inE * TxxE - inW * TxxW) / g->dx - (inN * TxzN - inS * TxzS) / g->dz + (inE * p[E] - inW * p[W]) / g->dx;
}

static double newton_z(const mdz_grid_desc *g, const mdz_fields *f, const rates_t *R, const double *p, int k, int l) {
    int nx = g->Nx, ncx = nx - 1, nxvz = nx + 1, nz = g->Nz;
    int c3 = k + l * nxvz, c1 = k + l * nx, c2 = k - 1 + (l - 1) * ncx;
    int S = c2, N = c2 + ncx, Wv = c1 - 1, Ev = c1;
    double inS = IN(g->BCp_type[S] == -1), inN = IN(g->BCp_type[N] == -1);
    double inW = IN(g->BCg_type[Wv] != 30 && g->BCv_type[c3 - 1] != 13);
    double inE = IN(g->BCg_type[Ev] != 30 && g->BCv_type[c3 + 1] != 13);
    double inSWc = 0, inNWc = 0, inSEc = 0, inNEc = 0, inSWv = 0, inSEv = 0, inNWv = 0, inNEv = 0;
    if (k > 1 || (k == 1 && g->BCv_type[c3 - 1] == -1)) { inSWc = IN(g->BCp_type[S - 1] == -1); inNWc = IN(g->BCp_type[N - 1] == -1); }
    if (k < nxvz - 2 || (k == nxvz - 2 && g->BCv_type[c3 + 1] == -1)) { inSEc = IN(g->BCp_type[S + 1] == -1); inNEc = IN(g->BCp_type[N + 1] == -1); }
    if (l > 0) { inSWv = IN(g->BCg_type[Wv - nx] != 30); inSEv = IN(g->BCg_type[Ev - nx] != 30); }
    if (l < nz - 1) { inNWv = IN(g->BCg_type[Wv + nx] != 30); inNEv = IN(g->BCg_type[Ev + nx] != 30); }
    double wE = wnorm(inN + inS + inNEc + inSEc), wW = wnorm(inN + inS + inNWc + inSWc);
    double wS = wnorm(inW + inE + inSWv + inSEv), wN = wnorm(inW + inE + inNWv + inNEv);
    const double *gx = R->gxz, *ex = R->exx, *ez = R->ezz;
    double gS = wS * (inW * gx[Wv] + inE * gx[Ev] + inSWv * CV(gx, Wv - nx, inSWv) + inSEv * CV(gx, Ev - nx, inSEv));
    double gN = wN * (inW * gx[Wv] + inE * gx[Ev] + inNWv * CV(gx, Wv + nx, inNWv) + inNEv * CV(gx, Ev + nx, inNEv));
    double TzzS = f->D21_n[S] * ex[S] + f->D22_n[S] * ez[S] + f->D23_n[S] * gS + f->D24_n[S] * p[S];
    double TzzN = f->D21_n[N] * ex[N] + f->D22_n[N] * ez[N] + f->D23_n[N] * gN + f->D24_n[N] * p[N];
    double exW = wW * (inN * ex[N] + inS * ex[S] + inNWc * CV(ex, N - 1, inNWc) + inSWc * CV(ex, S - 1, inSWc));
    double ezW = wW * (inN * ez[N] + inS * ez[S] + inNWc * CV(ez, N - 1, inNWc) + inSWc * CV(ez, S - 1, inSWc));
    double pW = wW * (inN * p[N] + inS * p[S] + inNWc * CV(p, N - 1, inNWc) + inSWc * CV(p, S - 1, inSWc));
    double exE = wE * (inN * ex[N] + inS * ex[S] + inNEc * CV(ex, N + 1, inNEc) + inSEc * CV(ex, S + 1, inSEc));
    double ezE = wE * (inN * ez[N] + inS * ez[S] + inNEc * CV(ez, N + 1, inNEc) + inSEc * CV(ez, S + 1, inSEc));
    double pE = wE * (inN * p[N] + inS * p[S] + inNEc * CV(p, N + 1, inNEc) + inSEc * CV(p, S + 1, inSEc));
    double TxzW = f->D31_s[Wv] * exW + f->D32_s[Wv] * ezW + f->D33_s[Wv] * gx[Wv] + f->D34_s[Wv] * pW;
    double TxzE = f->D31_s[Ev] * exE + f->D32_s[Ev] * ezE + f->D33_s[Ev] * gx[Ev] + f->D34_s[Ev] * pE;
#undef CV
    double r = -(inN * TzzN - inS * TzzS) / g->dz - (inE * TxzE - inW * TxzW) / g->dx + (p[N] - p[S]) / g->dz;
    /* The reference's Jacobian assembles the diagonal Vz neighbours only where
     * they are plain unknowns (tag -1, StokesAssemblyDecoupled.c:3669-3711):
     * a Neumann wall node (tag 2) south-west / south-east of the first inner
     * row, or north-west / north-east of the last, has no entry in that row.
     * Its coupling (the coefficients of :3573-3576, comp = 1) is taken out. */
    const double *vv = R->v;
    const double ixz = 1.0 / (g->dx * g->dz);
    if (l == 1) {
        if (g->BCv_type[c3 - nxvz - 1] == 2)
            r -= (-3.0 * f->D23_n[S] * inS * inSWv * wS + f->D31_s[Wv] * inSWc * inW * wW -
                  2.0 * f->D32_s[Wv] * inSWc * inW * wW) / 3.0 * ixz * vv[c3 - nxvz - 1];
        if (g->BCv_type[c3 - nxvz + 1] == 2)
            r -= (3.0 * f->D23_n[S] * inS * inSEv * wS - f->D31_s[Ev] * inE * inSEc * wE +
                  2.0 * f->D32_s[Ev] * inE * inSEc * wE) / 3.0 * ixz * vv[c3 - nxvz + 1];
    }
    if (l == nz - 2) {
        if (g->BCv_type[c3 + nxvz - 1] == 2)
            r -= (3.0 * f->D23_n[N] * inN * inNWv * wN - f->D31_s[Wv] * inNWc * inW * wW +
                  2.0 * f->D32_s[Wv] * inNWc * inW * wW) / 3.0 * ixz * vv[c3 + nxvz - 1];
        if (g->BCv_type[c3 + nxvz + 1] == 2)
            r -= (-3.0 * f->D23_n[N] * inN * inNEv * wN + f->D31_s[Ev] * inE * inNEc * wE -
                  2.0 * f->D32_s[Ev] * inE * inNEc * wE) / 3.0 * ixz * vv[c3 + nxvz + 1];
    }
    return r;
}

int orc_stokes_apply(const mdz_grid_desc *g, const mdz_fields *f, int jacobian, int residual, const double *u,
                     const double *v, const double *p, double *yu, double *yv, double *yp) {
    int nx = g->Nx, nz = g->Nz, ncx = nx - 1, ncz = nz - 1, nxvz = nx + 1;
    double celvol = g->dx * g->dz;
    rates_t R = {0, 0, 0, 0};
    if (jacobian) R = rates(g, u, v);
    /* rows are independent: threaded loops give the serial loop's bits */
#pragma omp parallel for schedule(static)
    for (int l = 0; l <= nz; l++)
        for (int k = 0; k < nx; k++) {
            int c = k + l * nx;
            double r = 0.0;
            if (g->BCu_type[c] == -1) {
                r = jacobian ? newton_x(g, f, &R, p, k, l) : picard_x(g, f, u, v, p, k, l);
                if (residual) r -= f->roger_x[c];
                r *= celvol;
            }
            yu[c] = r;
        }
#pragma omp parallel for schedule(static)
    for (int l = 0; l < nz; l++)
        for (int k = 0; k <= nx; k++) {
            int c = k + l * nxvz;
            double r = 0.0;
            if (g->BCv_type[c] == -1) {
                r = jacobian ? newton_z(g, f, &R, p, k, l) : picard_z(g, f, u, v, p, k, l);
                if (residual) r -= f->roger_z[c];
                r *= celvol;
            }
            yv[c] = r;
        }
#pragma omp parallel for schedule(static)
    for (int l = 0; l < ncz; l++)
        for (int k = 0; k < ncx; k++) {
            int c = k + l * ncx;
            double r = 0.0;
            if (g->BCp_type[c] == -1) {
                r = cont_row(g, u, v, k, l);
                if (residual) r -= f->rhs_p[c];
                r *= celvol;
            }
            yp[c] = r;
        }
    free(R.exx); free(R.ezz); free(R.gxz);
    return 0;
}

/* EvaluateStokesResidualDecoupled (SOURCE/StokesRoutines.c:839-920): residual
 * of the current state with p_corr, norms sqrt(sum F^2 / n) per block. */
int orc_residual(const mdz_grid_desc *g, mdz_fields *f, double *norms3) {
    orc_stokes_apply(g, f, 0, 1, f->u, f->v, f->p_corr, f->ru, f->rv, f->rp);
    double s[3] = {0, 0, 0};
    int n[3] = {0, 0, 0};
    size_t nu = (size_t)g->Nx * (g->Nz + 1), nv = (size_t)(g->Nx + 1) * g->Nz, np = (size_t)(g->Nx - 1) * (g->Nz - 1);
    for (size_t i = 0; i < nu; i++) if (g->BCu_type[i] == -1) { s[0] += f->ru[i] * f->ru[i]; n[0]++; }
    for (size_t i = 0; i < nv; i++) if (g->BCv_type[i] == -1) { s[1] += f->rv[i] * f->rv[i]; n[1]++; }
    for (size_t i = 0; i < np; i++) if (g->BCp_type[i] == -1) { s[2] += f->rp[i] * f->rp[i]; n[2]++; }
    for (int q = 0; q < 3; q++) norms3[q] = sqrt(s[q] / (n[q] ? n[q] : 1));
    return 0;
}
