/*
 * CPU oracle (test infrastructure only): plain-C restatement of the MDOODZ 6.0
 * hot path.  See mdz_oracle.h.  Written for clarity over speed: serial loops,
 * the scatter form of the reference's algorithms, FP64 throughout, compiled
 * with -ffp-contract=off so that no fused multiply-add changes a result.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "mdz_oracle.h"

/* Lines, sizes and tags of a node set, selected as the reference's `centroid`
 * argument does (SOURCE/ParticleRoutines.c:3241-3264). */
typedef struct { int nx, nz; const double *X, *Z; } nodeset_t;

static nodeset_t nodeset(const mdz_grid_desc *g, int centroid) {
    nodeset_t s;
    if (centroid == 1) { s.nx = g->Nx - 1; s.nz = g->Nz - 1; s.X = g->xc; s.Z = g->zc; }
    else if (centroid == 0) { s.nx = g->Nx; s.nz = g->Nz; s.X = g->xg; s.Z = g->zg; }
    else if (centroid == -1) { s.nx = g->Nx; s.nz = g->Nz + 1; s.X = g->xg; s.Z = g->zvx; }
    else { s.nx = g->Nx + 1; s.nz = g->Nz; s.X = g->xvz; s.Z = g->zg; }
    return s;
}

static int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* ------------------------------------------------------------------------ */
/* P2Mastah: SOURCE/ParticleRoutines.c:3226-3537.                            */
int orc_p2g(const mdz_grid_desc *g, int n, const double *x, const double *z, const int *phase, int n_phases,
            const double *mat_prop, double *node_field, const signed char *node_type, int flag, int avg, int prop,
            int centroid, int itp_stencil, double *phase_perc) {
    nodeset_t s = nodeset(g, centroid);
    int nn = s.nx * s.nz, k, p, i;
    double dx = g->dx, dz = g->dz;
    double hx = itp_stencil == 9 ? 3.0 * dx / 2.0 : dx / 2.0;   /* :3269-3272 */
    double hz = itp_stencil == 9 ? 3.0 * dz / 2.0 : dz / 2.0;
    double *W = calloc(nn, sizeof(double)), *BW = calloc(nn, sizeof(double));
    double *Wp = calloc((size_t)nn * n_phases, sizeof(double));
    if (!W || !BW || !Wp) { free(W); free(BW); free(Wp); return -1; }
    for (k = 0; k < n; k++) {
        if (phase[k] == -1) continue;                                        /* :3319 */
        int ph = phase[k];
        int ip = clampi((int)ceil((x[k] - s.X[0]) / dx + 0.5) - 1, 0, s.nx - 1);   /* :3324-3329 */
        int jp = clampi((int)ceil((z[k] - s.Z[0]) / dz + 0.5) - 1, 0, s.nz - 1);   /* :3331-3335 */
        double val = 0.0;
        if (prop == 0) {                                                      /* :3340-3355 */
            val = flag == 0 ? mat_prop[ph] : mat_prop[k];
            if (avg == 1) val = 1.0 / val;
            if (avg == 2) val = log(val);
        }
        int h = itp_stencil == 9 ? 1 : 0;
        for (int dj = -h; dj <= h; dj++)
            for (int di = -h; di <= h; di++) {
                int ii = ip + di, jj = jp + dj;                               /* 9-cell neighbours :3364-3466 */
                if (ii < 0 || ii > s.nx - 1 || jj < 0 || jj > s.nz - 1) continue;
                double Xn = s.X[ip] + di * dx, Zn = s.Z[jp] + dj * dz;
                if (di == 0) Xn = s.X[ip];
                if (dj == 0) Zn = s.Z[jp];
                double w = (1.0 - fabs(Xn - x[k]) / hx) * (1.0 - fabs(Zn - z[k]) / hz);
                int c = ii + jj * s.nx;
                W[c] += w;
                BW[c] += val * w;
                Wp[(size_t)ph * nn + c] += w;
            }
    }
    for (i = 0; i < nn; i++) {                                                /* :3497-3521 */
        int skip = fabs(W[i]) < 1e-30 || (node_type && (node_type[i] == 30 || node_type[i] == 31));
        if (prop == 0) {
            if (skip) continue;
            double v = BW[i] / W[i];
            if (avg == 1) v = 1.0 / v;
            if (avg == 2) v = exp(v);
            node_field[i] = v;
        } else {
            for (p = 0; p < n_phases; p++)
                phase_perc[(size_t)p * nn + i] = skip ? Wp[(size_t)p * nn + i] : Wp[(size_t)p * nn + i] / W[i];
        }
    }
    free(W); free(BW); free(Wp);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Counting of CountPartCell_Old: vertices SOURCE/ParticleRoutines.c:4530-4560,
 * cells :4898-4925 (nearest node, phase >= 0 only).  The reference does not
 * clamp; a marker exactly on the west/south wall would index -1 there, so the
 * indices are clamped into the grid here (no effect for interior markers). */
int orc_count(const mdz_grid_desc *g, int n, const double *x, const double *z, const int *phase, int n_phases,
              int *nb_part_cell, int *nb_part_vert, int *phase_count_cell, int *phase_count_vert) {
    int ncx = g->Nx - 1, ncz = g->Nz - 1, Nx = g->Nx, Nz = g->Nz, k;
    if (nb_part_cell) memset(nb_part_cell, 0, sizeof(int) * ncx * ncz);
    if (nb_part_vert) memset(nb_part_vert, 0, sizeof(int) * Nx * Nz);
    if (phase_count_cell) memset(phase_count_cell, 0, sizeof(int) * ncx * ncz * n_phases);
    if (phase_count_vert) memset(phase_count_vert, 0, sizeof(int) * Nx * Nz * n_phases);
    for (k = 0; k < n; k++) {
        if (phase[k] < 0) continue;
        int ic = clampi((int)ceil((x[k] - g->xg[0]) / g->dx + 0.5) - 1, 0, Nx - 1);
        int jc = clampi((int)ceil((z[k] - g->zg[0]) / g->dz + 0.5) - 1, 0, Nz - 1);
        if (nb_part_vert) nb_part_vert[ic + jc * Nx]++;
        if (phase_count_vert) phase_count_vert[(size_t)phase[k] * Nx * Nz + ic + jc * Nx]++;
        ic = clampi((int)ceil((x[k] - g->xc[0]) / g->dx + 0.5) - 1, 0, ncx - 1);
        jc = clampi((int)ceil((z[k] - g->zc[0]) / g->dz + 0.5) - 1, 0, ncz - 1);
        if (nb_part_cell) nb_part_cell[ic + jc * ncx]++;
        if (phase_count_cell) phase_count_cell[(size_t)phase[k] * ncx * ncz + ic + jc * ncx]++;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
static int is_air(signed char t) { return t == 30 || t == 31; }

static const signed char *nodeset_tags(const mdz_grid_desc *g, int centroid) {
    if (centroid == 1) return g->BCp_type;
    if (centroid == 0) return g->BCg_type;
    if (centroid == -1) return g->BCu_type;
    return g->BCv_type;
}

int orc_g2p(const mdz_grid_desc *g, int n, const double *x, const double *z, const int *phase,
            const double *F, int node_set, double *out) {
    double dx = g->dx, dz = g->dz;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < n; k++) {
        out[k] = 0.0;
        if (phase[k] == -1) continue;
        int iSW, iSE, iNW, iNE;
        double dxm, dzm;
        const signed char *tag = nodeset_tags(g, node_set);
        if (node_set != 1) {
            /* Interp_Grid2P :2520-2560 */
            nodeset_t s = nodeset(g, node_set);
            int jp = clampi((int)ceil((x[k] - s.X[0]) / dx) - 1, 0, s.nx - 2);
            int ip = clampi((int)ceil((z[k] - s.Z[0]) / dz) - 1, 0, s.nz - 2);
            dxm = fabs(x[k] - s.X[jp]);
            dzm = fabs(z[k] - s.Z[ip]);
            iSW = jp + ip * s.nx; iSE = iSW + 1; iNW = jp + (ip + 1) * s.nx; iNE = iNW + 1;
        } else {
            /* Interp_Grid2P_centroids2 (non-periodic branches) :2640-2800 */
            int ncx = g->Nx - 1, ncz = g->Nz - 1;
            int jp = (int)ceil((x[k] - g->xvz[0]) / dx) - 1;
            int ip = (int)ceil((z[k] - g->zvx[0]) / dz) - 1;
            int jw = jp - 1, je = jp, is = ip - 1, in = ip;
            if (jp <= 0) { jw = 0; je = 0; }
            if (jp >= ncx) { jw = ncx - 1; je = ncx - 1; }
            if (ip <= 0) { is = 0; in = 0; }
            if (ip >= ncz) { is = ncz - 1; in = ncz - 1; }
            iSW = jw + is * ncx; iSE = je + is * ncx; iNW = jw + in * ncx; iNE = je + in * ncx;
            dxm = x[k] - g->xvz[clampi(jp, 0, ncx)];
            dzm = z[k] - g->zvx[clampi(ip, 0, ncz)];
        }
        double v = 0.0;
        v += (1.0 - dxm / dx) * (1.0 - dzm / dz) * (is_air(tag[iSW]) ? F[iNW] : F[iSW]);
        v += (dxm / dx) * (1.0 - dzm / dz) * (is_air(tag[iSE]) ? F[iNE] : F[iSE]);
        v += (1.0 - dxm / dx) * (dzm / dz) * (is_air(tag[iNW]) ? F[iSW] : F[iNW]);
        v += (dxm / dx) * (dzm / dz) * (is_air(tag[iNE]) ? F[iSE] : F[iNE]);
        out[k] = v;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* V2P without the conservative correction: SOURCE/ParticleRoutines.c:60-252. */
static void orc_v2p(const mdz_grid_desc *g, double xk, double zk, const double *u, const double *v, double *vxm,
                    double *vzm) {
    double dx = g->dx, dz = g->dz;
    int nx = g->Nx, nz = g->Nz + 1;
    int jp = clampi((int)ceil((xk - g->xg[0]) / dx) - 1, 0, nx - 2);
    int ip = clampi((int)ceil((zk - g->zvx[0]) / dz) - 1, 0, nz - 2);
    double dxm = fabs(xk - g->xg[jp]), dzm = fabs(zk - g->zvx[ip]);
    int iSW = jp + ip * nx, iSE = iSW + 1, iNW = jp + (ip + 1) * nx, iNE = iNW + 1;
    const signed char *t = g->BCu_type;
    double VNW = u[iNW], VNE = u[iNE], VSW = u[iSW], VSE = u[iSE];
    if (t[iSW] == 30) VSW = u[iNW];
    if (t[iSE] == 30) VSE = u[iNE];
    if (t[iNW] == 30) VNW = u[iSW];
    if (t[iNE] == 30) VNE = u[iSE];
    if (t[iNE] == 30 && t[iSE] == 30) { VNE = VSW; VSE = VSW; }
    if (t[iNW] == 30 && t[iSW] == 30) { VNW = VSE; VSW = VSE; }
    double a = VSW * (1.0 - dxm / dx) + VSE * dxm / dx;
    double b = VNW * (1.0 - dxm / dx) + VNE * dxm / dx;
    *vxm = (1.0 - dzm / dz) * a + (dzm / dz) * b;

    nx = g->Nx + 1; nz = g->Nz;
    jp = clampi((int)ceil((xk - g->xvz[0]) / dx) - 1, 0, nx - 2);
    ip = clampi((int)ceil((zk - g->zg[0]) / dz) - 1, 0, nz - 2);
    dxm = fabs(xk - g->xvz[jp]); dzm = fabs(zk - g->zg[ip]);
    iSW = jp + ip * nx; iSE = iSW + 1; iNW = jp + (ip + 1) * nx; iNE = iNW + 1;
    t = g->BCv_type;
    VSE = v[iSE]; VSW = v[iSW]; VNE = v[iNE]; VNW = v[iNW];
    if (t[iSW] == 30) VSW = v[iNE];
    if (t[iSE] == 30) VSE = v[iNE];
    if (t[iNW] == 30) VNW = v[iSW];
    if (t[iNE] == 30) VNE = v[iSE];
    if (t[iNE] == 30 && t[iSE] == 30) { VNE = VSW; VSE = VSW; }
    if (t[iNW] == 30 && t[iSW] == 30) { VNW = VSE; VSW = VSE; }
    a = VSW * (1.0 - dzm / dz) + VNW * dzm / dz;
    b = VSE * (1.0 - dzm / dz) + VNE * dzm / dz;
    *vzm = (1.0 - dxm / dx) * a + (dxm / dx) * b;
}

/* RogerGuntherII: SOURCE/AdvectionRoutines.c:569-628. */
int orc_rk4(const mdz_grid_desc *g, int n, double *x, double *z, int *phase, double *vx, double *vz,
            const double *u, const double *v, double dt) {
#pragma omp parallel for schedule(static)
    for (int k = 0; k < n; k++) {
        double xA = x[k], zA = z[k];
        double VA[2] = {0, 0}, VB[2] = {0, 0}, VC[2] = {0, 0}, VD[2] = {0, 0};
#define OUT() if (x[k] < g->xmin || x[k] > g->xmax || z[k] < g->zmin || z[k] > g->zmax) phase[k] = -1;
        if (phase[k] != -1) orc_v2p(g, x[k], z[k], u, v, &VA[0], &VA[1]);
        if (phase[k] != -1) { x[k] = xA + 0.5 * dt * VA[0]; z[k] = zA + 0.5 * dt * VA[1]; }
        OUT();
        if (phase[k] != -1) orc_v2p(g, x[k], z[k], u, v, &VB[0], &VB[1]);
        if (phase[k] != -1) { x[k] = xA + 0.5 * dt * VB[0]; z[k] = zA + 0.5 * dt * VB[1]; }
        OUT();
        if (phase[k] != -1) orc_v2p(g, x[k], z[k], u, v, &VC[0], &VC[1]);
        if (phase[k] != -1) { x[k] = xA + 1.0 * dt * VC[0]; z[k] = zA + 1.0 * dt * VC[1]; }
        OUT();
        if (phase[k] != -1) orc_v2p(g, x[k], z[k], u, v, &VD[0], &VD[1]);
        double ax = (1.0 / 6.0) * (VA[0] + 2.0 * VB[0] + 2.0 * VC[0] + VD[0]);
        double az = (1.0 / 6.0) * (VA[1] + 2.0 * VB[1] + 2.0 * VC[1] + VD[1]);
        if (phase[k] != -1) {
            x[k] = xA + dt * ax; z[k] = zA + dt * az;
            vx[k] = ax; vz[k] = az;
        }
        OUT();
#undef OUT
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Marker reseeding: CountPartCell with RESEED = 1 on one OpenMP thread
 * (SOURCE/ParticleRoutines.c:3543-4480).  Quarter-cell binning of the active
 * markers on the grid extended by one cell (:3905-3950); every quarter cell
 * of the inner region whose centroid is not air and that holds fewer than
 * (int)(ceil(min_part_cell) / 4) markers gets one marker at its centre
 * (AddPartCell2, :977-1030), which copies the nearest of the markers in the
 * 5x5 quarter cells around it (FindClosestPhase2, :841-890; candidates in the
 * reference's visiting order :4105-4283, a later one wins only when strictly
 * closer); new markers, numbered quarter-column by quarter-column, first fill
 * the slots of inactive markers in index order, then append (:4285-4330);
 * AssignMarkerProperties (:648-762) copies phase, velocity and strains, and
 * T and the stresses from the neighbour (direct = 1) or from the grid
 * (Centers2Particle :259-455, Vertices2Particle :461-520; direct = 0).  The
 * air test reads BCp (the reference reads BCt, whose air tag 30 sits on the
 * same cells).  attr: the MDZ_M_* marker attributes; the cohesion multiplier
 * is copied.  Returns the new marker count; -1 when a deficient quarter cell
 * has no marker within two quarter cells (the reference exits with 333), -2
 * when the new markers would not fit in cap. */
static double orc_c2p(const mdz_grid_desc *g, double x, double z, const double *F) {
    const int Nx = g->Nx - 1, Nz = g->Nz - 1;   /* centroid counts */
    const double *X = g->xvz, *Z = g->zvx, dx = g->dx, dz = g->dz;
    const int j = (int)(ceil((x - X[0]) / dx) - 1), i = (int)(ceil((z - Z[0]) / dz) - 1);
    int iSW, iSE, iNW, iNE, ic, jc;
    if (j > 0 && j < Nx && i > 0 && i < Nz) {
        ic = i - 1; jc = j - 1;
        iSW = jc + ic * Nx; iSE = iSW + 1; iNW = jc + (ic + 1) * Nx; iNE = iNW + 1;
    } else if (j == 0 && i > 0 && i < Nz) {
        ic = i - 1; iSW = iSE = ic * Nx; iNW = iNE = (ic + 1) * Nx;
    } else if (j == Nx && i > 0 && i < Nz) {
        ic = i - 1; jc = Nx - 1; iSW = iSE = jc + ic * Nx; iNW = iNE = jc + (ic + 1) * Nx;
    } else if (i == 0 && j > 0 && j < Nx) {
        jc = j - 1; iSW = iNW = jc; iSE = iNE = jc + 1;
    } else if (i == Nz && j > 0 && j < Nx) {
        ic = Nz - 1; jc = j - 1; iSW = iNW = jc + ic * Nx; iSE = iNE = jc + ic * Nx + 1;
    } else if (i == 0 && j == 0) {
        iSW = iSE = iNW = iNE = 0;
    } else if (i == 0 && j == Nx) {
        iSW = iSE = iNW = iNE = Nx - 1;
    } else if (i == Nz && j == 0) {
        iSW = iSE = iNW = iNE = (Nz - 1) * Nx;
    } else if (i == Nz && j == Nx) {
        iSW = iSE = iNW = iNE = (Nx - 1) + (Nz - 1) * Nx;
    } else {
        return 0.0;   /* outside the extended frame: not reached for markers inside the box */
    }
    const double dxm = x - X[j], dzm = z - Z[i];
    const signed char *t = g->BCp_type;
    double val = 0.0, sw = 0.0, w;
    if (t[iSW] != 30 && t[iSW] != 31) { w = (1.0 - dxm / dx) * (1.0 - dzm / dz); val += w * F[iSW]; sw += w; }
    if (t[iSE] != 30 && t[iSE] != 31) { w = (dxm / dx) * (1.0 - dzm / dz); val += w * F[iSE]; sw += w; }
    if (t[iNW] != 30 && t[iNW] != 31) { w = (1.0 - dxm / dx) * (dzm / dz); val += w * F[iNW]; sw += w; }
    if (t[iNE] != 30 && t[iNE] != 31) { w = (dxm / dx) * (dzm / dz); val += w * F[iNE]; sw += w; }
    if (sw > 1e-13) val /= sw;
    return val;
}

static double orc_v2p_vert(const mdz_grid_desc *g, double x, double z, const double *F) {
    const int Nx = g->Nx;
    const double dx = g->dx, dz = g->dz;
    const int j = (int)(ceil(fabs(x - g->xg[0]) / dx) - 1), i = (int)(ceil(fabs(z - g->zg[0]) / dz) - 1);
    const double dxm = x - g->xg[j], dzm = z - g->zg[i];
    const int iSW = j + i * Nx, iSE = iSW + 1, iNW = j + (i + 1) * Nx, iNE = iNW + 1;
    const signed char *t = g->BCg_type;
    double val = 0.0, sw = 0.0, w;
    if (t[iSW] != 30 && t[iSW] != 31) { w = (1.0 - dxm / dx) * (1.0 - dzm / dz); val += w * F[iSW]; sw += w; }
    if (t[iSE] != 30 && t[iSE] != 31) { w = (dxm / dx) * (1.0 - dzm / dz); val += w * F[iSE]; sw += w; }
    if (t[iNW] != 30 && t[iNW] != 31) { w = (1.0 - dxm / dx) * (dzm / dz); val += w * F[iNW]; sw += w; }
    if (t[iNE] != 30 && t[iNE] != 31) { w = (dxm / dx) * (dzm / dz); val += w * F[iNE]; sw += w; }
    if (sw > 1e-13) val /= sw;
    return val;
}

int orc_reseed(const mdz_grid_desc *g, int n, int cap, double *x, double *z, int *phase, double *vx, double *vz,
               double *const *attr, int min_part_cell, int direct, const double *T_n, const double *sxxd_n,
               const double *szzd_n, const double *sxz_s, const double *p_n, int *n_added) {
    const double dx = g->dx, dz = g->dz;
    const int Ncx = g->Nx - 1, Ncz = g->Nz - 1, nxl = 2 * (Ncx + 2), nzl = 2 * (Ncz + 2), nq = nxl * nzl;
    const double xge = g->xg[0] - dx, zge = g->zg[0] - dz;
    const double xce = 0.5 * (xge + (xge + dx)), zce = 0.5 * (zge + (zge + dz));
    int *cnt = calloc((size_t)nq, sizeof(int)), *start = calloc((size_t)nq + 1, sizeof(int));
    int *list = malloc(sizeof(int) * (size_t)(n > 0 ? n : 1)), *qk = malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    /* quarter-cell bins, marker indices ascending inside each */
    for (int k = 0; k < n; k++) {
        qk[k] = -1;
        if (phase[k] < 0) continue;
        int ic = (int)(ceil((x[k] - (xce - dx / 4.0)) / dx * 2.0 + 0.5) - 1);
        int jc = (int)(ceil((z[k] - (zce - dz / 4.0)) / dz * 2.0 + 0.5) - 1);
        ic = ic < 0 ? 0 : (ic > nxl - 1 ? nxl - 1 : ic);
        jc = jc < 0 ? 0 : (jc > nzl - 1 ? nzl - 1 : jc);
        qk[k] = ic + jc * nxl;
        cnt[qk[k]]++;
    }
    for (int q = 0; q < nq; q++) start[q + 1] = start[q] + cnt[q];
    {
        int *cur = calloc((size_t)nq, sizeof(int));
        for (int k = 0; k < n; k++)
            if (qk[k] >= 0) list[start[qk[k]] + cur[qk[k]]++] = k;
        free(cur);
    }
    const int thr = (int)(ceil((double)min_part_cell) / 4.0);
    /* window visiting order (dk, dl) */
    static const int W[25][2] = {{0, 0}, {-1, 0}, {1, 0}, {0, -1}, {0, 1}, {-1, -1}, {1, -1}, {-1, 1}, {1, 1},
                                 {-2, 0}, {2, 0}, {0, -2}, {0, 2}, {-2, -2}, {2, -2}, {-2, 2}, {2, 2},
                                 {-1, -2}, {1, -2}, {-1, 2}, {1, 2}, {-2, -1}, {-2, 1}, {2, -1}, {2, 1}};
    int nnew = 0, cap_new = 4 * Ncx * Ncz;
    double *nx_ = malloc(sizeof(double) * (size_t)cap_new), *nz_ = malloc(sizeof(double) * (size_t)cap_new);
    int *src = malloc(sizeof(int) * (size_t)cap_new), status = 0;
    for (int k = 2; k < nxl - 2 && !status; k++)
        for (int l = 2; l < nzl - 2; l++) {
            const int kd = k + l * nxl;
            int ic = (int)(ceil(((xge + dx / 4.0 + k * dx / 2.0) - g->xc[0]) / dx + 0.5) - 1);
            int jc = (int)(ceil(((zge + dz / 4.0 + l * dz / 2.0) - g->zc[0]) / dz + 0.5) - 1);
            ic = ic < 0 ? 0 : (ic > Ncx - 1 ? Ncx - 1 : ic);
            jc = jc < 0 ? 0 : (jc > Ncz - 1 ? Ncz - 1 : jc);
            if (g->BCp_type[ic + jc * Ncx] == 30) continue;
            if (!(cnt[kd] < thr)) continue;
            int neighs = 0;
            for (int w = 0; w < 25; w++) neighs += cnt[kd + W[w][0] + W[w][1] * nxl];
            if (neighs == 0) { status = -1; break; }
            const double xn = g->xg[0] + (k - 2) * dx / 2.0 + dx / 4.0, zn = g->zg[0] + (l - 2) * dz / 2.0 + dz / 4.0;
            if (!(xn > g->xmin && zn > g->zmin && zn < g->zmax)) continue;
            double best = g->xmax - g->xmin;
            int bi = -1;
            for (int w = 0; w < 25; w++) {
                const int q = kd + W[w][0] + W[w][1] * nxl;
                for (int s = start[q]; s < start[q + 1]; s++) {
                    const int m = list[s];
                    if (bi < 0) bi = m;   /* the reference's start: the first candidate */
                    /* squares by pow as the reference writes them (libm's pow(a, 2) and
                     * a * a can differ in the last bit) */
                    const double d = sqrt(pow(xn - x[m], 2.0) + pow(zn - z[m], 2.0));
                    if (d < best) { best = d; bi = m; }
                }
            }
            nx_[nnew] = xn; nz_[nnew] = zn; src[nnew] = bi; nnew++;
        }
    int out = status;
    if (!status) {
        int nreuse = 0;
        for (int k = 0; k < n; k++) nreuse += phase[k] == -1;
        const int n_final = n + (nnew > nreuse ? nnew - nreuse : 0);
        if (n_final > cap) out = -2;
        else {
            int *reuse = malloc(sizeof(int) * (size_t)(nreuse > 0 ? nreuse : 1)), r = 0;
            for (int k = 0; k < n; k++) if (phase[k] == -1) reuse[r++] = k;
            for (int q = 0; q < nnew; q++) {
                const int slot = q < nreuse ? reuse[q] : n + (q - nreuse), m = src[q];
                x[slot] = nx_[q]; z[slot] = nz_[q];
                phase[slot] = phase[m]; vx[slot] = vx[m]; vz[slot] = vz[m];
                attr[MDZ_M_STRAIN][slot] = attr[MDZ_M_STRAIN][m];
                attr[MDZ_M_STRAIN_PL][slot] = attr[MDZ_M_STRAIN_PL][m];
                attr[MDZ_M_CMUL][slot] = attr[MDZ_M_CMUL][m];
                if (direct) {
                    attr[MDZ_M_T][slot] = attr[MDZ_M_T][m];
                    attr[MDZ_M_P][slot] = attr[MDZ_M_P][m];
                    attr[MDZ_M_SXXD][slot] = attr[MDZ_M_SXXD][m];
                    attr[MDZ_M_SZZD][slot] = attr[MDZ_M_SZZD][m];
                    attr[MDZ_M_SXZ][slot] = attr[MDZ_M_SXZ][m];
                } else {
                    attr[MDZ_M_T][slot] = orc_c2p(g, x[slot], z[slot], T_n);
                    attr[MDZ_M_P][slot] = orc_c2p(g, x[slot], z[slot], p_n);   /* mesh->p_in :672 */
                    attr[MDZ_M_SXXD][slot] = orc_c2p(g, x[slot], z[slot], sxxd_n);
                    attr[MDZ_M_SZZD][slot] = orc_c2p(g, x[slot], z[slot], szzd_n);
                    attr[MDZ_M_SXZ][slot] = orc_v2p_vert(g, x[slot], z[slot], sxz_s);
                }
            }
            free(reuse);
            out = n_final;
            if (n_added) *n_added = nnew;
        }
    }
    free(cnt); free(start); free(list); free(qk); free(nx_); free(nz_); free(src);
    return out;
}
