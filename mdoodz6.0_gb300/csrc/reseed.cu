// Marker reseeding: the reseeding half of CountPartCell (RESEED = 1,
// SOURCE/ParticleRoutines.c:3543-4480) on the resident markers, with the
// result the reference gives on one OpenMP thread.
//
//   quarter cells  the grid extended by one cell on each side, split into
//                  (2 (Ncx + 2)) x (2 (Ncz + 2)) quarter cells; an active
//                  marker's quarter cell is ceil(((x - (xc_e0 - dx/4)) / dx) 2
//                  + 0.5) - 1, clamped (:3905-3921), counted and listed in
//                  ascending marker index (a stable counting sort: count,
//                  scan, scatter, per-bin index sort);
//   deficiency     each quarter cell of the inner region whose centroid is not
//                  air and that holds fewer than (int)(ceil(min_part_cell) / 4)
//                  markers gets one marker at its centre (AddPartCell2
//                  :977-1030); every such cell is independent of the others,
//                  one thread each;
//   neighbour      the new marker copies the nearest marker of the 5x5 quarter
//                  cells around it, visited in the reference's order
//                  (:4105-4283) and replaced only by a strictly closer one
//                  (FindClosestPhase2 :841-890);
//   slots          new markers are numbered quarter-column by quarter-column
//                  (the reference's k-outer, l-inner loop); the first ones
//                  take the slots of inactive markers in index order, the
//                  rest are appended (:4285-4330): two scans;
//   properties     phase, velocity and strains are copied, T, P and the stresses
//                  copied (DirectNeighbour = 1) or interpolated from the grid
//                  (Centers2Particle :259-455, Vertices2Particle :461-520)
//                  (AssignMarkerProperties :648-762).  The cohesion multiplier
//                  travels with the copied marker.
//
// Sources of a copy are active markers, destinations inactive slots or slots
// past the old count: no thread reads what another writes.  Index arithmetic
// rounds every product before its sum (__dmul_rn / __dadd_rn) so that no
// contraction moves a marker to another quarter cell.  Distances square with
// a * a where the reference calls pow(a, 2); the two can differ in the last
// bit, so a nearest-marker choice can differ only between two candidates whose
// distances agree to one unit in the last place.
#include <cmath>
#include "mdz_internal.cuh"

struct mdz_reseed_ws {
    long long cap = 0;
    int nq = 0, ni = 0;
    int *qcell = nullptr, *qsorted = nullptr;            // per marker
    int *qcount = nullptr, *qstart = nullptr, *qcursor = nullptr, *qpart = nullptr;   // per quarter cell
    int *flag = nullptr, *rank = nullptr, *src = nullptr, *ipart = nullptr;           // per inner quarter cell
    int *inact = nullptr, *islot = nullptr, *reuse = nullptr, *mpart = nullptr;       // per marker
    int *status = nullptr;                               // [0] no-neighbour flag
};

void mdz_reseed_free(mdz_ctx *ctx) {
    mdz_reseed_ws *W = ctx->reseed;
    if (!W) return;
    int *p[] = {W->qcell, W->qsorted, W->qcount, W->qstart, W->qcursor, W->qpart, W->flag, W->rank,
                W->src, W->ipart, W->inact, W->islot, W->reuse, W->mpart, W->status};
    for (int *q : p)
        if (q) cudaFree(q);
    delete W;
    ctx->reseed = nullptr;
}

// Quarter-grid geometry, every constant formed as the reference forms it.
struct quarter_geom {
    int nxl, nzl, Ncx, Ncz, Nx;
    double dx, dz, xge, zge, qx0, qz0;   // extended vertex origin; quarter-index origin xc_e0 - dx/4
    double xg0, zg0, xc0, zc0, xmin, xmax, zmin, zmax;
};

static quarter_geom make_quarter_geom(const mdz_ctx *ctx) {
    const mdz_grid_desc &d = ctx->host_desc;
    quarter_geom q;
    q.Ncx = d.Nx - 1; q.Ncz = d.Nz - 1; q.Nx = d.Nx;
    q.nxl = 2 * (q.Ncx + 2); q.nzl = 2 * (q.Ncz + 2);
    q.dx = d.dx; q.dz = d.dz;
    q.xg0 = d.xg[0]; q.zg0 = d.zg[0]; q.xc0 = d.xc[0]; q.zc0 = d.zc[0];
    q.xge = q.xg0 - q.dx;
    q.zge = q.zg0 - q.dz;
    const double xce = 0.5 * (q.xge + (q.xge + q.dx)), zce = 0.5 * (q.zge + (q.zge + q.dz));
    q.qx0 = xce - q.dx / 4.0;
    q.qz0 = zce - q.dz / 4.0;
    q.xmin = d.xmin; q.xmax = d.xmax; q.zmin = d.zmin; q.zmax = d.zmax;
    return q;
}

// ceil(v + 0.5) - 1 of the reference's nearest-node formula, as an int
__device__ __forceinline__ int nearest_of(double v) { return (int)(ceil(__dadd_rn(v, 0.5)) - 1.0); }

__global__ void k_quarter_count(int n, const double *__restrict__ x, const double *__restrict__ z,
                                const int *__restrict__ phase, quarter_geom q, int *__restrict__ qcell,
                                int *__restrict__ qcount) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    if (phase[k] < 0) { qcell[k] = -1; return; }
    int ic = nearest_of(__dmul_rn(__ddiv_rn(x[k] - q.qx0, q.dx), 2.0));
    int jc = nearest_of(__dmul_rn(__ddiv_rn(z[k] - q.qz0, q.dz), 2.0));
    ic = ic < 0 ? 0 : (ic > q.nxl - 1 ? q.nxl - 1 : ic);
    jc = jc < 0 ? 0 : (jc > q.nzl - 1 ? q.nzl - 1 : jc);
    const int c = ic + jc * q.nxl;
    qcell[k] = c;
    atomicAdd(&qcount[c], 1);
}

// Window of AddPartCell2's neighbour list, in the reference's visiting order.
__constant__ signed char c_window[25][2] = {
    {0, 0},   {-1, 0}, {1, 0},  {0, -1}, {0, 1},  {-1, -1}, {1, -1}, {-1, 1},  {1, 1},
    {-2, 0},  {2, 0},  {0, -2}, {0, 2},  {-2, -2}, {2, -2}, {-2, 2}, {2, 2},
    {-1, -2}, {1, -2}, {-1, 2}, {1, 2},  {-2, -1}, {-2, 1}, {2, -1}, {2, 1}};

// New-marker position of inner quarter cell (k, l): xg[0] + ic dx/2 + dx/4 with
// ic = k - 2 (halving and quartering are exact as products with 0.5, 0.25).
__device__ __forceinline__ double new_pos(double o, int i, double h) {
    return __dadd_rn(__dadd_rn(o, __dmul_rn(__dmul_rn((double)i, h), 0.5)), __dmul_rn(h, 0.25));
}

// One thread per inner quarter cell; t runs over (k, l) with k fastest, the
// flags are stored in the reference's creation order q = (k-2) (nzl-4) + (l-2).
// The count test comes first (integer), then the air test of the cell's
// centroid, the neighbour count and the box test of the new position.
__global__ void k_reseed_cells(quarter_geom q, const signed char *__restrict__ tagp, const int *__restrict__ qstart,
                               int thr, int *__restrict__ flag, int *__restrict__ status) {
    const int wi = q.nxl - 4, wj = q.nzl - 4;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= wi * wj) return;
    const int k = 2 + t % wi, l = 2 + t / wi, qo = (k - 2) * wj + (l - 2), kd = k + l * q.nxl;
    int f = 0;
    if (qstart[kd + 1] - qstart[kd] < thr) {
        // centroid of the quarter cell's coarse cell, for the air test
        const double cx = __dadd_rn(__dadd_rn(q.xge, __dmul_rn(q.dx, 0.25)), __dmul_rn(__dmul_rn((double)k, q.dx), 0.5));
        const double cz = __dadd_rn(__dadd_rn(q.zge, __dmul_rn(q.dz, 0.25)), __dmul_rn(__dmul_rn((double)l, q.dz), 0.5));
        int ic = nearest_of(__ddiv_rn(cx - q.xc0, q.dx)), jc = nearest_of(__ddiv_rn(cz - q.zc0, q.dz));
        ic = ic < 0 ? 0 : (ic > q.Ncx - 1 ? q.Ncx - 1 : ic);
        jc = jc < 0 ? 0 : (jc > q.Ncz - 1 ? q.Ncz - 1 : jc);
        if (tagp[ic + jc * q.Ncx] != 30) {
            int neighs = 0;
            for (int w = 0; w < 25; w++) {
                const int c = kd + c_window[w][0] + c_window[w][1] * q.nxl;
                neighs += qstart[c + 1] - qstart[c];
            }
            if (neighs == 0) {
                atomicOr(status, 1);
            } else {
                const double xn = new_pos(q.xg0, k - 2, q.dx), zn = new_pos(q.zg0, l - 2, q.dz);
                f = xn > q.xmin && zn > q.zmin && zn < q.zmax;
            }
        }
    }
    flag[qo] = f;
}

// Inverse of the ranks: list[rank] = quarter cell, so that the search below
// runs one thread per new marker.
__global__ void k_reseed_list(int ni, const int *__restrict__ flag, const int *__restrict__ rank,
                              int *__restrict__ list) {
    const int qo = blockIdx.x * blockDim.x + threadIdx.x;
    if (qo < ni && flag[qo]) list[rank[qo]] = qo;
}

__global__ void k_inactive_flags(int n, const int *__restrict__ phase, int *__restrict__ inact) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) inact[k] = phase[k] == -1 ? 1 : 0;
}

__global__ void k_inactive_list(int n, const int *__restrict__ inact, const int *__restrict__ islot,
                                int *__restrict__ reuse) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n && inact[k]) reuse[islot[k]] = k;
}

// Centers2Particle, non-periodic (SOURCE/ParticleRoutines.c:259-455): bilinear
// on the ghosted centroid lines with the reference's edge and corner folds.
__device__ double c2p(const mdz_dgrid &g, double x, double z, const double *__restrict__ F) {
    const int Nx = g.ncx, Nz = g.ncz;
    const double dx = g.dx, dz = g.dz;
    const int j = (int)(ceil((x - g.xvz[0]) / dx) - 1.0), i = (int)(ceil((z - g.zvx[0]) / dz) - 1.0);
    int iSW, iSE, iNW, iNE;
    if (j > 0 && j < Nx && i > 0 && i < Nz) {
        iSW = (j - 1) + (i - 1) * Nx; iSE = iSW + 1; iNW = (j - 1) + i * Nx; iNE = iNW + 1;
    } else if (j == 0 && i > 0 && i < Nz) {
        iSW = iSE = (i - 1) * Nx; iNW = iNE = i * Nx;
    } else if (j == Nx && i > 0 && i < Nz) {
        iSW = iSE = (Nx - 1) + (i - 1) * Nx; iNW = iNE = (Nx - 1) + i * Nx;
    } else if (i == 0 && j > 0 && j < Nx) {
        iSW = iNW = j - 1; iSE = iNE = j;
    } else if (i == Nz && j > 0 && j < Nx) {
        iSW = iNW = (j - 1) + (Nz - 1) * Nx; iSE = iNE = j + (Nz - 1) * Nx;
    } else if (i == 0 && j == 0) {
        iSW = iSE = iNW = iNE = 0;
    } else if (i == 0 && j == Nx) {
        iSW = iSE = iNW = iNE = Nx - 1;
    } else if (i == Nz && j == 0) {
        iSW = iSE = iNW = iNE = (Nz - 1) * Nx;
    } else if (i == Nz && j == Nx) {
        iSW = iSE = iNW = iNE = (Nx - 1) + (Nz - 1) * Nx;
    } else {
        return 0.0;   // outside the ghosted frame: new markers lie inside the box
    }
    const double ax = (x - g.xvz[j]) / dx, az = (z - g.zvx[i]) / dz;
    const signed char *t = g.BCp;
    double val = 0.0, sw = 0.0, w;
    if (t[iSW] != 30 && t[iSW] != 31) { w = (1.0 - ax) * (1.0 - az); val += w * F[iSW]; sw += w; }
    if (t[iSE] != 30 && t[iSE] != 31) { w = ax * (1.0 - az); val += w * F[iSE]; sw += w; }
    if (t[iNW] != 30 && t[iNW] != 31) { w = (1.0 - ax) * az; val += w * F[iNW]; sw += w; }
    if (t[iNE] != 30 && t[iNE] != 31) { w = ax * az; val += w * F[iNE]; sw += w; }
    return sw > 1e-13 ? val / sw : val;
}

// Vertices2Particle (SOURCE/ParticleRoutines.c:461-520): bilinear on the vertices.
__device__ double v2p_vertices(const mdz_dgrid &g, double x, double z, const double *__restrict__ F) {
    const int Nx = g.Nx;
    const double dx = g.dx, dz = g.dz;
    const int j = (int)(ceil(fabs(x - g.xg[0]) / dx) - 1.0), i = (int)(ceil(fabs(z - g.zg[0]) / dz) - 1.0);
    const double ax = (x - g.xg[j]) / dx, az = (z - g.zg[i]) / dz;
    const int iSW = j + i * Nx, iSE = iSW + 1, iNW = j + (i + 1) * Nx, iNE = iNW + 1;
    const signed char *t = g.BCg;
    double val = 0.0, sw = 0.0, w;
    if (t[iSW] != 30 && t[iSW] != 31) { w = (1.0 - ax) * (1.0 - az); val += w * F[iSW]; sw += w; }
    if (t[iSE] != 30 && t[iSE] != 31) { w = ax * (1.0 - az); val += w * F[iSE]; sw += w; }
    if (t[iNW] != 30 && t[iNW] != 31) { w = (1.0 - ax) * az; val += w * F[iNW]; sw += w; }
    if (t[iNE] != 30 && t[iNE] != 31) { w = ax * az; val += w * F[iNE]; sw += w; }
    return sw > 1e-13 ? val / sw : val;
}

struct reseed_fields {
    const double *T_n, *sxxd_n, *szzd_n, *sxz_s, *p_n;
};

// One thread per new marker r: its quarter cell, the nearest of the markers
// in the 5x5 quarter cells around it (the reference's visiting order; a
// candidate replaces the best only when strictly closer: the square test
// skips the square root of every candidate that cannot be), and the copy.
__global__ void k_reseed_write(quarter_geom q, mdz_dgrid g, int n, int nnew, int nreuse, const int *__restrict__ list,
                               const int *__restrict__ qstart, const int *__restrict__ qsorted,
                               const int *__restrict__ reuse, double *x, double *z, int *phase, double *vx,
                               double *vz, mdz_attr_ptrs A, int direct, reseed_fields F) {
    const int wj = q.nzl - 4;
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nnew) return;
    const int qo = list[r];
    const int k = 2 + qo / wj, l = 2 + qo % wj, kd = k + l * q.nxl;
    const double xn = new_pos(q.xg0, k - 2, q.dx), zn = new_pos(q.zg0, l - 2, q.dz);
    double best = q.xmax - q.xmin, best2 = INFINITY;
    int m = -1;
    for (int w = 0; w < 25; w++) {
        const int c = kd + c_window[w][0] + c_window[w][1] * q.nxl;
        for (int s = qstart[c], e = qstart[c + 1]; s < e; s++) {
            const int j = qsorted[s];
            if (m < 0) m = j;
            const double ax = xn - x[j], az = zn - z[j];
            const double d2 = __dadd_rn(__dmul_rn(ax, ax), __dmul_rn(az, az));
            if (d2 < best2) {   // sqrt is monotone: d2 >= best2 cannot give d < best
                const double d = sqrt(d2);
                if (d < best) { best = d; best2 = d2; m = j; }
            }
        }
    }
    const int slot = r < nreuse ? reuse[r] : n + (r - nreuse);
    x[slot] = xn;
    z[slot] = zn;
    phase[slot] = phase[m];
    vx[slot] = vx[m];
    vz[slot] = vz[m];
    A.a[MDZ_M_STRAIN][slot] = A.a[MDZ_M_STRAIN][m];
    A.a[MDZ_M_STRAIN_PL][slot] = A.a[MDZ_M_STRAIN_PL][m];
    A.a[MDZ_M_CMUL][slot] = A.a[MDZ_M_CMUL][m];
    if (direct) {
        A.a[MDZ_M_T][slot] = A.a[MDZ_M_T][m];
        A.a[MDZ_M_P][slot] = A.a[MDZ_M_P][m];
        A.a[MDZ_M_SXXD][slot] = A.a[MDZ_M_SXXD][m];
        A.a[MDZ_M_SZZD][slot] = A.a[MDZ_M_SZZD][m];
        A.a[MDZ_M_SXZ][slot] = A.a[MDZ_M_SXZ][m];
    } else {
        A.a[MDZ_M_T][slot] = c2p(g, xn, zn, F.T_n);
        A.a[MDZ_M_P][slot] = c2p(g, xn, zn, F.p_n);
        A.a[MDZ_M_SXXD][slot] = c2p(g, xn, zn, F.sxxd_n);
        A.a[MDZ_M_SZZD][slot] = c2p(g, xn, zn, F.szzd_n);
        A.a[MDZ_M_SXZ][slot] = v2p_vertices(g, xn, zn, F.sxz_s);
    }
}

// exclusive scan of in[0..n) into out[0..n] (out[n] = total), partial: scratch
static mdz_status scan_ints(mdz_ctx *ctx, int n, const int *in, int *out, int *partial, cudaStream_t st) {
    const int nb = (n + 1023) / 1024;
    k_scan_blocks<<<nb, 1024, 0, st>>>(n, in, out, partial);
    MDZ_LAUNCHED(ctx);
    k_scan_partials<<<1, 1024, 0, st>>>(nb, partial);
    MDZ_LAUNCHED(ctx);
    k_scan_add<<<nb, 1024, 0, st>>>(n, out, partial);
    MDZ_LAUNCHED(ctx);
    return MDZ_OK;
}

static mdz_status reseed_ws(mdz_ctx *ctx, const quarter_geom &q, mdz_reseed_ws *&W) {
    if (!ctx->reseed) ctx->reseed = new mdz_reseed_ws();
    W = ctx->reseed;
    const int nq = q.nxl * q.nzl, ni = (q.nxl - 4) * (q.nzl - 4);
    const long long cap = ctx->m.cap > 0 ? ctx->m.cap : 1;
    if (W->cap == cap && W->nq == nq) return MDZ_OK;
    mdz_reseed_free(ctx);
    ctx->reseed = W = new mdz_reseed_ws();
    auto A = [&](int *&p, long long cnt) { return cudaMalloc((void **)&p, sizeof(int) * (size_t)(cnt > 0 ? cnt : 1)); };
    MDZ_CUDA(ctx, A(W->qcell, cap));
    MDZ_CUDA(ctx, A(W->qsorted, cap));
    MDZ_CUDA(ctx, A(W->qcount, nq + 1));
    MDZ_CUDA(ctx, A(W->qstart, nq + 1));
    MDZ_CUDA(ctx, A(W->qcursor, nq + 1));
    MDZ_CUDA(ctx, A(W->qpart, (nq + 1023) / 1024 + 1));
    MDZ_CUDA(ctx, A(W->flag, ni));
    MDZ_CUDA(ctx, A(W->rank, ni + 1));
    MDZ_CUDA(ctx, A(W->src, ni));   // list: quarter cell of each new marker
    MDZ_CUDA(ctx, A(W->ipart, (ni + 1023) / 1024 + 1));
    MDZ_CUDA(ctx, A(W->inact, cap));
    MDZ_CUDA(ctx, A(W->islot, cap + 1));
    MDZ_CUDA(ctx, A(W->reuse, cap));
    MDZ_CUDA(ctx, A(W->mpart, (cap + 1023) / 1024 + 1));
    MDZ_CUDA(ctx, A(W->status, 4));
    W->cap = cap;
    W->nq = nq;
    W->ni = ni;
    return MDZ_OK;
}

mdz_status mdz_dev_reseed(mdz_ctx *ctx, int min_part_cell, int direct, const double *T_n, const double *sxxd_n,
                          const double *szzd_n, const double *sxz_s, const double *p_n, cudaStream_t st,
                          int *n_added) {
    if (n_added) *n_added = 0;
    if (min_part_cell < 0) return mdz_fail(ctx, MDZ_ERR_ARG, "CountPartCell: min_part_cell < 0");
    if (!direct && (!T_n || !sxxd_n || !szzd_n || !sxz_s || !p_n))
        return mdz_fail(ctx, MDZ_ERR_ARG, "CountPartCell: DirectNeighbour = 0 needs T, sxxd, szzd, sxz and p");
    const quarter_geom q = make_quarter_geom(ctx);
    // quarter-cell indices are 32-bit: (2 Ncx + 4)(2 Ncz + 4) must stay below 2^31
    if ((long long)q.nxl * q.nzl > 2147483000LL)
        return mdz_fail(ctx, MDZ_ERR_UNSUPPORTED, "CountPartCell: %d x %d quarter cells exceed 2^31", q.nxl, q.nzl);
    mdz_reseed_ws *W = nullptr;
    mdz_status s = reseed_ws(ctx, q, W);
    if (s != MDZ_OK) return s;
    const int n = ctx->m.n, nq = W->nq, ni = W->ni;
    // quarter-cell bins, ascending marker index inside each
    MDZ_CUDA(ctx, cudaMemsetAsync(W->qcount, 0, sizeof(int) * (nq + 1), st));
    MDZ_CUDA(ctx, cudaMemsetAsync(W->qcursor, 0, sizeof(int) * (nq + 1), st));
    MDZ_CUDA(ctx, cudaMemsetAsync(W->status, 0, sizeof(int) * 4, st));
    if (n > 0) {
        k_quarter_count<<<mdz_blocks(n), MDZ_THREADS, 0, st>>>(n, ctx->m.x, ctx->m.z, ctx->m.phase, q, W->qcell,
                                                               W->qcount);
        MDZ_LAUNCHED(ctx);
    }
    if ((s = scan_ints(ctx, nq, W->qcount, W->qstart, W->qpart, st)) != MDZ_OK) return s;
    if (n > 0) {
        k_bin_scatter<<<mdz_blocks(n), MDZ_THREADS, 0, st>>>(n, W->qcell, W->qstart, W->qcursor, W->qsorted);
        MDZ_LAUNCHED(ctx);
    }
    k_bin_sort_segments<<<mdz_blocks(nq), MDZ_THREADS, 0, st>>>(nq, W->qstart, W->qsorted);
    MDZ_LAUNCHED(ctx);
    // deficient quarter cells and their nearest markers, then the ranks
    const int thr = (int)(std::ceil((double)min_part_cell) / 4.0);
    k_reseed_cells<<<mdz_blocks(ni), MDZ_THREADS, 0, st>>>(q, ctx->g.BCp, W->qstart, thr, W->flag, W->status);
    MDZ_LAUNCHED(ctx);
    if ((s = scan_ints(ctx, ni, W->flag, W->rank, W->ipart, st)) != MDZ_OK) return s;
    k_reseed_list<<<mdz_blocks(ni), MDZ_THREADS, 0, st>>>(ni, W->flag, W->rank, W->src);
    MDZ_LAUNCHED(ctx);
    // inactive slots in index order
    int nreuse = 0;
    if (n > 0) {
        k_inactive_flags<<<mdz_blocks(n), MDZ_THREADS, 0, st>>>(n, ctx->m.phase, W->inact);
        MDZ_LAUNCHED(ctx);
        if ((s = scan_ints(ctx, n, W->inact, W->islot, W->mpart, st)) != MDZ_OK) return s;
        k_inactive_list<<<mdz_blocks(n), MDZ_THREADS, 0, st>>>(n, W->inact, W->islot, W->reuse);
        MDZ_LAUNCHED(ctx);
    }
    int h[3] = {0, 0, 0};
    MDZ_CUDA(ctx, cudaMemcpyAsync(&h[0], W->rank + ni, sizeof(int), cudaMemcpyDeviceToHost, st));
    if (n > 0) MDZ_CUDA(ctx, cudaMemcpyAsync(&h[1], W->islot + n, sizeof(int), cudaMemcpyDeviceToHost, st));
    MDZ_CUDA(ctx, cudaMemcpyAsync(&h[2], W->status, sizeof(int), cudaMemcpyDeviceToHost, st));
    MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    const int nnew = h[0];
    nreuse = h[1];
    if (h[2]) return mdz_fail(ctx, MDZ_ERR_STATE, "CountPartCell: a quarter cell lacking markers has no marker within two quarter cells");
    const long long n_final = (long long)n + (nnew > nreuse ? nnew - nreuse : 0);
    if (n_final > ctx->m.cap)
        return mdz_fail(ctx, MDZ_ERR_CAPACITY, "CountPartCell: %lld markers after reseeding > capacity %lld", n_final,
                        ctx->m.cap);
    if (nnew > 0) {
        mdz_attr_ptrs A;
        for (int a = 0; a < MDZ_M_NATTR; a++) A.a[a] = ctx->m.attr[a];
        k_reseed_write<<<mdz_blocks(nnew), MDZ_THREADS, 0, st>>>(q, ctx->g, n, nnew, nreuse, W->src, W->qstart,
                                                                 W->qsorted, W->reuse, ctx->m.x, ctx->m.z,
                                                                 ctx->m.phase, ctx->m.vx, ctx->m.vz, A, direct,
                                                                 reseed_fields{T_n, sxxd_n, szzd_n, sxz_s, p_n});
        MDZ_LAUNCHED(ctx);
    }
    ctx->m.n = (int)n_final;
    ctx->bins.valid = false;
    if (n_added) *n_added = nnew;
    return MDZ_OK;
}

extern "C" mdz_status mdz_CountPartCell(mdz_ctx *ctx, int reseed, int min_part_cell, int direct_neighbour,
                                        const double *T_n, const double *sxxd_n, const double *szzd_n,
                                        const double *sxz_s, const double *p_n, int *n_added) {
    if (!ctx) return MDZ_ERR_ARG;
    if (n_added) *n_added = 0;
    if (!reseed) return MDZ_OK;
    cudaStream_t st = ctx->stream;
    const mdz_dgrid &g = ctx->g;
    const size_t nc = (size_t)g.ncx * g.ncz, nv = (size_t)g.Nx * g.Nz;
    const double *d[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    if (!direct_neighbour) {
        if (!T_n || !sxxd_n || !szzd_n || !sxz_s || !p_n)
            return mdz_fail(ctx, MDZ_ERR_ARG, "CountPartCell: DirectNeighbour = 0 needs T, sxxd, szzd, sxz and p");
        const double *hsrc[5] = {T_n, sxxd_n, szzd_n, sxz_s, p_n};
        static const int slot[5] = {0, 1, 2, 3, 6};   // staging slots (5 holds the time step's workspace)
        for (int i = 0; i < 5; i++) {
            const size_t cnt = i == 3 ? nv : nc;
            double *p = (double *)mdz_stage(ctx, slot[i], sizeof(double) * cnt);
            if (!p) return mdz_fail(ctx, MDZ_ERR_CUDA, "CountPartCell: staging allocation failed");
            MDZ_CUDA(ctx, cudaMemcpyAsync(p, hsrc[i], sizeof(double) * cnt, cudaMemcpyHostToDevice, st));
            d[i] = p;
        }
    }
    int added = 0;
    mdz_status s = mdz_dev_reseed(ctx, min_part_cell, direct_neighbour, d[0], d[1], d[2], d[3], d[4], st, &added);
    if (s != MDZ_OK) return s;
    MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    if (n_added) *n_added = added;
    return MDZ_OK;
}
