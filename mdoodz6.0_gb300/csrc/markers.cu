// Marker-side kernels: cell binning (stable counting sort), batched
// marker->grid projection as a deterministic per-node gather, marker counts,
// grid->marker interpolation and RK4 advection.
//
// Reference behaviour followed (paths inside the MDOODZ 6.0 repository):
//   P2Mastah                  SOURCE/ParticleRoutines.c:3226-3537
//   CountPartCell_Old counts  SOURCE/ParticleRoutines.c:4485-4980
//   Interp_Grid2P             SOURCE/ParticleRoutines.c:2439-2608
//   Interp_Grid2P_centroids2  SOURCE/ParticleRoutines.c:2612-2862
//   V2P (TarasCorr = 0)       SOURCE/ParticleRoutines.c:60-252
//   RogerGuntherII / isoutPart SOURCE/AdvectionRoutines.c:569-628, 314-335
#include <cmath>
#include "mdz_internal.cuh"

// Nearest-node index along one line of a node set, as the reference computes
// it: ceil(d/h + 0.5) - 1 with d measured from the first line, clamped.
__device__ __forceinline__ int nearest_line(double x, double X0, double h, double ih, int n) {
    int i = (int)ceil_quot(x - X0, h, ih, 0.5) - 1;
    i = i < 0 ? 0 : i;
    return i > n - 1 ? n - 1 : i;
}

// Lower-left cell index along one line (V2P / Interp_Grid2P): ceil(d/h) - 1.
__device__ __forceinline__ int lower_line(double x, double X0, double h, double ih) {
    return (int)ceil_quot(x - X0, h, ih, 0.0) - 1;
}

// ---------------------------------------------------------------------------
// Binning: cell of each active marker = nearest centroid (the same formula and
// clamps as P2Mastah on centroids), per-cell counts.
__global__ void k_bin_count(int n, const double *__restrict__ x, const double *__restrict__ z,
                            const int *__restrict__ phase, const double *__restrict__ xc,
                            const double *__restrict__ zc, double dx, double dz, double idx, double idz, int ncx,
                            int ncz, int *__restrict__ cell, int *__restrict__ count) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    if (phase[k] == -1) { cell[k] = -1; return; }
    int ic = nearest_line(x[k], xc[0], dx, idx, ncx);
    int jc = nearest_line(z[k], zc[0], dz, idz, ncz);
    int c = ic + jc * ncx;
    cell[k] = c;
    atomicAdd(&count[c], 1);
}

// Block-wise inclusive scan (1024 elements per block) of int counts; writes
// exclusive results to out[i+1] and block totals to partial[].
__global__ void k_scan_blocks(int n, const int *__restrict__ in, int *__restrict__ out, int *__restrict__ partial) {
    __shared__ int warp_sums[32];
    int i = blockIdx.x * 1024 + threadIdx.x;
    int v = i < n ? in[i] : 0;
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int s = v;
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, s, o);
        if (lane >= o) s += t;
    }
    if (lane == 31) warp_sums[wid] = s;
    __syncthreads();
    if (wid == 0) {
        int w = warp_sums[lane];
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        warp_sums[lane] = w;
    }
    __syncthreads();
    if (wid > 0) s += warp_sums[wid - 1];
    if (i < n) out[i + 1] = s;
    if (threadIdx.x == 1023) partial[blockIdx.x] = s;
}

// Serial-over-blocks scan of the block totals (one CTA; blocks <= a few thousand).
__global__ void k_scan_partials(int nb, int *partial) {
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nb; base += 1024) {
        int i = base + threadIdx.x;
        int v = i < nb ? partial[i] : 0;
        // inclusive scan across the CTA, simple two-level
        __shared__ int buf[1024];
        buf[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {
            int t = threadIdx.x >= o ? buf[threadIdx.x - o] : 0;
            __syncthreads();
            buf[threadIdx.x] += t;
            __syncthreads();
        }
        int excl = buf[threadIdx.x] - v + carry;
        __syncthreads();
        if (i < nb) partial[i] = excl;
        if (threadIdx.x == 1023) carry += buf[1023];
        __syncthreads();
    }
}

__global__ void k_scan_add(int n, int *__restrict__ out, const int *__restrict__ partial) {
    int i = blockIdx.x * 1024 + threadIdx.x;
    if (i == 0) out[0] = 0;
    if (i < n) out[i + 1] += partial[blockIdx.x];
}

__global__ void k_bin_scatter(int n, const int *__restrict__ cell, const int *__restrict__ start,
                              int *__restrict__ cursor, int *__restrict__ sorted) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int c = cell[k];
    if (c < 0) return;
    int pos = start[c] + atomicAdd(&cursor[c], 1);
    sorted[pos] = k;
}

// Make the order inside each cell ascending in marker index, so that every
// projection sums in a fixed order (bit-reproducible run to run).
__global__ void k_bin_sort_segments(int ncells, const int *__restrict__ start, int *__restrict__ sorted) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    int b = start[c], e = start[c + 1];
    for (int i = b + 1; i < e; i++) {
        int v = sorted[i], j = i - 1;
        while (j >= b && sorted[j] > v) { sorted[j + 1] = sorted[j]; j--; }
        sorted[j + 1] = v;
    }
}

// Nearest vertex of the marker at each sorted position (the projection onto
// vertices tests every marker of its four candidate cells against the node:
// with the index stored once per binning the three markers in four that
// belong to another vertex cost an integer compare instead of two FP64 index
// computations, FP64 being a small fraction of the FP32 rate on this part).
// Same formula, lines and clamps as the projection's own nearest_line.
__global__ void k_bin_vertices(int n, const int *__restrict__ nbinned, const int *__restrict__ sorted,
                               const double *__restrict__ x, const double *__restrict__ z,
                               const double *__restrict__ xg, const double *__restrict__ zg, double dx, double dz,
                               double idx, double idz, int Nx, int Nz, int *__restrict__ qvert) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n || q >= *nbinned) return;
    const int k = sorted[q];
    const int ip = nearest_line(x[k], xg[0], dx, idx, Nx), jp = nearest_line(z[k], zg[0], dz, idz, Nz);
    qvert[q] = ip | (jp << 16);
}

mdz_status mdz_ensure_bins(mdz_ctx *ctx, cudaStream_t st) {
    mdz_bins &B = ctx->bins;
    if (B.valid) return MDZ_OK;
    const mdz_dgrid &g = ctx->g;
    int n = ctx->m.n, nc = B.ncells;
    MDZ_CUDA(ctx, cudaMemsetAsync(B.count, 0, sizeof(int) * (nc + 1), st));
    MDZ_CUDA(ctx, cudaMemsetAsync(B.cursor, 0, sizeof(int) * (nc + 1), st));
    if (n > 0) {
        k_bin_count<<<mdz_blocks(n), MDZ_THREADS, 0, st>>>(n, ctx->m.x, ctx->m.z, ctx->m.phase, g.xc, g.zc, g.dx, g.dz,
                                                           g.idx, g.idz, g.ncx, g.ncz, B.cell, B.count);
        MDZ_LAUNCHED(ctx);
    }
    int nb = (nc + 1023) / 1024;
    k_scan_blocks<<<nb, 1024, 0, st>>>(nc, B.count, B.start, B.scan_partials);
    MDZ_LAUNCHED(ctx);
    k_scan_partials<<<1, 1024, 0, st>>>(nb, B.scan_partials);
    MDZ_LAUNCHED(ctx);
    k_scan_add<<<nb, 1024, 0, st>>>(nc, B.start, B.scan_partials);
    MDZ_LAUNCHED(ctx);
    if (n > 0) {
        k_bin_scatter<<<mdz_blocks(n), MDZ_THREADS, 0, st>>>(n, B.cell, B.start, B.cursor, B.sorted);
        MDZ_LAUNCHED(ctx);
    }
    k_bin_sort_segments<<<mdz_blocks(nc), MDZ_THREADS, 0, st>>>(nc, B.start, B.sorted);
    MDZ_LAUNCHED(ctx);
    if (n > 0) {
        k_bin_vertices<<<mdz_blocks(n), MDZ_THREADS, 0, st>>>(n, B.start + nc, B.sorted, ctx->m.x, ctx->m.z, g.xg,
                                                              g.zg, g.dx, g.dz, g.idx, g.idz, g.Nx, g.Nz, B.qvert);
        MDZ_LAUNCHED(ctx);
    }
    B.valid = true;
    return MDZ_OK;
}

// ---------------------------------------------------------------------------
// Batched projection.  One thread per node gathers, from the markers of the
// cells that can hold its contributors, exactly the tent weights P2Mastah
// scatters: each marker finds its nearest node (ip, jp) with the reference's
// formula and clamps, then contributes to (ip, jp) and, for the 9-cell
// stencil, to the 8 neighbours, with distances measured from X[ip] +/- dx.
struct p2g_fields {
    const double *val[MDZ_P2G_MAX_FIELDS];   // per-marker values, or per-phase table
    int per_phase[MDZ_P2G_MAX_FIELDS];       // 1: val is indexed by phase (flag 0)
    int avg[MDZ_P2G_MAX_FIELDS];
    double *out[MDZ_P2G_MAX_FIELDS];
    int *empty;   // when set, counts active nodes that received no marker weight (phase fractions only)
};

// Candidate cell range along one direction for node i of a node set whose
// lines are of kind `kind` (0: centroid lines, 1: vertex lines, 2: ghosted lines).
__device__ __forceinline__ void cell_range(int i, int h, int kind, int n_nodes, int n_cells, int &lo, int &hi) {
    lo = i - h - kind;
    hi = i + h;
    if (i - h <= 0) lo = 0;
    if (i + h >= n_nodes - 1) hi = n_cells - 1;
    lo = lo < 0 ? 0 : lo;
    hi = hi > n_cells - 1 ? n_cells - 1 : hi;
}

template <int NF, int NPH>
__global__ void __launch_bounds__(128) k_p2g_gather(
    int nnx, int nnz, const double *__restrict__ X, const double *__restrict__ Z, const signed char *__restrict__ tag,
    int kindx, int kindz, int h, double dx, double dz, double idx, double idz, double idxi, double idzi, int ncx,
    int ncz, const int *__restrict__ start, const int *__restrict__ sorted, const int *__restrict__ qvert,
    const double *__restrict__ mx, const double *__restrict__ mz, const int *__restrict__ mphase, p2g_fields F,
    int nph_rt, double *__restrict__ phase_perc) {
    int node = blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= nnx * nnz) return;
    int i = node % nnx, j = node / nnx;
    int clo, chi, rlo, rhi;
    cell_range(i, h, kindx, nnx, ncx, clo, chi);
    cell_range(j, h, kindz, nnz, ncz, rlo, rhi);
    double Wm = 0.0, BmWm[NF > 0 ? NF : 1], Wph[NPH > 0 ? NPH : 1];
#pragma unroll
    for (int f = 0; f < NF; f++) BmWm[f] = 0.0;
#pragma unroll
    for (int p = 0; p < NPH; p++) Wph[p] = 0.0;
    const double X0 = X[0], Z0 = Z[0];
    // (1/dx, 1/dz and the reciprocal interpolation widths come from the host:
    // an FP64 division per thread is a long instruction sequence on this part)
    // contribution of marker k, whose nearest node (ip, jp) is within h of this one
    auto add = [&](int k, int ip, int jp, int di, int dj) {
        const double xk = mx[k], zk = mz[k];
        double Xn = X[ip], Zn = Z[jp];
        if (di > 0) Xn = X[ip] + dx;
        if (di < 0) Xn = X[ip] - dx;
        if (dj > 0) Zn = Z[jp] + dz;
        if (dj < 0) Zn = Z[jp] - dz;
        double dxm = fabs(Xn - xk), dzm = fabs(Zn - zk);
        double w = (1.0 - dxm * idxi) * (1.0 - dzm * idzi);
        int p = mphase[k];
        Wm += w;
#pragma unroll
        for (int pp = 0; pp < NPH; pp++)
            if (p == pp) Wph[pp] += w;
#pragma unroll
        for (int f = 0; f < NF; f++) {
            double v = F.per_phase[f] ? F.val[f][p] : F.val[f][k];
            if (F.avg[f] == 1) v = 1.0 / v;
            if (F.avg[f] == 2) v = log(v);
            BmWm[f] += v * w;
        }
    };
    // Markers in the order the reference's loop meets them: cell rows
    // upwards, cells left to right, markers by index inside a cell.
    const bool cellnode = kindx == 0 && kindz == 0;   // centroids: the bin cell is the nearest centroid
    for (int r = rlo; r <= rhi; r++) {
        if (cellnode) {
            for (int c = clo; c <= chi; c++) {
                const int di = i - c, dj = j - r;
                if (di < -h || di > h || dj < -h || dj > h) continue;
                const int cell = c + r * ncx;
                for (int q = start[cell], e = start[cell + 1]; q < e; q++) add(sorted[q], c, r, di, dj);
            }
            continue;
        }
        int b = start[clo + r * ncx], e = start[chi + r * ncx + 1];
        for (int q = b; q < e; q++) {
            int ip, jp;
            if (qvert) {   // vertices: the stored nearest vertex
                const int pk = qvert[q];
                ip = pk & 0xffff;
                jp = pk >> 16;
            } else {
                const int k = sorted[q];
                ip = nearest_line(mx[k], X0, dx, idx, nnx);
                jp = nearest_line(mz[k], Z0, dz, idz, nnz);
            }
            int di = i - ip, dj = j - jp;
            if (di < -h || di > h || dj < -h || dj > h) continue;
            add(sorted[q], ip, jp, di, dj);
        }
    }
    const bool air = tag[node] == 30 || tag[node] == 31;
    bool skip = fabs(Wm) < 1e-30 || air;
    if (F.empty && phase_perc && !air && fabs(Wm) < 1e-30) atomicAdd(F.empty, 1);
#pragma unroll
    for (int f = 0; f < NF; f++) {
        if (skip) continue;
        double v = BmWm[f] / Wm;
        if (F.avg[f] == 1) v = 1.0 / v;
        if (F.avg[f] == 2) v = exp(v);
        F.out[f][node] = v;
    }
    if (phase_perc) {
        int nn = nnx * nnz;
#pragma unroll
        for (int p = 0; p < NPH; p++)
            if (p < nph_rt) phase_perc[(size_t)p * nn + node] = skip ? Wph[p] : Wph[p] / Wm;
    }
}

template <int NF>
static void launch_p2g_nf(int nph, dim3 gr, dim3 bl, cudaStream_t st, int nnx, int nnz, const double *X,
                          const double *Z, const signed char *tag, int kx, int kz, int h, double dx, double dz,
                          double dxi, double dzi, int ncx, int ncz, const mdz_ctx *ctx, const p2g_fields &F,
                          double *pp) {
    const mdz_bins &B = ctx->bins;
    const int *qv = kx == 1 && kz == 1 ? B.qvert : nullptr;   // vertex lines in both directions
    if (pp == nullptr || nph <= 0)
        k_p2g_gather<NF, 0><<<gr, bl, 0, st>>>(nnx, nnz, X, Z, tag, kx, kz, h, dx, dz, 1.0 / dx, 1.0 / dz, 1.0 / dxi,
                                               1.0 / dzi, ncx, ncz, B.start,
                                               B.sorted, qv, ctx->m.x, ctx->m.z, ctx->m.phase, F, 0, nullptr);
    else if (nph <= 4)
        k_p2g_gather<NF, 4><<<gr, bl, 0, st>>>(nnx, nnz, X, Z, tag, kx, kz, h, dx, dz, 1.0 / dx, 1.0 / dz, 1.0 / dxi,
                                               1.0 / dzi, ncx, ncz, B.start,
                                               B.sorted, qv, ctx->m.x, ctx->m.z, ctx->m.phase, F, nph, pp);
    else
        k_p2g_gather<NF, MDZ_MAX_PHASES><<<gr, bl, 0, st>>>(nnx, nnz, X, Z, tag, kx, kz, h, dx, dz, 1.0 / dx, 1.0 / dz,
                                                            1.0 / dxi, 1.0 / dzi, ncx, ncz, B.start, B.sorted, qv, ctx->m.x,
                                                            ctx->m.z, ctx->m.phase, F, nph, pp);
}

// Core projection on the resident markers (device pointers everywhere).
static mdz_status p2g_core(mdz_ctx *ctx, const p2g_fields &F, int nf, double *d_phase_perc, int centroid,
                           int itp_stencil, cudaStream_t st) {
    if (itp_stencil != 1 && itp_stencil != 9)
        return mdz_fail(ctx, MDZ_ERR_ARG, "P2G: itp_stencil must be 1 or 9 (got %d)", itp_stencil);
    if (centroid < -2 || centroid > 1) return mdz_fail(ctx, MDZ_ERR_ARG, "P2G: bad node set %d", centroid);
    if (nf < 0 || nf > MDZ_P2G_MAX_FIELDS) return mdz_fail(ctx, MDZ_ERR_ARG, "P2G: too many fields (%d)", nf);
    mdz_status s = mdz_ensure_bins(ctx, st);
    if (s != MDZ_OK) return s;
    const mdz_dgrid &g = ctx->g;
    mdz_nodeset ns = mdz_get_nodeset(ctx, centroid);
    int kx = centroid == MDZ_NODES_CENTROIDS ? 0 : (centroid == MDZ_NODES_VZ ? 2 : 1);
    int kz = centroid == MDZ_NODES_CENTROIDS ? 0 : (centroid == MDZ_NODES_VX ? 2 : 1);
    int h = itp_stencil == 9 ? 1 : 0;
    double dxi = itp_stencil == 9 ? 3.0 * g.dx / 2.0 : g.dx / 2.0;
    double dzi = itp_stencil == 9 ? 3.0 * g.dz / 2.0 : g.dz / 2.0;
    int nn = ns.nx * ns.nz;
    dim3 bl(128), gr(mdz_blocks(nn, 128));
    int nph = d_phase_perc ? ctx->n_phases : 0;
    p2g_fields Fc = F;
    Fc.empty = d_phase_perc ? ctx->p2g_empty : nullptr;
    cudaEvent_t ev;
    mdz_prof_begin(ctx, MDZ_PROF_P2G, st, &ev);
    switch (nf) {
#define CASE(N) case N: launch_p2g_nf<N>(nph, gr, bl, st, ns.nx, ns.nz, ns.X, ns.Z, ns.tag, kx, kz, h, g.dx, g.dz, dxi, dzi, g.ncx, g.ncz, ctx, Fc, d_phase_perc); break;
        CASE(0) CASE(1) CASE(2) CASE(3) CASE(4) CASE(5) CASE(6) CASE(7) CASE(8)
#undef CASE
    }
    MDZ_LAUNCHED(ctx);
    {   // algorithmic bytes: each marker's position, phase and per-marker
        // fields read once; each node's fields and phase fractions written once
        int nfm = 0;
        for (int f = 0; f < nf; f++) nfm += F.per_phase[f] ? 0 : 1;
        const double bytes = (double)ctx->m.n * (20.0 + 8.0 * nfm) + 8.0 * (double)nn * (nf + nph);
        mdz_prof_end(ctx, MDZ_PROF_P2G, bytes, st, ev);
    }
    return MDZ_OK;
}

extern "C" mdz_status mdz_dev_p2g(mdz_ctx *ctx, int n_fields, const double *const *d_values, const int *avg,
                                  double *const *d_out, double *d_phase_perc, int centroid, int itp_stencil,
                                  void *stream) {
    if (!ctx) return MDZ_ERR_ARG;
    if (n_fields < 0 || n_fields > MDZ_P2G_MAX_FIELDS || (n_fields > 0 && (!d_values || !avg || !d_out)))
        return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_dev_p2g: bad field arguments");
    if (d_phase_perc && centroid != MDZ_NODES_CENTROIDS && centroid != MDZ_NODES_VERTICES)
        return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_dev_p2g: phase fractions exist on centroids and vertices only");
    p2g_fields F{};
    for (int f = 0; f < n_fields; f++) {
        if (avg[f] < 0 || avg[f] > 2) return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_dev_p2g: avg must be 0, 1 or 2");
        F.val[f] = d_values[f]; F.per_phase[f] = 0; F.avg[f] = avg[f]; F.out[f] = d_out[f];
    }
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    return p2g_core(ctx, F, n_fields, d_phase_perc, centroid, itp_stencil, st);
}

extern "C" mdz_status mdz_P2Mastah(mdz_ctx *ctx, const double *mat_prop, double *node_field,
                                   const signed char *node_type, int flag, int avg, int prop, int centroid,
                                   int itp_stencil, double *phase_perc) {
    if (!ctx) return MDZ_ERR_ARG;
    if (centroid < -2 || centroid > 1) return mdz_fail(ctx, MDZ_ERR_ARG, "P2Mastah: bad node set %d", centroid);
    if (flag != 0 && flag != 1) return mdz_fail(ctx, MDZ_ERR_ARG, "P2Mastah: flag must be 0 or 1");
    if (avg < 0 || avg > 2) return mdz_fail(ctx, MDZ_ERR_ARG, "P2Mastah: avg must be 0, 1 or 2");
    if (prop == 1 && (!phase_perc || (centroid != 0 && centroid != 1)))
        return mdz_fail(ctx, MDZ_ERR_ARG, "P2Mastah: prop=1 needs phase_perc on centroids or vertices");
    if (prop == 0 && (!mat_prop || !node_field)) return mdz_fail(ctx, MDZ_ERR_ARG, "P2Mastah: null field pointers");
    cudaStream_t st = ctx->stream;
    mdz_nodeset ns = mdz_get_nodeset(ctx, centroid);
    size_t nn = (size_t)ns.nx * ns.nz;
    int n = ctx->m.n;
    // node tags: the caller's array decides which nodes are skipped
    signed char *dtag = nullptr;
    if (node_type) {
        dtag = (signed char *)mdz_stage(ctx, 3, nn);
        if (!dtag) return mdz_fail(ctx, MDZ_ERR_CUDA, "P2Mastah: staging allocation failed");
        MDZ_CUDA(ctx, cudaMemcpyAsync(dtag, node_type, nn, cudaMemcpyHostToDevice, st));
    }
    p2g_fields F{};
    int nf = 0;
    double *dout = nullptr, *dpp = nullptr;
    if (prop == 0) {
        size_t nval = flag == 0 ? (size_t)ctx->n_phases : (size_t)n;
        double *dval = (double *)mdz_stage(ctx, 0, sizeof(double) * (nval ? nval : 1));
        dout = (double *)mdz_stage(ctx, 1, sizeof(double) * nn);
        if (!dval || !dout) return mdz_fail(ctx, MDZ_ERR_CUDA, "P2Mastah: staging allocation failed");
        if (nval) MDZ_CUDA(ctx, cudaMemcpyAsync(dval, mat_prop, sizeof(double) * nval, cudaMemcpyHostToDevice, st));
        MDZ_CUDA(ctx, cudaMemcpyAsync(dout, node_field, sizeof(double) * nn, cudaMemcpyHostToDevice, st));
        F.val[0] = dval; F.per_phase[0] = flag == 0; F.avg[0] = avg; F.out[0] = dout;
        nf = 1;
    } else {
        dpp = (double *)mdz_stage(ctx, 2, sizeof(double) * nn * ctx->n_phases);
        if (!dpp) return mdz_fail(ctx, MDZ_ERR_CUDA, "P2Mastah: staging allocation failed");
    }
    // swap in the caller's tags for this call
    mdz_dgrid saved = ctx->g;
    if (dtag) {
        if (centroid == 1) ctx->g.BCp = dtag;
        else if (centroid == 0) ctx->g.BCg = dtag;
        else if (centroid == -1) ctx->g.BCu = dtag;
        else ctx->g.BCv = dtag;
    }
    mdz_status s = p2g_core(ctx, F, nf, dpp, centroid, itp_stencil, st);
    ctx->g = saved;
    if (s != MDZ_OK) return s;
    if (prop == 0) MDZ_CUDA(ctx, cudaMemcpyAsync(node_field, dout, sizeof(double) * nn, cudaMemcpyDeviceToHost, st));
    else MDZ_CUDA(ctx, cudaMemcpyAsync(phase_perc, dpp, sizeof(double) * nn * ctx->n_phases, cudaMemcpyDeviceToHost, st));
    MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    return MDZ_OK;
}

// ---------------------------------------------------------------------------
// Counts per cell / vertex and per (node, phase): integer, exact.
template <int NPH>
__global__ void k_count_nodes(int nnx, int nnz, int kindx, int kindz, const double *__restrict__ X,
                              const double *__restrict__ Z, double dx, double dz, int ncx, int ncz,
                              const int *__restrict__ start, const int *__restrict__ sorted,
                              const double *__restrict__ mx, const double *__restrict__ mz,
                              const int *__restrict__ mphase, int nph, int *__restrict__ count,
                              int *__restrict__ phase_count) {
    int node = blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= nnx * nnz) return;
    int i = node % nnx, j = node / nnx;
    int clo, chi, rlo, rhi;
    cell_range(i, 0, kindx, nnx, ncx, clo, chi);
    cell_range(j, 0, kindz, nnz, ncz, rlo, rhi);
    int cnt = 0, pc[NPH];
#pragma unroll
    for (int p = 0; p < NPH; p++) pc[p] = 0;
    for (int r = rlo; r <= rhi; r++) {
        int b = start[clo + r * ncx], e = start[chi + r * ncx + 1];
        for (int q = b; q < e; q++) {
            int k = sorted[q];
            if (nearest_line(mx[k], X[0], dx, 1.0 / dx, nnx) != i || nearest_line(mz[k], Z[0], dz, 1.0 / dz, nnz) != j)
                continue;
            int p = mphase[k];
            if (p < 0) continue;
            cnt++;
#pragma unroll
            for (int pp = 0; pp < NPH; pp++)
                if (p == pp) pc[pp]++;
        }
    }
    if (count) count[node] = cnt;
    if (phase_count) {
        int nn = nnx * nnz;
#pragma unroll
        for (int p = 0; p < NPH; p++)
            if (p < nph) phase_count[(size_t)p * nn + node] = pc[p];
    }
}

extern "C" mdz_status mdz_count_markers(mdz_ctx *ctx, int *nb_part_cell, int *nb_part_vert, int *phase_count_cell,
                                        int *phase_count_vert) {
    if (!ctx) return MDZ_ERR_ARG;
    cudaStream_t st = ctx->stream;
    mdz_status s = mdz_ensure_bins(ctx, st);
    if (s != MDZ_OK) return s;
    const mdz_dgrid &g = ctx->g;
    for (int which = 0; which < 2; which++) {
        int *hc = which ? nb_part_vert : nb_part_cell;
        int *hp = which ? phase_count_vert : phase_count_cell;
        if (!hc && !hp) continue;
        int centroid = which ? MDZ_NODES_VERTICES : MDZ_NODES_CENTROIDS;
        mdz_nodeset ns = mdz_get_nodeset(ctx, centroid);
        int nn = ns.nx * ns.nz, kind = which ? 1 : 0;
        int *dc = (int *)mdz_stage(ctx, 4, sizeof(int) * nn);
        int *dp = (int *)mdz_stage(ctx, 5, sizeof(int) * (size_t)nn * ctx->n_phases);
        if (!dc || !dp) return mdz_fail(ctx, MDZ_ERR_CUDA, "count: staging allocation failed");
        if (ctx->n_phases <= 4)
            k_count_nodes<4><<<mdz_blocks(nn), MDZ_THREADS, 0, st>>>(ns.nx, ns.nz, kind, kind, ns.X, ns.Z, g.dx, g.dz,
                                                                    g.ncx, g.ncz, ctx->bins.start, ctx->bins.sorted,
                                                                    ctx->m.x, ctx->m.z, ctx->m.phase, ctx->n_phases,
                                                                    dc, dp);
        else
            k_count_nodes<MDZ_MAX_PHASES><<<mdz_blocks(nn), MDZ_THREADS, 0, st>>>(
                ns.nx, ns.nz, kind, kind, ns.X, ns.Z, g.dx, g.dz, g.ncx, g.ncz, ctx->bins.start, ctx->bins.sorted,
                ctx->m.x, ctx->m.z, ctx->m.phase, ctx->n_phases, dc, dp);
        MDZ_LAUNCHED(ctx);
        if (hc) MDZ_CUDA(ctx, cudaMemcpyAsync(hc, dc, sizeof(int) * nn, cudaMemcpyDeviceToHost, st));
        if (hp) MDZ_CUDA(ctx, cudaMemcpyAsync(hp, dp, sizeof(int) * (size_t)nn * ctx->n_phases, cudaMemcpyDeviceToHost, st));
        MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    }
    return MDZ_OK;
}

// ---------------------------------------------------------------------------
// Grid -> marker.  Interp_Grid2P on a node set with lines X (n x) and Z (n z).
__device__ __forceinline__ bool air(signed char t) { return t == 30 || t == 31; }

__device__ double g2p_bilinear(double xk, double zk, const double *__restrict__ F, const double *__restrict__ X,
                               const double *__restrict__ Z, int Nx, int Nz, const signed char *__restrict__ tag,
                               double dx, double dz) {
    const double idx = 1.0 / dx, idz = 1.0 / dz;
    int jp = lower_line(xk, X[0], dx, idx);
    if (jp < 0) jp = 0;
    if (jp > Nx - 2) jp = Nx - 2;
    int ip = lower_line(zk, Z[0], dz, idz);
    if (ip < 0) ip = 0;
    if (ip > Nz - 2) ip = Nz - 2;
    double dxm = fabs(xk - X[jp]), dzm = fabs(zk - Z[ip]);
    int iSW = jp + ip * Nx, iSE = iSW + 1, iNW = jp + (ip + 1) * Nx, iNE = iNW + 1;
    double v = 0.0;
    const double wx = dxm * idx, wz = dzm * idz;
    v += (1.0 - wx) * (1.0 - wz) * (air(tag[iSW]) ? F[iNW] : F[iSW]);
    v += wx * (1.0 - wz) * (air(tag[iSE]) ? F[iNE] : F[iSE]);
    v += (1.0 - wx) * wz * (air(tag[iNW]) ? F[iSW] : F[iNW]);
    v += wx * wz * (air(tag[iNE]) ? F[iSE] : F[iNE]);
    return v;
}

__global__ void k_g2p_nodes(int n, const double *__restrict__ mx, const double *__restrict__ mz,
                            const int *__restrict__ mphase, const double *__restrict__ F, const double *__restrict__ X,
                            const double *__restrict__ Z, int Nx, int Nz, const signed char *__restrict__ tag,
                            double dx, double dz, double *__restrict__ out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    if (mphase[k] == -1) { out[k] = 0.0; return; }
    out[k] = g2p_bilinear(mx[k], mz[k], F, X, Z, Nx, Nz, tag, dx, dz);
}

// Interp_Grid2P_centroids2, non-periodic: centroid field (ncx x ncz) in the
// ghosted frame xvz/zvx; outside ring rows/columns repeat the edge value.
__global__ void k_g2p_centroids_ext(int n, const double *__restrict__ mx, const double *__restrict__ mz,
                                    const int *__restrict__ mphase, const double *__restrict__ F,
                                    const double *__restrict__ xvz, const double *__restrict__ zvx, int ncx, int ncz,
                                    const signed char *__restrict__ tag, double dx, double dz,
                                    double *__restrict__ out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    if (mphase[k] == -1) { out[k] = 0.0; return; }
    double xk = mx[k], zk = mz[k];
    const double idx = 1.0 / dx, idz = 1.0 / dz;
    int jp = lower_line(xk, xvz[0], dx, idx);
    int ip = lower_line(zk, zvx[0], dz, idz);
    int jw, je, is, in_;   // centroid columns west/east and rows south/north
    if (jp > 0 && jp < ncx) { jw = jp - 1; je = jp; }
    else if (jp <= 0) { jw = 0; je = 0; }
    else { jw = ncx - 1; je = ncx - 1; }
    if (ip > 0 && ip < ncz) { is = ip - 1; in_ = ip; }
    else if (ip <= 0) { is = 0; in_ = 0; }
    else { is = ncz - 1; in_ = ncz - 1; }
    int iSW = jw + is * ncx, iSE = je + is * ncx, iNW = jw + in_ * ncx, iNE = je + in_ * ncx;
    // clamp the line index used for the distances like the reference's ranges
    int jx = jp < 0 ? 0 : (jp > ncx ? ncx : jp);
    int iz = ip < 0 ? 0 : (ip > ncz ? ncz : ip);
    double dxm = xk - xvz[jx], dzm = zk - zvx[iz];
    double v = 0.0;
    const double wx = dxm * idx, wz = dzm * idz;
    v += (1.0 - wx) * (1.0 - wz) * (air(tag[iSW]) ? F[iNW] : F[iSW]);
    v += wx * (1.0 - wz) * (air(tag[iSE]) ? F[iNE] : F[iSE]);
    v += (1.0 - wx) * wz * (air(tag[iNW]) ? F[iSW] : F[iNW]);
    v += wx * wz * (air(tag[iNE]) ? F[iSE] : F[iNE]);
    out[k] = v;
}

extern "C" mdz_status mdz_Interp_Grid2P(mdz_ctx *ctx, const double *node_field, int node_set, double *marker_field) {
    if (!ctx) return MDZ_ERR_ARG;
    if (!node_field || !marker_field) return mdz_fail(ctx, MDZ_ERR_ARG, "Interp_Grid2P: null pointer");
    if (node_set < -2 || node_set > 1) return mdz_fail(ctx, MDZ_ERR_ARG, "Interp_Grid2P: bad node set");
    cudaStream_t st = ctx->stream;
    const mdz_dgrid &g = ctx->g;
    mdz_nodeset ns = mdz_get_nodeset(ctx, node_set);
    size_t nn = (size_t)ns.nx * ns.nz;
    int n = ctx->m.n;
    double *dF = (double *)mdz_stage(ctx, 0, sizeof(double) * nn);
    double *dO = (double *)mdz_stage(ctx, 1, sizeof(double) * (n ? n : 1));
    if (!dF || !dO) return mdz_fail(ctx, MDZ_ERR_CUDA, "Interp_Grid2P: staging allocation failed");
    MDZ_CUDA(ctx, cudaMemcpyAsync(dF, node_field, sizeof(double) * nn, cudaMemcpyHostToDevice, st));
    if (n > 0) {
        if (node_set == MDZ_NODES_CENTROIDS)
            k_g2p_centroids_ext<<<mdz_blocks(n), MDZ_THREADS, 0, st>>>(n, ctx->m.x, ctx->m.z, ctx->m.phase, dF, g.xvz,
                                                                       g.zvx, g.ncx, g.ncz, g.BCp, g.dx, g.dz, dO);
        else
            k_g2p_nodes<<<mdz_blocks(n), MDZ_THREADS, 0, st>>>(n, ctx->m.x, ctx->m.z, ctx->m.phase, dF, ns.X, ns.Z,
                                                               ns.nx, ns.nz, ns.tag, g.dx, g.dz, dO);
        MDZ_LAUNCHED(ctx);
        MDZ_CUDA(ctx, cudaMemcpyAsync(marker_field, dO, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    }
    MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    return MDZ_OK;
}

// ---------------------------------------------------------------------------
// RK4 advection.  V2P without the conservative correction: Vx bilinear on
// (xg, zvx) and Vz on (xvz, zg), lower-left cell ceil(d/h) - 1 clamped to
// [0, N-2], tag-30 substitutions as in the reference.
__device__ void v2p(double xk, double zk, const double *__restrict__ u, const double *__restrict__ v,
                    const double *__restrict__ xg, const double *__restrict__ zg, const double *__restrict__ zvx,
                    const double *__restrict__ xvz, int Nx, int Nz, const signed char *__restrict__ tu,
                    const double dx, const double dz, const double idx, const double idz,
                    const signed char *__restrict__ tv, double &vxm, double &vzm) {
    // Vx: Nx x (Nz+1)
    {
        int nx = Nx, nz = Nz + 1;
        int jp = lower_line(xk, xg[0], dx, idx);
        jp = jp < 0 ? 0 : (jp > nx - 2 ? nx - 2 : jp);
        int ip = lower_line(zk, zvx[0], dz, idz);
        ip = ip < 0 ? 0 : (ip > nz - 2 ? nz - 2 : ip);
        double dxm = fabs(xk - xg[jp]), dzm = fabs(zk - zvx[ip]);
        int iSW = jp + ip * nx, iSE = iSW + 1, iNW = jp + (ip + 1) * nx, iNE = iNW + 1;
        double VNW = u[iNW], VNE = u[iNE], VSW = u[iSW], VSE = u[iSE];
        if (tu[iSW] == 30) VSW = u[iNW];
        if (tu[iSE] == 30) VSE = u[iNE];
        if (tu[iNW] == 30) VNW = u[iSW];
        if (tu[iNE] == 30) VNE = u[iSE];
        if (tu[iNE] == 30 && tu[iSE] == 30) { VNE = VSW; VSE = VSW; }
        if (tu[iNW] == 30 && tu[iSW] == 30) { VNW = VSE; VSW = VSE; }
        const double wx = dxm * idx, wz = dzm * idz;
        double v13 = VSW * (1.0 - wx) + VSE * wx;
        double v24 = VNW * (1.0 - wx) + VNE * wx;
        vxm = (1.0 - wz) * v13 + wz * v24;
    }
    // Vz: (Nx+1) x Nz
    {
        int nx = Nx + 1, nz = Nz;
        int jp = lower_line(xk, xvz[0], dx, idx);
        jp = jp < 0 ? 0 : (jp > nx - 2 ? nx - 2 : jp);
        int ip = lower_line(zk, zg[0], dz, idz);
        ip = ip < 0 ? 0 : (ip > nz - 2 ? nz - 2 : ip);
        double dxm = fabs(xk - xvz[jp]), dzm = fabs(zk - zg[ip]);
        int iSW = jp + ip * nx, iSE = iSW + 1, iNW = jp + (ip + 1) * nx, iNE = iNW + 1;
        double VSE = v[iSE], VSW = v[iSW], VNE = v[iNE], VNW = v[iNW];
        if (tv[iSW] == 30) VSW = v[iNE];
        if (tv[iSE] == 30) VSE = v[iNE];
        if (tv[iNW] == 30) VNW = v[iSW];
        if (tv[iNE] == 30) VNE = v[iSE];
        if (tv[iNE] == 30 && tv[iSE] == 30) { VNE = VSW; VSE = VSW; }
        if (tv[iNW] == 30 && tv[iSW] == 30) { VNW = VSE; VSW = VSE; }
        const double wx = dxm * idx, wz = dzm * idz;
        double v12 = VSW * (1.0 - wz) + VNW * wz;
        double v34 = VSE * (1.0 - wz) + VNE * wz;
        vzm = (1.0 - wx) * v12 + wx * v34;
    }
}

__global__ void k_rk4(int n, double *__restrict__ mx, double *__restrict__ mz, int *__restrict__ mphase,
                      double *__restrict__ mvx, double *__restrict__ mvz, const double *__restrict__ u,
                      const double *__restrict__ v, const double *__restrict__ xg, const double *__restrict__ zg,
                      const double *__restrict__ zvx, const double *__restrict__ xvz, int Nx, int Nz,
                      const signed char *__restrict__ tu, const signed char *__restrict__ tv, double dx, double dz,
                      double idx, double idz, double dt, double xmin, double xmax, double zmin, double zmax) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int ph = mphase[k];
    double xA = mx[k], zA = mz[k], x = xA, z = zA;
    double VxA = 0, VzA = 0, VxB = 0, VzB = 0, VxC = 0, VzC = 0, VxD = 0, VzD = 0;
#define OUT_CHECK() if (x < xmin || x > xmax || z < zmin || z > zmax) ph = -1;
    if (ph != -1) v2p(x, z, u, v, xg, zg, zvx, xvz, Nx, Nz, tu, dx, dz, idx, idz, tv, VxA, VzA);
    if (ph != -1) { x = xA + 0.5 * dt * VxA; z = zA + 0.5 * dt * VzA; }
    OUT_CHECK();
    if (ph != -1) v2p(x, z, u, v, xg, zg, zvx, xvz, Nx, Nz, tu, dx, dz, idx, idz, tv, VxB, VzB);
    if (ph != -1) { x = xA + 0.5 * dt * VxB; z = zA + 0.5 * dt * VzB; }
    OUT_CHECK();
    if (ph != -1) v2p(x, z, u, v, xg, zg, zvx, xvz, Nx, Nz, tu, dx, dz, idx, idz, tv, VxC, VzC);
    if (ph != -1) { x = xA + 1.0 * dt * VxC; z = zA + 1.0 * dt * VzC; }
    OUT_CHECK();
    if (ph != -1) v2p(x, z, u, v, xg, zg, zvx, xvz, Nx, Nz, tu, dx, dz, idx, idz, tv, VxD, VzD);
    VxA = (1.0 / 6.0) * (VxA + 2.0 * VxB + 2.0 * VxC + VxD);
    VzA = (1.0 / 6.0) * (VzA + 2.0 * VzB + 2.0 * VzC + VzD);
    if (ph != -1) {
        x = xA + dt * VxA; z = zA + dt * VzA;
        mvx[k] = VxA; mvz[k] = VzA;
    }
    OUT_CHECK();
#undef OUT_CHECK
    mx[k] = x; mz[k] = z; mphase[k] = ph;
}

mdz_status mdz_dev_rk4(mdz_ctx *ctx, const double *du, const double *dv, double dt, cudaStream_t st) {
    const mdz_dgrid &g = ctx->g;
    int n = ctx->m.n;
    if (n > 0) {
        k_rk4<<<mdz_blocks(n), MDZ_THREADS, 0, st>>>(n, ctx->m.x, ctx->m.z, ctx->m.phase, ctx->m.vx, ctx->m.vz, du, dv,
                                                     g.xg, g.zg, g.zvx, g.xvz, g.Nx, g.Nz, g.BCu, g.BCv, g.dx, g.dz,
                                                     g.idx, g.idz, dt, g.xmin, g.xmax, g.zmin, g.zmax);
        MDZ_LAUNCHED(ctx);
    }
    ctx->bins.valid = false;
    return MDZ_OK;
}

extern "C" mdz_status mdz_RogerGuntherII(mdz_ctx *ctx, const double *u, const double *v, double dt) {
    if (!ctx) return MDZ_ERR_ARG;
    if (!u || !v) return mdz_fail(ctx, MDZ_ERR_ARG, "RogerGuntherII: null velocity");
    cudaStream_t st = ctx->stream;
    const mdz_dgrid &g = ctx->g;
    size_t nu = (size_t)g.Nx * (g.Nz + 1), nv = (size_t)(g.Nx + 1) * g.Nz;
    double *du = (double *)mdz_stage(ctx, 0, sizeof(double) * nu);
    double *dv = (double *)mdz_stage(ctx, 1, sizeof(double) * nv);
    if (!du || !dv) return mdz_fail(ctx, MDZ_ERR_CUDA, "RogerGuntherII: staging allocation failed");
    MDZ_CUDA(ctx, cudaMemcpyAsync(du, u, sizeof(double) * nu, cudaMemcpyHostToDevice, st));
    MDZ_CUDA(ctx, cudaMemcpyAsync(dv, v, sizeof(double) * nv, cudaMemcpyHostToDevice, st));
    mdz_status s = mdz_dev_rk4(ctx, du, dv, dt, st);
    if (s != MDZ_OK) return s;
    MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    return MDZ_OK;
}
