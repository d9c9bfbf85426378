// Output preparation: the data-parallel part of WriteOutputHDF5
// (SOURCE/HDF5Output.c:237-895) for the state this library keeps.
//
//   mdz_Interp_Phase2VizGrid  closest-marker phase map on a visualisation grid
//                             (SOURCE/ParticleRoutines.c:3004-3095, called by
//                             HDF5Output.c:266-297 at 1x and 2x resolution)
//   mdz_output_field          a resident field cast to float and scaled back to
//                             dimensional units (DoubleToFloat + ScaleBack,
//                             HDF5Output.c:44-73)
//
// The HDF5 calls themselves stay with the caller (the library is a host
// dependency of the reference and not part of this path).
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>
#include "mdz_internal.cuh"

namespace {

// Visualisation cell of marker k and its weight, with the reference's
// arithmetic (divisions by the visualisation spacing, the nearest-line index
// through ceil of the correctly rounded quotient); false when the marker
// cannot mark the map (inactive, in an air centroid, zero weight).
struct viz_geom {
    const double *X, *Z;   // visualisation lines (nxv, nzv)
    int nx, nz;            // visualisation cells
    double dxv, dzv;       // X[1] - X[0], Z[1] - Z[0]
    double xc0, zc0, dx, dz, idx, idz;   // centroid lines of the grid
    int ncx, ncz;
};

__device__ __forceinline__ bool viz_weight(const viz_geom &V, double x, double z, const signed char *bcp, int &cell,
                                           double &w) {
    int j = (int)ceil_quot(x - (V.X[0] + 0.5 * V.dxv), V.dxv, 1.0 / V.dxv, 0.5) - 1;
    j = j < 0 ? 0 : (j > V.nx - 1 ? V.nx - 1 : j);
    int i = (int)ceil_quot(z - (V.Z[0] + 0.5 * V.dzv), V.dzv, 1.0 / V.dzv, 0.5) - 1;
    i = i < 0 ? 0 : (i > V.nz - 1 ? V.nz - 1 : i);
    const double dxm = fabs(0.5 * (V.X[j] + V.X[j + 1]) - x);
    const double dzm = fabs(0.5 * (V.Z[i + 1] + V.Z[i]) - z);
    int ic = (int)ceil_quot(x - V.xc0, V.dx, V.idx, 0.5) - 1;
    ic = ic < 0 ? 0 : (ic > V.ncx - 1 ? V.ncx - 1 : ic);
    int jc = (int)ceil_quot(z - V.zc0, V.dz, V.idz, 0.5) - 1;
    jc = jc < 0 ? 0 : (jc > V.ncz - 1 ? V.ncz - 1 : jc);
    const signed char flag = bcp[ic + jc * V.ncx];
    if (flag == 30 || flag == 31) return false;
    w = (1.0 - (dxm / V.dxv)) * (1.0 - (dzm / V.dzv));
    cell = j + i * V.nx;
    return w > 0.0;
}

// The reference keeps, per visualisation cell, the first marker (in index
// order) whose weight exceeds every earlier one's: the largest weight, the
// smallest index among equal weights.  Pass 1 takes the largest weight per
// cell (positive doubles order as their bit patterns), pass 2 the smallest
// index attaining it, pass 3 writes the phases.
__global__ void k_viz_max(int n, const double *__restrict__ mx, const double *__restrict__ mz,
                          const int *__restrict__ ph, viz_geom V, const signed char *__restrict__ bcp,
                          unsigned long long *__restrict__ wmax) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n || ph[k] == -1) return;
    int c;
    double w;
    if (viz_weight(V, mx[k], mz[k], bcp, c, w)) atomicMax(&wmax[c], (unsigned long long)__double_as_longlong(w));
}

__global__ void k_viz_first(int n, const double *__restrict__ mx, const double *__restrict__ mz,
                            const int *__restrict__ ph, viz_geom V, const signed char *__restrict__ bcp,
                            const unsigned long long *__restrict__ wmax, int *__restrict__ win) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n || ph[k] == -1) return;
    int c;
    double w;
    if (viz_weight(V, mx[k], mz[k], bcp, c, w) && (unsigned long long)__double_as_longlong(w) == wmax[c])
        atomicMin(&win[c], k);
}

__global__ void k_viz_fill(int nc, const int *__restrict__ win, const int *__restrict__ ph,
                           signed char *__restrict__ compo) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < nc) compo[c] = win[c] == INT_MAX ? (signed char)-1 : (signed char)ph[win[c]];
}

__global__ void k_win_init(int nc, int *__restrict__ win) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < nc) win[c] = INT_MAX;
}

// FieldF = (float) FieldD, then FieldF = FieldF * scale (a double product
// rounded to float), as DoubleToFloat and ScaleBack do
__global__ void k_cast_scale(size_t n, const double *__restrict__ a, double scale, float *__restrict__ out) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float f = (float)a[i];
    out[i] = (float)((double)f * scale);
}

}  // namespace

extern "C" mdz_status mdz_Interp_Phase2VizGrid(mdz_ctx *ctx, int res_fact, signed char *compo, double *xviz,
                                               double *zviz) {
    if (!ctx) return MDZ_ERR_ARG;
    if (res_fact < 1 || res_fact > 16 || !compo)
        return mdz_fail(ctx, MDZ_ERR_ARG, "Interp_Phase2VizGrid: res_fact 1..16 and an output array");
    const mdz_dgrid &g = ctx->g;
    const mdz_grid_desc &h = ctx->host_desc;
    const int nxv = res_fact * (g.Nx - 1) + 1, nzv = res_fact * (g.Nz - 1) + 1;
    const int nx = nxv - 1, nz = nzv - 1, nc = nx * nz;
    // the visualisation lines as the reference builds them: by accumulation
    // from the first grid line (HDF5Output.c:270-276)
    std::vector<double> X(nxv), Z(nzv);
    X[0] = h.xg[0];
    Z[0] = h.zg[0];
    for (int k = 1; k < nxv; k++) X[k] = X[k - 1] + g.dx / res_fact;
    for (int k = 1; k < nzv; k++) Z[k] = Z[k - 1] + g.dz / res_fact;
    if (xviz) memcpy(xviz, X.data(), sizeof(double) * nxv);
    if (zviz) memcpy(zviz, Z.data(), sizeof(double) * nzv);
    cudaStream_t st = ctx->stream;
    const size_t bytes = sizeof(double) * (nxv + nzv) + sizeof(unsigned long long) * nc + sizeof(int) * nc + nc + 64;
    unsigned char *buf = (unsigned char *)mdz_stage(ctx, 2, bytes);
    if (!buf) return mdz_fail(ctx, MDZ_ERR_CUDA, "Interp_Phase2VizGrid: staging allocation failed");
    double *dX = (double *)buf, *dZ = dX + nxv;
    unsigned long long *wmax = (unsigned long long *)(dZ + nzv);
    int *win = (int *)(wmax + nc);
    signed char *dc = (signed char *)(win + nc);
    MDZ_CUDA(ctx, cudaMemcpyAsync(dX, X.data(), sizeof(double) * nxv, cudaMemcpyHostToDevice, st));
    MDZ_CUDA(ctx, cudaMemcpyAsync(dZ, Z.data(), sizeof(double) * nzv, cudaMemcpyHostToDevice, st));
    MDZ_CUDA(ctx, cudaMemsetAsync(wmax, 0, sizeof(unsigned long long) * nc, st));
    k_win_init<<<mdz_blocks(nc), MDZ_THREADS, 0, st>>>(nc, win);
    MDZ_LAUNCHED(ctx);
    viz_geom V{dX, dZ, nx, nz, X[1] - X[0], Z[1] - Z[0], h.xc[0], h.zc[0], g.dx, g.dz, g.idx, g.idz, g.ncx, g.ncz};
    const int n = ctx->m.n;
    if (n > 0) {
        k_viz_max<<<mdz_blocks(n), MDZ_THREADS, 0, st>>>(n, ctx->m.x, ctx->m.z, ctx->m.phase, V, g.BCp, wmax);
        MDZ_LAUNCHED(ctx);
        k_viz_first<<<mdz_blocks(n), MDZ_THREADS, 0, st>>>(n, ctx->m.x, ctx->m.z, ctx->m.phase, V, g.BCp, wmax, win);
        MDZ_LAUNCHED(ctx);
    }
    k_viz_fill<<<mdz_blocks(nc), MDZ_THREADS, 0, st>>>(nc, win, ctx->m.phase, dc);
    MDZ_LAUNCHED(ctx);
    MDZ_CUDA(ctx, cudaMemcpyAsync(compo, dc, nc, cudaMemcpyDeviceToHost, st));
    MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    return MDZ_OK;
}

extern "C" mdz_status mdz_output_field(mdz_ctx *ctx, const char *name, double scale, float *out) {
    if (!ctx) return MDZ_ERR_ARG;
    if (!name || !out) return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_output_field: null argument");
    mdz_status s = mdz_ensure_fields(ctx);
    if (s != MDZ_OK) return s;
    const double *src = nullptr;
    size_t n = 0;
#define PICK(fname, kind)                                        \
    if (!strcmp(name, #fname)) {                                 \
        src = ctx->d.fname;                                      \
        n = mdz_field_count(ctx, MDZ_K_##kind);                  \
    }
    MDZ_FIELD_LIST(PICK)
#undef PICK
    if (!src) return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_output_field: no resident field '%s'", name);
    cudaStream_t st = ctx->stream;
    float *d = (float *)mdz_stage(ctx, 2, sizeof(float) * n);
    if (!d) return mdz_fail(ctx, MDZ_ERR_CUDA, "mdz_output_field: staging allocation failed");
    k_cast_scale<<<mdz_blocks(n), MDZ_THREADS, 0, st>>>(n, src, scale, d);
    MDZ_LAUNCHED(ctx);
    MDZ_CUDA(ctx, cudaMemcpyAsync(out, d, sizeof(float) * n, cudaMemcpyDeviceToHost, st));
    MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    return MDZ_OK;
}
