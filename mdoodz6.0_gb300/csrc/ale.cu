// Deforming pure-shear box (PureShearALE, SOURCE/AdvectionRoutines.c:634-734,
// model.ispureshear_ale = 1 without a free surface): the walls move with the
// mean velocity of their Dirichlet nodes and the grid lines are regenerated
// over the new box (SetGridCoordinates, SOURCE/GridRoutines.c:230-300).
//
// The four wall sums are tiny (one line of nodes each) but their rounding
// decides the new bounds, so they are added in the reference's loop order:
// one warp per wall stages 32 values at a time in shared memory and its
// first lane adds them in sequence.  The bounds and the grid lines are then
// formed on the host exactly as SetGridCoordinates forms them (sequential
// accumulation of the spacing; host code is built without fused
// multiply-adds) and uploaded.
#include <cstring>
#include "mdz_internal.cuh"

mdz_status mdz_ensure_fields(mdz_ctx *ctx);

// out[2w] = sum, out[2w+1] = count of wall w: 0 west (Vx rows 0..Nz-1 of
// column 0, tag 0), 1 east (column Nx-1), 2 south (Vz columns 0..Nx-1 of row
// 0, tag 0), 3 north (row Nz-1, tag 0 or 30).  One block of 128 threads.
__global__ void k_wall_sums(mdz_dgrid g, const double *__restrict__ u, const double *__restrict__ v,
                            double *__restrict__ out) {
    __shared__ double val[4][32];
    __shared__ int take[4][32];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (w >= 4) return;
    const int Nx = g.Nx, Nz = g.Nz;
    const int n = w < 2 ? Nz : Nx;
    double s = 0.0;
    int cnt = 0;
    for (int base = 0; base < n; base += 32) {
        const int j = base + lane;
        double x = 0.0;
        int t = 0;
        if (j < n) {
            size_t c;
            if (w == 0) { c = (size_t)j * Nx; t = g.BCu[c] == 0; x = u[c]; }
            else if (w == 1) { c = (size_t)(Nx - 1) + (size_t)j * Nx; t = g.BCu[c] == 0; x = u[c]; }
            else if (w == 2) { c = (size_t)j; t = g.BCv[c] == 0; x = v[c]; }
            else { c = (size_t)j + (size_t)(Nz - 1) * (Nx + 1); t = g.BCv[c] == 0 || g.BCv[c] == 30; x = v[c]; }
        }
        val[w][lane] = x;
        take[w][lane] = t;
        __syncwarp();
        if (lane == 0) {
            const int m = n - base < 32 ? n - base : 32;
            for (int q = 0; q < m; q++)
                if (take[w][q]) { s += val[w][q]; cnt++; }
        }
        __syncwarp();
    }
    if (lane == 0) { out[2 * w] = s; out[2 * w + 1] = (double)cnt; }
}

// SetGridCoordinates on the context's host copies, then the device lines,
// the device grid's bounds and spacings and the solver levels.
static mdz_status set_grid_lines(mdz_ctx *ctx, cudaStream_t st) {
    mdz_grid_desc &d = ctx->host_desc;
    const int Nx = d.Nx, Nz = d.Nz;
    d.dx = (d.xmax - d.xmin) / (Nx - 1);
    d.dz = (d.zmax - d.zmin) / (Nz - 1);
    const double x0[6] = {d.xmin, d.zmin, d.xmin + d.dx / 2.0, d.zmin + d.dz / 2.0, d.xmin - d.dx / 2.0,
                          d.zmin - d.dz / 2.0};
    const double h[6] = {d.dx, d.dz, d.dx, d.dz, d.dx, d.dz};
    mdz_dgrid &g = ctx->g;
    double *dev[6] = {g.xg, g.zg, g.xc, g.zc, g.xvz, g.zvx};
    for (int i = 0; i < 6; i++) {
        std::vector<double> &line = ctx->hline[i];
        double c = x0[i];
        for (size_t k = 0; k < line.size(); k++) {
            line[k] = c;
            c = c + h[i];
        }
        MDZ_CUDA(ctx, cudaMemcpyAsync(dev[i], line.data(), sizeof(double) * line.size(), cudaMemcpyHostToDevice, st));
    }
    MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    g.dx = d.dx; g.dz = d.dz;
    g.idx = 1.0 / d.dx; g.idz = 1.0 / d.dz;
    g.xmin = d.xmin; g.xmax = d.xmax; g.zmin = d.zmin; g.zmax = d.zmax;
    ctx->bins.valid = false;
    return mdz_solver_regrid(ctx);
}

mdz_status mdz_set_box(mdz_ctx *ctx, double xmin, double xmax, double zmin, double zmax, cudaStream_t st) {
    mdz_grid_desc &d = ctx->host_desc;
    d.xmin = xmin; d.xmax = xmax; d.zmin = zmin; d.zmax = zmax;
    return set_grid_lines(ctx, st);
}

mdz_status mdz_dev_pure_shear_ale(mdz_ctx *ctx, const double *u, const double *v, double dt, cudaStream_t st) {
    if (!ctx->ale_sums) MDZ_CUDA(ctx, cudaMalloc((void **)&ctx->ale_sums, 8 * sizeof(double)));
    k_wall_sums<<<1, 128, 0, st>>>(ctx->g, u, v, ctx->ale_sums);
    MDZ_LAUNCHED(ctx);
    double s[8];
    MDZ_CUDA(ctx, cudaMemcpyAsync(s, ctx->ale_sums, sizeof s, cudaMemcpyDeviceToHost, st));
    MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    // the reference divides by its integer counts where they are positive
    double VxW = s[0], VxE = s[2], VzS = s[4], VzN = s[6];
    if (s[1] > 0) VxW /= (int)s[1];
    if (s[3] > 0) VxE /= (int)s[3];
    if (s[5] > 0) VzS /= (int)s[5];
    if (s[7] > 0) VzN /= (int)s[7];
    const double dxmin = VxW * dt, dxmax = VxE * dt, dzmin = VzS * dt, dzmax = VzN * dt;
    mdz_grid_desc &d = ctx->host_desc;
    const double xmin = d.xmin + dxmin, xmax = d.xmax + dxmax, zmin = d.zmin + dzmin, zmax = d.zmax + dzmax;
    if (!(xmax > xmin) || !(zmax > zmin))
        return mdz_fail(ctx, MDZ_ERR_STATE, "PureShearALE: the box would collapse (x %g..%g, z %g..%g)", xmin, xmax,
                        zmin, zmax);
    return mdz_set_box(ctx, xmin, xmax, zmin, zmax, st);
}

extern "C" mdz_status mdz_PureShearALE(mdz_ctx *ctx, const double *u_in, const double *v_in, double dt,
                                       double *bounds) {
    if (!ctx) return MDZ_ERR_ARG;
    if (!(dt >= 0.0)) return mdz_fail(ctx, MDZ_ERR_ARG, "PureShearALE: dt must be >= 0");
    mdz_status s = mdz_ensure_fields(ctx);
    if (s != MDZ_OK) return s;
    const mdz_dgrid &g = ctx->g;
    cudaStream_t st = ctx->stream;
    if (u_in)
        MDZ_CUDA(ctx, cudaMemcpyAsync(ctx->d.u, u_in, sizeof(double) * g.Nx * (g.Nz + 1), cudaMemcpyHostToDevice, st));
    if (v_in)
        MDZ_CUDA(ctx, cudaMemcpyAsync(ctx->d.v, v_in, sizeof(double) * (g.Nx + 1) * g.Nz, cudaMemcpyHostToDevice, st));
    if ((s = mdz_dev_pure_shear_ale(ctx, ctx->d.u, ctx->d.v, dt, st)) != MDZ_OK) return s;
    if (bounds) {
        const mdz_grid_desc &d = ctx->host_desc;
        bounds[0] = d.xmin; bounds[1] = d.xmax; bounds[2] = d.zmin; bounds[3] = d.zmax;
    }
    return MDZ_OK;
}

extern "C" mdz_status mdz_set_boundary_values(mdz_ctx *ctx, const double *BCu_val, const double *BCv_val) {
    if (!ctx) return MDZ_ERR_ARG;
    const mdz_dgrid &g = ctx->g;
    cudaStream_t st = ctx->stream;
    if (BCu_val)
        MDZ_CUDA(ctx, cudaMemcpyAsync(g.BCu_val, BCu_val, sizeof(double) * g.Nx * (g.Nz + 1), cudaMemcpyHostToDevice,
                                      st));
    if (BCv_val)
        MDZ_CUDA(ctx, cudaMemcpyAsync(g.BCv_val, BCv_val, sizeof(double) * (g.Nx + 1) * g.Nz, cudaMemcpyHostToDevice,
                                      st));
    MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    return MDZ_OK;
}

extern "C" mdz_status mdz_get_grid(mdz_ctx *ctx, double *box, double *xg, double *zg, double *xc, double *zc,
                                   double *xvz, double *zvx) {
    if (!ctx) return MDZ_ERR_ARG;
    const mdz_grid_desc &d = ctx->host_desc;
    if (box) {
        box[0] = d.xmin; box[1] = d.xmax; box[2] = d.zmin; box[3] = d.zmax; box[4] = d.dx; box[5] = d.dz;
    }
    double *out[6] = {xg, zg, xc, zc, xvz, zvx};
    for (int i = 0; i < 6; i++)
        if (out[i]) memcpy(out[i], ctx->hline[i].data(), sizeof(double) * ctx->hline[i].size());
    return MDZ_OK;
}
