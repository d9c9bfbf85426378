// Stokes operator launches (residual and linear apply, FP64 and FP32),
// residual norms, Krylov vector kernels with warp-shuffle reductions, and the
// host drop-ins EvaluateStokesResidualDecoupled / operator apply.
#include <cmath>
#include <cstring>
#include "mdz_internal.cuh"
#include "stokes_ops.cuh"
#include "stokes.cuh"

// ---------------------------------------------------------------------------
// y = K x (linear) or F = (K x - b) (residual), each row times the cell volume.
// Non-equation entries of y are written 0 so Krylov vectors stay masked.
template <typename T, bool NEWTON, bool RES>
__global__ void __launch_bounds__(256) k_stokes_apply(stokes_geom G, stokes_coefs<T> D, stokes_cvec<T> x,
                                                      stokes_vec<T> y, stokes_cvec<T> b, T celvol) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int Nx = G.Nx, Nz = G.Nz;
    if (i < Nx && j <= Nz) {            // Vx node (i, j)
        int c = i + j * Nx;
        T r = 0;
        if (G.BCu[c] == -1) {
            r = xrow<T, NEWTON>(G, D, x, i, j);
            if (RES) r -= b.u[c];
            r *= celvol;
        }
        y.u[c] = r;
    }
    if (i <= Nx && j < Nz) {            // Vz node (i, j)
        int c = i + j * (Nx + 1);
        T r = 0;
        if (G.BCv[c] == -1) {
            r = zrow<T, NEWTON>(G, D, x, i, j);
            if (RES) r -= b.v[c];
            r *= celvol;
        }
        y.v[c] = r;
    }
    if (i < Nx - 1 && j < Nz - 1) {     // centroid (i, j)
        int c = i + j * (Nx - 1);
        T r = 0;
        if (G.BCp[c] == -1) {
            r = crow<T>(G, x, i, j);
            if (RES) r -= b.p[c];
            r *= celvol;
        }
        y.p[c] = r;
    }
}

stokes_geom mdz_stokes_geom(const mdz_ctx *ctx) {
    const mdz_dgrid &g = ctx->g;
    return make_geom(g.Nx, g.Nz, g.dx, g.dz, g.BCu, g.BCv, g.BCp, g.BCg);
}

template <typename T>
void stokes_apply_launch(const stokes_geom &G, const stokes_coefs<T> &D, stokes_cvec<T> x, stokes_vec<T> y,
                         const stokes_cvec<T> *b, bool newton, cudaStream_t st) {
    dim3 bl(32, 8), gr((G.Nx + 1 + 31) / 32, (G.Nz + 1 + 7) / 8);
    T celvol = gc<T>(G, GC_CELVOL);
    stokes_cvec<T> bb = b ? *b : stokes_cvec<T>{nullptr, nullptr, nullptr};
    if (b) {
        if (newton) k_stokes_apply<T, true, true><<<gr, bl, 0, st>>>(G, D, x, y, bb, celvol);
        else k_stokes_apply<T, false, true><<<gr, bl, 0, st>>>(G, D, x, y, bb, celvol);
    } else {
        if (newton) k_stokes_apply<T, true, false><<<gr, bl, 0, st>>>(G, D, x, y, bb, celvol);
        else k_stokes_apply<T, false, false><<<gr, bl, 0, st>>>(G, D, x, y, bb, celvol);
    }
}
template void stokes_apply_launch<double>(const stokes_geom &, const stokes_coefs<double> &, stokes_cvec<double>,
                                          stokes_vec<double>, const stokes_cvec<double> *, bool, cudaStream_t);
template void stokes_apply_launch<float>(const stokes_geom &, const stokes_coefs<float> &, stokes_cvec<float>,
                                         stokes_vec<float>, const stokes_cvec<float> *, bool, cudaStream_t);

// ---------------------------------------------------------------------------
// Sums of squares per equation block and counts of equations: out[0..2] = sum F^2
// over x-momentum, z-momentum, continuity rows; out[3..5] = row counts.
template <typename T>
__global__ void k_residual_norms(int nu, int nv, int np, const T *__restrict__ fu, const T *__restrict__ fv,
                                 const T *__restrict__ fp, const signed char *__restrict__ tu,
                                 const signed char *__restrict__ tv, const signed char *__restrict__ tp,
                                 double *part, unsigned int *counter, double *out) {
    double acc[6] = {0, 0, 0, 0, 0, 0};
    int n = nu > nv ? nu : nv;
    n = n > np ? n : np;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (i < nu && tu[i] == -1) { double f = fu[i]; acc[0] += f * f; acc[3] += 1; }
        if (i < nv && tv[i] == -1) { double f = fv[i]; acc[1] += f * f; acc[4] += 1; }
        if (i < np && tp[i] == -1) { double f = fp[i]; acc[2] += f * f; acc[5] += 1; }
    }
    mdz_grid_sum<6, double>(acc, part, counter, out);   // fixed order: the same bits every run
}

template <typename T>
mdz_status stokes_norms_launch(mdz_ctx *ctx, stokes_cvec<T> f, double *d_out6, cudaStream_t st) {
    const mdz_dgrid &g = ctx->g;
    int nu = g.Nx * (g.Nz + 1), nv = (g.Nx + 1) * g.Nz, np = g.ncx * g.ncz;
    int n = nu > nv ? nu : nv;
    int blocks = mdz_blocks(n, 256);
    if (blocks > 152 * 8) blocks = 152 * 8;
    k_residual_norms<T><<<blocks, 256, 0, st>>>(nu, nv, np, f.u, f.v, f.p, g.BCu, g.BCv, g.BCp,
                                                ctx->red_part + MDZ_RP_NORMS, ctx->red_cnt + MDZ_RC_NORMS, d_out6);
    MDZ_LAUNCHED(ctx);
    return MDZ_OK;
}
template mdz_status stokes_norms_launch<double>(mdz_ctx *, stokes_cvec<double>, double *, cudaStream_t);
template mdz_status stokes_norms_launch<float>(mdz_ctx *, stokes_cvec<float>, double *, cudaStream_t);

// ---------------------------------------------------------------------------
// Host drop-ins.
static bool supported_bcs(const mdz_ctx *ctx) {
    // inner (-1), Dirichlet on the boundary (0) and free-slip ghosts (13) only
    const mdz_grid_desc &d = ctx->host_desc;
    size_t nu = (size_t)d.Nx * (d.Nz + 1), nv = (size_t)(d.Nx + 1) * d.Nz, np = (size_t)(d.Nx - 1) * (d.Nz - 1);
    for (size_t i = 0; i < nu; i++) if (d.BCu_type[i] != -1 && d.BCu_type[i] != 0 && d.BCu_type[i] != 13) return false;
    for (size_t i = 0; i < nv; i++) if (d.BCv_type[i] != -1 && d.BCv_type[i] != 0 && d.BCv_type[i] != 13) return false;
    for (size_t i = 0; i < np; i++) if (d.BCp_type[i] != -1) return false;
    for (size_t i = 0; i < (size_t)d.Nx * d.Nz; i++) if (d.BCg_type[i] == 30) return false;
    // equations only on inner nodes: boundary rows/columns must not be -1
    for (int l = 0; l <= d.Nz; l++)
        for (int k = 0; k < d.Nx; k++) {
            bool inner = k > 0 && k < d.Nx - 1 && l > 0 && l < d.Nz;
            if (d.BCu_type[k + l * d.Nx] == -1 && !inner) return false;
        }
    for (int l = 0; l < d.Nz; l++)
        for (int k = 0; k <= d.Nx; k++) {
            bool inner = k > 0 && k < d.Nx && l > 0 && l < d.Nz - 1;
            if (d.BCv_type[k + l * (d.Nx + 1)] == -1 && !inner) return false;
        }
    return true;
}

mdz_status mdz_check_stokes_bcs(mdz_ctx *ctx) {
    if (!ctx->bcs_checked) {
        ctx->bcs_ok = supported_bcs(ctx);
        ctx->bcs_checked = true;
    }
    if (!ctx->bcs_ok)
        return mdz_fail(ctx, MDZ_ERR_UNSUPPORTED,
                        "Stokes: only inner equations with Dirichlet (0) / free-slip (13) boundaries are implemented");
    return MDZ_OK;
}

stokes_coefs<double> mdz_coefs64(const mdz_fields &f) {
    return stokes_coefs<double>{f.D11_n, f.D12_n, f.D13_n, f.D14_n, f.D21_n, f.D22_n, f.D23_n, f.D24_n,
                                f.D31_s, f.D32_s, f.D33_s, f.D34_s};
}

mdz_status mdz_dev_residual(mdz_ctx *ctx, const mdz_fields &f, double *d_norms6, cudaStream_t st) {
    stokes_geom G = mdz_stokes_geom(ctx);
    stokes_cvec<double> x{f.u, f.v, f.p_corr}, b{f.roger_x, f.roger_z, f.rhs_p};
    stokes_vec<double> y{f.ru, f.rv, f.rp};
    stokes_apply_launch<double>(G, mdz_coefs64(f), x, y, &b, false, st);
    MDZ_LAUNCHED(ctx);
    if (d_norms6) return stokes_norms_launch<double>(ctx, stokes_cvec<double>{f.ru, f.rv, f.rp}, d_norms6, st);
    return MDZ_OK;
}

extern "C" mdz_status mdz_EvaluateStokesResidualDecoupled(mdz_ctx *ctx, mdz_fields *f, double *norms3) {
    if (!ctx || !f) return ctx ? mdz_fail(ctx, MDZ_ERR_ARG, "EvaluateStokesResidualDecoupled: null") : MDZ_ERR_ARG;
    mdz_status s = mdz_check_stokes_bcs(ctx);
    if (s != MDZ_OK) return s;
    if ((s = mdz_ensure_fields(ctx)) != MDZ_OK) return s;
    cudaStream_t st = ctx->stream;
    if ((s = mdz_upload_fields(ctx, f, st)) != MDZ_OK) return s;
    double *dn = (double *)(ctx->d_counters + 8);
    if ((s = mdz_dev_residual(ctx, ctx->d, dn, st)) != MDZ_OK) return s;
    double h[6];
    MDZ_CUDA(ctx, cudaMemcpyAsync(h, dn, sizeof h, cudaMemcpyDeviceToHost, st));
    static const char *const names[] = {"ru", "rv", "rp"};
    if ((s = mdz_download_fields(ctx, f, names, 3, st)) != MDZ_OK) return s;
    if (norms3) {
        for (int q = 0; q < 3; q++) norms3[q] = sqrt(h[q] / (h[q + 3] > 0 ? h[q + 3] : 1.0));
    }
    if (!std::isfinite(h[0]) || !std::isfinite(h[1]) || !std::isfinite(h[2]))
        return mdz_fail(ctx, MDZ_ERR_NAN, "EvaluateStokesResidualDecoupled: NaN residual");
    return MDZ_OK;
}

extern "C" mdz_status mdz_StokesOperatorApply(mdz_ctx *ctx, mdz_fields *f, int jacobian, const double *xu,
                                              const double *xv, const double *xp, double *yu, double *yv,
                                              double *yp) {
    if (!ctx || !f || !xu || !xv || !xp || !yu || !yv || !yp)
        return ctx ? mdz_fail(ctx, MDZ_ERR_ARG, "StokesOperatorApply: null") : MDZ_ERR_ARG;
    mdz_status s = mdz_check_stokes_bcs(ctx);
    if (s != MDZ_OK) return s;
    if ((s = mdz_ensure_fields(ctx)) != MDZ_OK) return s;
    cudaStream_t st = ctx->stream;
    if ((s = mdz_upload_fields(ctx, f, st)) != MDZ_OK) return s;
    const mdz_dgrid &g = ctx->g;
    size_t nu = (size_t)g.Nx * (g.Nz + 1), nv = (size_t)(g.Nx + 1) * g.Nz, np = (size_t)g.ncx * g.ncz;
    double *buf = (double *)mdz_stage(ctx, 6, sizeof(double) * 2 * (nu + nv + np));
    if (!buf) return mdz_fail(ctx, MDZ_ERR_CUDA, "StokesOperatorApply: staging allocation failed");
    double *dxu = buf, *dxv = dxu + nu, *dxp = dxv + nv, *dyu = dxp + np, *dyv = dyu + nu, *dyp = dyv + nv;
    MDZ_CUDA(ctx, cudaMemcpyAsync(dxu, xu, nu * 8, cudaMemcpyHostToDevice, st));
    MDZ_CUDA(ctx, cudaMemcpyAsync(dxv, xv, nv * 8, cudaMemcpyHostToDevice, st));
    MDZ_CUDA(ctx, cudaMemcpyAsync(dxp, xp, np * 8, cudaMemcpyHostToDevice, st));
    stokes_apply_launch<double>(mdz_stokes_geom(ctx), mdz_coefs64(ctx->d), stokes_cvec<double>{dxu, dxv, dxp},
                                stokes_vec<double>{dyu, dyv, dyp}, nullptr, jacobian != 0, st);
    MDZ_LAUNCHED(ctx);
    MDZ_CUDA(ctx, cudaMemcpyAsync(yu, dyu, nu * 8, cudaMemcpyDeviceToHost, st));
    MDZ_CUDA(ctx, cudaMemcpyAsync(yv, dyv, nv * 8, cudaMemcpyDeviceToHost, st));
    MDZ_CUDA(ctx, cudaMemcpyAsync(yp, dyp, np * 8, cudaMemcpyDeviceToHost, st));
    MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    return MDZ_OK;
}
