// Device mirrors of the grid fields and the host-pointer drop-ins for the
// grid-side reference functions (StrainRateComponents, NonNewtonianViscosityGrid,
// RheologicalOperators, EvaluateRHS).
#include <cstring>
#include "mdz_internal.cuh"
#include "mlp.cuh"

size_t mdz_field_count(const mdz_ctx *ctx, int kind) {
    const mdz_dgrid &g = ctx->g;
    switch (kind) {
        case MDZ_K_VX: return (size_t)g.Nx * (g.Nz + 1);
        case MDZ_K_VZ: return (size_t)(g.Nx + 1) * g.Nz;
        case MDZ_K_CEN: return (size_t)g.ncx * g.ncz;
        case MDZ_K_VER: return (size_t)g.Nx * g.Nz;
        case MDZ_K_PPN: return (size_t)g.ncx * g.ncz * ctx->n_phases;
        default: return (size_t)g.Nx * g.Nz * ctx->n_phases;
    }
}

mdz_status mdz_ensure_fields(mdz_ctx *ctx) {
    if (ctx->fields_ready) return MDZ_OK;
    mdz_fields &d = ctx->d;
#define ALLOC(name, kind)                                                                           \
    {                                                                                               \
        size_t n = mdz_field_count(ctx, MDZ_K_##kind);                                              \
        MDZ_CUDA(ctx, cudaMalloc((void **)&d.name, sizeof(double) * n));                            \
        MDZ_CUDA(ctx, cudaMemset(d.name, 0, sizeof(double) * n));                                   \
    }
    MDZ_FIELD_LIST(ALLOC)
#undef ALLOC
    MDZ_CUDA(ctx, cudaMalloc((void **)&ctx->d_counters, sizeof(int) * 64));
    MDZ_CUDA(ctx, cudaMemset(ctx->d_counters, 0, sizeof(int) * 64));
    ctx->fields_ready = true;
    return MDZ_OK;
}

void mdz_free_fields(mdz_ctx *ctx) {
    if (!ctx->fields_ready) return;
    mdz_fields &d = ctx->d;
#define FREE(name, kind) if (d.name) cudaFree(d.name);
    MDZ_FIELD_LIST(FREE)
#undef FREE
    if (ctx->d_counters) cudaFree(ctx->d_counters);
    ctx->fields_ready = false;
}

// Upload every non-null host field (the host drop-ins are synchronous and
// simple: they mirror the caller's whole grid state), or download a named set.
mdz_status mdz_upload_fields(mdz_ctx *ctx, const mdz_fields *h, cudaStream_t st) {
    mdz_fields &d = ctx->d;
#define UP(name, kind)                                                                                         \
    if (h->name)                                                                                               \
        MDZ_CUDA(ctx, cudaMemcpyAsync(d.name, h->name, sizeof(double) * mdz_field_count(ctx, MDZ_K_##kind),   \
                                      cudaMemcpyHostToDevice, st));
    MDZ_FIELD_LIST(UP)
#undef UP
    return MDZ_OK;
}

mdz_status mdz_download_fields(mdz_ctx *ctx, const mdz_fields *h, const char *const *names, int n, cudaStream_t st) {
    const mdz_fields &d = ctx->d;
    for (int i = 0; i < n; i++) {
#define DOWN(name, kind)                                                                                       \
    if (!strcmp(names[i], #name) && h->name)                                                                   \
        MDZ_CUDA(ctx, cudaMemcpyAsync(h->name, d.name, sizeof(double) * mdz_field_count(ctx, MDZ_K_##kind),   \
                                      cudaMemcpyDeviceToHost, st));
        MDZ_FIELD_LIST(DOWN)
#undef DOWN
    }
    MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    return MDZ_OK;
}

#define NAMES(...) static const char *const names[] = {__VA_ARGS__}; const int nnames = sizeof(names) / sizeof(names[0]);

extern "C" mdz_status mdz_StrainRateComponents(mdz_ctx *ctx, mdz_fields *f) {
    if (!ctx || !f || !f->u || !f->v) return ctx ? mdz_fail(ctx, MDZ_ERR_ARG, "StrainRateComponents: need u, v") : MDZ_ERR_ARG;
    mdz_status s = mdz_ensure_fields(ctx);
    if (s != MDZ_OK) return s;
    cudaStream_t st = ctx->stream;
    if ((s = mdz_upload_fields(ctx, f, st)) != MDZ_OK) return s;
    if ((s = mdz_dev_strain_rates(ctx, ctx->d, st)) != MDZ_OK) return s;
    NAMES("div_u", "exxd", "ezzd", "exz", "exz_n", "exxd_s", "ezzd_s");
    return mdz_download_fields(ctx, f, names, nnames, st);
}

static mdz_status viscosity_grid(mdz_ctx *ctx, const mdz_materials *m, const mdz_rheo_params *prm, mdz_fields *f,
                                 int learned, long long *stats) {
    if (!ctx || !m || !prm || !f) return ctx ? mdz_fail(ctx, MDZ_ERR_ARG, "NonNewtonianViscosityGrid: null argument") : MDZ_ERR_ARG;
    mdz_status s = mdz_check_materials(ctx, m);
    if (s != MDZ_OK) return s;
    if ((s = mdz_ensure_fields(ctx)) != MDZ_OK) return s;
    cudaStream_t st = ctx->stream;
    if ((s = mdz_upload_fields(ctx, f, st)) != MDZ_OK) return s;
    MDZ_CUDA(ctx, cudaMemsetAsync(ctx->d_counters, 0, sizeof(int) * 4, st));
    MDZ_CUDA(ctx, cudaMemsetAsync(ctx->d_counters + 48, 0, sizeof(unsigned long long), st));
    if (learned) {
        if ((s = mdz_dev_viscosity_learned(ctx, m, prm, ctx->d, ctx->d_counters, st)) != MDZ_OK) return s;
    } else {
        if ((s = mdz_dev_viscosity(ctx, m, prm, ctx->d, ctx->d_counters, st)) != MDZ_OK) return s;
    }
    int cnt[4] = {0, 0, 0, 0};
    unsigned long long its = 0;
    MDZ_CUDA(ctx, cudaMemcpyAsync(cnt, ctx->d_counters, sizeof cnt, cudaMemcpyDeviceToHost, st));
    MDZ_CUDA(ctx, cudaMemcpyAsync(&its, ctx->d_counters + 48, sizeof its, cudaMemcpyDeviceToHost, st));
    MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    if (stats) {
        stats[0] = cnt[0];
        stats[1] = cnt[1];
        stats[2] = cnt[2];
        stats[3] = (long long)its;
    }
    const int fails = cnt[0];
    NAMES("div_u_s", "T_s", "P_s", "d0_s", "phi0_s", "eta_n", "eta_s", "eta_phys_n", "eta_phys_s", "VE_n", "VE_s",
          "sxxd", "szzd", "sxz", "sxz_n", "eII_el", "eII_pl", "eII_pwl", "eII_lin", "eII_cst", "eII_exp", "eII_gbs",
          "d_n", "exx_el",
          "ezz_el", "exz_el", "exx_diss", "ezz_diss", "exz_diss", "detadexx_n", "detadezz_n", "detadgxz_n",
          "detadp_n", "ddivpdexx_n", "ddivpdezz_n", "ddivpdgxz_n", "ddivpdp_n", "detadexx_s", "detadezz_s",
          "detadgxz_s", "detadp_s", "p_corr", "div_u_el", "div_u_pl", "div_u_r", "Wtot", "Wel", "Wdiss", "X_n",
          "X_s", "OverS_n", "OverS_s");
    s = mdz_download_fields(ctx, f, names, nnames, st);
    (void)fails;
    return s;
}

extern "C" mdz_status mdz_NonNewtonianViscosityGrid(mdz_ctx *ctx, const mdz_materials *m, const mdz_rheo_params *prm,
                                                    mdz_fields *f, int *n_not_converged) {
    long long st4[4] = {0, 0, 0, 0};
    mdz_status s = viscosity_grid(ctx, m, prm, f, 0, st4);
    if (n_not_converged) *n_not_converged = (int)st4[0];
    return s;
}

extern "C" mdz_status mdz_NonNewtonianViscosityGrid_learned(mdz_ctx *ctx, const mdz_materials *m,
                                                            const mdz_rheo_params *prm, mdz_fields *f, int learned,
                                                            long long *stats) {
    return viscosity_grid(ctx, m, prm, f, learned, stats);
}

extern "C" mdz_status mdz_RheologicalOperators(mdz_ctx *ctx, const mdz_rheo_params *prm, mdz_fields *f, int jacobian) {
    if (!ctx || !prm || !f) return ctx ? mdz_fail(ctx, MDZ_ERR_ARG, "RheologicalOperators: null argument") : MDZ_ERR_ARG;
    mdz_status s = mdz_ensure_fields(ctx);
    if (s != MDZ_OK) return s;
    cudaStream_t st = ctx->stream;
    if ((s = mdz_upload_fields(ctx, f, st)) != MDZ_OK) return s;
    if ((s = mdz_dev_operators(ctx, prm, ctx->d, jacobian, st)) != MDZ_OK) return s;
    NAMES("D11_n", "D12_n", "D13_n", "D14_n", "D21_n", "D22_n", "D23_n", "D24_n", "D31_s", "D32_s", "D33_s", "D34_s");
    return mdz_download_fields(ctx, f, names, nnames, st);
}

extern "C" mdz_status mdz_EvaluateRHS(mdz_ctx *ctx, const mdz_rheo_params *prm, double gx, double gz, mdz_fields *f) {
    if (!ctx || !prm || !f) return ctx ? mdz_fail(ctx, MDZ_ERR_ARG, "EvaluateRHS: null argument") : MDZ_ERR_ARG;
    mdz_status s = mdz_ensure_fields(ctx);
    if (s != MDZ_OK) return s;
    cudaStream_t st = ctx->stream;
    if ((s = mdz_upload_fields(ctx, f, st)) != MDZ_OK) return s;
    if ((s = mdz_dev_rhs(ctx, prm, gx, gz, ctx->d, st)) != MDZ_OK) return s;
    NAMES("roger_x", "roger_z", "rhs_p", "gx", "gz");
    return mdz_download_fields(ctx, f, names, nnames, st);
}
