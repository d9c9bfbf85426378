// Learned initial guess for the local rheology: placeholder until the MLP
// kernels are in; the time step refuses learned_guess = 1 without weights.
#include "mlp.cuh"

bool mdz_mlp_ready(const mdz_ctx *ctx) { (void)ctx; return false; }

mdz_status mdz_dev_viscosity_learned(mdz_ctx *ctx, const mdz_materials *m, const mdz_rheo_params *prm,
                                     const mdz_fields &f, int *d_counters, cudaStream_t st) {
    (void)m; (void)prm; (void)f; (void)d_counters; (void)st;
    return mdz_fail(ctx, MDZ_ERR_STATE, "learned guess: no MLP weights loaded");
}
