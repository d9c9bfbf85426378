// Learned initial guess for the local rheology (declarations).
#pragma once
#include "mdz_internal.cuh"

bool mdz_mlp_ready(const mdz_ctx *ctx);
// NonNewtonianViscosityGrid with the MLP supplying the starting eta_ve / gdot
// of each local Newton solve; counters: [0] failures, [1] fall-backs to the
// plain start, [2] learned solves.
mdz_status mdz_dev_viscosity_learned(mdz_ctx *ctx, const mdz_materials *m, const mdz_rheo_params *prm,
                                     const mdz_fields &f, int *d_counters, cudaStream_t st);
