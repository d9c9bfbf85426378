// Declarations shared by the Stokes operator, the solver and the time step.
#pragma once
#include "mdz_internal.cuh"
#include "stokes_ops.cuh"

stokes_geom mdz_stokes_geom(const mdz_ctx *ctx);
stokes_coefs<double> mdz_coefs64(const mdz_fields &f);
mdz_status mdz_check_stokes_bcs(mdz_ctx *ctx);

template <typename T>
void stokes_apply_launch(const stokes_geom &G, const stokes_coefs<T> &D, stokes_cvec<T> x, stokes_vec<T> y,
                         const stokes_cvec<T> *b, bool newton, cudaStream_t st);
template <typename T>
mdz_status stokes_norms_launch(mdz_ctx *ctx, stokes_cvec<T> f, double *d_out6, cudaStream_t st);

// Picard residual of the current state (u, v, p_corr, D from RheologicalOperators(0)),
// written to ru, rv, rp; optional device norms (sum F^2 per block, row counts).
mdz_status mdz_dev_residual(mdz_ctx *ctx, const mdz_fields &f, double *d_norms6, cudaStream_t st);
