// Solver entry points shared with the time step.
#pragma once
#include "mdz_internal.cuh"

struct mdz_solve_stats {
    int iterations;      // Krylov iterations (summed over refinement cycles)
    int refinements;     // FP64 defect-correction cycles (1 for the plain form)
    double rel_residual; // final ||F - K dx|| / ||F|| in FP64
    int mg_levels;
};

mdz_status mdz_solver_ensure(mdz_ctx *ctx);
void mdz_solver_free(mdz_ctx *ctx);
int mdz_solver_levels(const mdz_ctx *ctx);
// K dx = F on device arrays (u | v | p contiguous grid layout).
// reuse_mg: keep the multigrid hierarchy of the previous solve of this
// precision (if it was built for the same operator) instead of rebuilding it
// from the current viscosities.
mdz_status mdz_dev_solve(mdz_ctx *ctx, const mdz_fields &f, bool newton, int precision, double rtol, int maxit,
                         const double *F, double *dx, mdz_solve_stats *stats, cudaStream_t st, bool reuse_mg = false);
