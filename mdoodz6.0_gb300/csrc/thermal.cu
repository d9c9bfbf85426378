// Energy equation: the implicit step of EnergyDirectSolve
// (SOURCE/ThermalRoutines.c:72-551) on the centroids, matrix-free.
//
// The reference assembles a five-point matrix (row per active centroid:
// rho Cv / dt plus the conductances k / h^2 of its faces, Dirichlet walls
// doubling the face conductance, the off-diagonals minus the conductances)
// and factorises it with CHOLMOD.  Here the same rows are applied on the fly
// (the diagonal and the right-hand side formed once per solve, exactly as the
// reference sums them) and the system, symmetric positive definite for the
// Cartesian case, is solved by conjugate gradients with the diagonal as
// preconditioner, in FP64, from the old temperature.  Every inner product is
// a deterministic grid sum (fixed order), so a solve takes the same
// iterations and gives the same bits on every run.
#include <cmath>
#include "mdz_internal.cuh"

mdz_status mdz_ensure_fields(mdz_ctx *ctx);
mdz_status mdz_upload_fields(mdz_ctx *ctx, const mdz_fields *h, cudaStream_t st);
mdz_status mdz_download_fields(mdz_ctx *ctx, const mdz_fields *h, const char *const *names, int n, cudaStream_t st);

#define ZEROC_K 273.15

namespace {

constexpr int EN_THREADS = 256;
constexpr int EN_MAX_BLOCKS = 2048;   // partial slots per reduced value

struct energy_bc_dev {
    const signed char *type, *typW, *typE, *typS, *typN;
    const double *valW, *valE, *valS, *valN;
    double ixx, izz;   // 1/dx/dx, 1/dz/dz as the reference forms them (host: no FP64 division per row)
};

__device__ __forceinline__ bool active(const energy_bc_dev &B, int c) { return B.type[c] != 30; }

// Diagonal and right-hand side (b + bbc) of centroid row c, in the
// reference's order of additions (:158-187, :196-330).
__global__ void k_energy_setup(mdz_dgrid g, mdz_fields f, energy_bc_dev B, double dt, double gz, int shear,
                               int adiab, double *__restrict__ diag, double *__restrict__ rhs) {
    const int ncx = g.ncx, ncz = g.ncz, nx = g.Nx, nxvz = g.Nx + 1;
    const int c2 = blockIdx.x * blockDim.x + threadIdx.x;
    if (c2 >= ncx * ncz) return;
    const int k = c2 % ncx, l = c2 / ncx;
    if (!active(B, c2)) { diag[c2] = 1.0; rhs[c2] = 0.0; return; }
    const double ixx = B.ixx, izz = B.izz;
    const double rhoCp = f.rho_n[c2] * f.Cv[c2], T = f.T[c2];
    double b = 1.0 * rhoCp * T / dt;
    b += 1.0 * f.Qr[c2];
    if (shear == 1) b += f.Wdiss[c2];
    if (adiab == 1) {
        const int c3 = k + l * nxvz;
        b += T * f.alp[c2] * 0.5 * (f.v[c3 + 1] + f.v[c3 + 1 + nxvz]) * gz * f.rho_n[c2];
    } else if (adiab == 2) {
        b += T * f.alp[c2] * (f.p[c2] - f.p0_n[c2]) / dt;
    }
    const int c1 = k + (l + 1) * nx, c3 = k + l * nxvz + 1;
    const double AW = f.kx[c1], AE = f.kx[c1 + 1], AS = f.kz[c3], AN = f.kz[c3 + nxvz];
    double val = 1.0 * rhoCp / dt, bbc = 0.0;
    if (l > 0 && active(B, c2 - ncx)) val += AS * izz;
    if (k > 0 && active(B, c2 - 1)) val += AW * ixx;
    if (k < ncx - 1 && active(B, c2 + 1)) val += AE * ixx;
    if (l < ncz - 1 && active(B, c2 + ncx)) val += AN * izz;
    if (l == 0 && B.typS[k] == 1) { val += 2.0 * AS * izz; bbc += 2.0 * AS * izz * B.valS[k]; }
    if (l == 0 && B.typS[k] == 2) bbc += -1.0 / g.dx * B.valS[k];
    if (k == 0 && B.typW[l] == 1) { val += 2.0 * AW * ixx; bbc += 2.0 * AW * ixx * B.valW[l]; }
    if (k == ncx - 1 && B.typE[l] == 1) { val += 2.0 * AE * ixx; bbc += 2.0 * AE * ixx * B.valE[l]; }
    if (l == ncz - 1 && B.typN[k] == 1) { val += 2.0 * AN * izz; bbc += 2.0 * AN * izz * B.valN[k]; }
    diag[c2] = val;
    rhs[c2] = b + 1.0 * bbc;
}

// y = A x on the active rows (0 elsewhere); optionally dot = x . y over them
__device__ __forceinline__ double energy_row(const mdz_dgrid &g, const mdz_fields &f, const energy_bc_dev &B,
                                             const double *diag, const double *x, int c2) {
    const int ncx = g.ncx, ncz = g.ncz, nx = g.Nx, nxvz = g.Nx + 1;
    const int k = c2 % ncx, l = c2 / ncx;
    const double ixx = B.ixx, izz = B.izz;
    const int c1 = k + (l + 1) * nx, c3 = k + l * nxvz + 1;
    double y = diag[c2] * x[c2];
    if (l > 0 && active(B, c2 - ncx)) y += -1.0 * f.kz[c3] * izz * x[c2 - ncx];
    if (k > 0 && active(B, c2 - 1)) y += -1.0 * f.kx[c1] * ixx * x[c2 - 1];
    if (k < ncx - 1 && active(B, c2 + 1)) y += -1.0 * f.kx[c1 + 1] * ixx * x[c2 + 1];
    if (l < ncz - 1 && active(B, c2 + ncx)) y += -1.0 * f.kz[c3 + nxvz] * izz * x[c2 + ncx];
    return y;
}

// r = b - A x, z = r / diag, p = z; sums: r.z, r.r, b.b
__global__ void k_energy_init(mdz_dgrid g, mdz_fields f, energy_bc_dev B, const double *__restrict__ diag,
                              const double *__restrict__ rhs, const double *__restrict__ x, double *__restrict__ r,
                              double *__restrict__ z, double *__restrict__ p, double *part, unsigned int *cnt,
                              double *out) {
    double acc[3] = {0, 0, 0};
    const int n = g.ncx * g.ncz;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        double rr = 0.0, zz = 0.0;
        if (active(B, c)) {
            rr = rhs[c] - energy_row(g, f, B, diag, x, c);
            zz = rr / diag[c];
            acc[0] += rr * zz; acc[1] += rr * rr; acc[2] += rhs[c] * rhs[c];
        }
        r[c] = rr; z[c] = zz; p[c] = zz;
    }
    mdz_grid_sum<3, double>(acc, part, cnt, out);
}

// q = A p; sum p.q
__global__ void k_energy_apply(mdz_dgrid g, mdz_fields f, energy_bc_dev B, const double *__restrict__ diag,
                               const double *__restrict__ p, double *__restrict__ q, double *part, unsigned int *cnt,
                               double *out) {
    double acc[1] = {0};
    const int n = g.ncx * g.ncz;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        double y = 0.0;
        if (active(B, c)) {
            y = energy_row(g, f, B, diag, p, c);
            acc[0] += p[c] * y;
        }
        q[c] = y;
    }
    mdz_grid_sum<1, double>(acc, part, cnt, out);
}

// x += alpha p, r -= alpha q, z = r / diag; sums r.z, r.r   (alpha = s[0] / s[1])
__global__ void k_energy_update(int n, const signed char *__restrict__ type, const double *__restrict__ diag,
                                const double *__restrict__ s, const double *__restrict__ pq,
                                const double *__restrict__ p, const double *__restrict__ q, double *__restrict__ x,
                                double *__restrict__ r, double *__restrict__ z, double *part, unsigned int *cnt,
                                double *out) {
    const double alpha = s[0] / pq[0];
    double acc[2] = {0, 0};
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        if (type[c] == 30) continue;
        x[c] += alpha * p[c];
        const double rr = r[c] - alpha * q[c], zz = rr / diag[c];
        r[c] = rr;
        z[c] = zz;
        acc[0] += rr * zz;
        acc[1] += rr * rr;
    }
    mdz_grid_sum<2, double>(acc, part, cnt, out);
}

// p = z + beta p   (beta = s_new[0] / s_old[0])
__global__ void k_energy_dir(int n, const double *__restrict__ s_new, const double *__restrict__ s_old,
                             const double *__restrict__ z, double *__restrict__ p) {
    const double beta = s_new[0] / s_old[0];
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) p[c] = z[c] + beta * p[c];
}

// T <- x, dT = x - T on active cells; air: dT = 0, T = 0 C; count T < 0
__global__ void k_energy_finish(int n, const signed char *__restrict__ type, const double *__restrict__ x,
                                double *__restrict__ T, double *__restrict__ dT, double t_air, int *neg) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    if (type[c] != 30) {
        dT[c] = 1.0 * (x[c] - T[c]);
        T[c] = T[c] + dT[c];
        if (T[c] < 0.0) atomicAdd(neg, 1);
    } else {
        dT[c] = 0.0;
        T[c] = t_air;
    }
}

}  // namespace

extern "C" mdz_status mdz_EnergyDirectSolve(mdz_ctx *ctx, mdz_fields *f, const mdz_thermal_bc *bc, double dt,
                                            double gz, int shear_heating, int adiab_heating, double scale_T,
                                            double rel_tol, int max_iterations, int *iterations,
                                            double *rel_residual) {
    if (!ctx || !f || !bc) return ctx ? mdz_fail(ctx, MDZ_ERR_ARG, "EnergyDirectSolve: null argument") : MDZ_ERR_ARG;
    if (!(dt > 0.0) || !(scale_T > 0.0))
        return mdz_fail(ctx, MDZ_ERR_ARG, "EnergyDirectSolve: dt and scale_T must be > 0");
    if (!bc->type || !bc->typW || !bc->typE || !bc->typS || !bc->typN || !bc->valW || !bc->valE || !bc->valS ||
        !bc->valN)
        return mdz_fail(ctx, MDZ_ERR_ARG, "EnergyDirectSolve: thermal boundary arrays missing");
    if (!f->T || !f->rho_n || !f->Cv || !f->Qr || !f->kx || !f->kz)
        return mdz_fail(ctx, MDZ_ERR_ARG, "EnergyDirectSolve: needs T, rho_n, Cv, Qr, kx, kz");
    if ((shear_heating == 1 && !f->Wdiss) || (adiab_heating == 1 && (!f->alp || !f->v)) ||
        (adiab_heating == 2 && (!f->alp || !f->p || !f->p0_n)))
        return mdz_fail(ctx, MDZ_ERR_ARG, "EnergyDirectSolve: heating terms need Wdiss / alp, v / alp, p, p0_n");
    const mdz_dgrid &g = ctx->g;
    const int ncx = g.ncx, ncz = g.ncz, n = ncx * ncz;
    for (int c = 0; c < n; c++)
        if (bc->type[c] != -1 && bc->type[c] != 30)
            return mdz_fail(ctx, MDZ_ERR_UNSUPPORTED,
                            "EnergyDirectSolve: centroid thermal tags other than -1 and 30 (free surface, periodic) "
                            "are not implemented");
    if (rel_tol <= 0.0) rel_tol = 1e-13;
    if (max_iterations <= 0) max_iterations = 10000;
    mdz_status s = mdz_ensure_fields(ctx);
    if (s != MDZ_OK) return s;
    cudaStream_t st = ctx->stream;
    if ((s = mdz_upload_fields(ctx, f, st)) != MDZ_OK) return s;
    // boundary arrays and work vectors in one staging buffer
    const size_t nb = (size_t)n + 2 * (ncx + ncz), nw = 2 * (size_t)(ncx + ncz);
    const size_t bytes = sizeof(double) * (7 * (size_t)n + nw + 8) + nb + 64;
    unsigned char *buf = (unsigned char *)mdz_stage(ctx, 8, bytes);
    if (!buf) return mdz_fail(ctx, MDZ_ERR_CUDA, "EnergyDirectSolve: staging allocation failed");
    double *diag = (double *)buf, *rhs = diag + n, *x = rhs + n, *r = x + n, *z = r + n, *p = z + n, *q = p + n;
    double *vals = q + n, *sc = vals + nw;   // sc: [0..2] init sums, [3] p.q, [4..5] update sums, [6] old r.z
    signed char *tags = (signed char *)(sc + 8);
    int *neg = (int *)(((uintptr_t)(tags + nb) + 15) & ~(uintptr_t)15);
    MDZ_CUDA(ctx, cudaMemcpyAsync(tags, bc->type, n, cudaMemcpyHostToDevice, st));
    MDZ_CUDA(ctx, cudaMemcpyAsync(tags + n, bc->typW, ncz, cudaMemcpyHostToDevice, st));
    MDZ_CUDA(ctx, cudaMemcpyAsync(tags + n + ncz, bc->typE, ncz, cudaMemcpyHostToDevice, st));
    MDZ_CUDA(ctx, cudaMemcpyAsync(tags + n + 2 * ncz, bc->typS, ncx, cudaMemcpyHostToDevice, st));
    MDZ_CUDA(ctx, cudaMemcpyAsync(tags + n + 2 * ncz + ncx, bc->typN, ncx, cudaMemcpyHostToDevice, st));
    MDZ_CUDA(ctx, cudaMemcpyAsync(vals, bc->valW, sizeof(double) * ncz, cudaMemcpyHostToDevice, st));
    MDZ_CUDA(ctx, cudaMemcpyAsync(vals + ncz, bc->valE, sizeof(double) * ncz, cudaMemcpyHostToDevice, st));
    MDZ_CUDA(ctx, cudaMemcpyAsync(vals + 2 * ncz, bc->valS, sizeof(double) * ncx, cudaMemcpyHostToDevice, st));
    MDZ_CUDA(ctx, cudaMemcpyAsync(vals + 2 * ncz + ncx, bc->valN, sizeof(double) * ncx, cudaMemcpyHostToDevice, st));
    MDZ_CUDA(ctx, cudaMemsetAsync(neg, 0, sizeof(int), st));
    energy_bc_dev B{tags, tags + n, tags + n + ncz, tags + n + 2 * ncz, tags + n + 2 * ncz + ncx,
                    vals, vals + ncz, vals + 2 * ncz, vals + 2 * ncz + ncx, 1.0 / g.dx / g.dx, 1.0 / g.dz / g.dz};
    const mdz_fields &d = ctx->d;
    k_energy_setup<<<mdz_blocks(n, EN_THREADS), EN_THREADS, 0, st>>>(g, d, B, dt, gz, shear_heating, adiab_heating,
                                                                      diag, rhs);
    MDZ_LAUNCHED(ctx);
    MDZ_CUDA(ctx, cudaMemcpyAsync(x, d.T, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));   // start: old T
    int blocks = mdz_blocks(n, EN_THREADS);
    if (blocks > EN_MAX_BLOCKS) blocks = EN_MAX_BLOCKS;
    double *part = ctx->red_part + MDZ_RP_ENERGY;
    unsigned int *cnt = ctx->red_cnt + MDZ_RC_ENERGY;
    k_energy_init<<<blocks, EN_THREADS, 0, st>>>(g, d, B, diag, rhs, x, r, z, p, part, cnt, sc);
    MDZ_LAUNCHED(ctx);
    double h[3];
    MDZ_CUDA(ctx, cudaMemcpyAsync(h, sc, sizeof h, cudaMemcpyDeviceToHost, st));
    MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    const double bnorm = std::sqrt(h[2]);
    double rel = bnorm > 0.0 ? std::sqrt(h[1]) / bnorm : 0.0;
    int it = 0;
    // sc[0]: r.z of the current iteration (the update kernel reads it as the
    // numerator of alpha), sc[4]: the new r.z; they swap roles through sc[6]
    while (rel > rel_tol && it < max_iterations) {
        k_energy_apply<<<blocks, EN_THREADS, 0, st>>>(g, d, B, diag, p, q, part + 0, cnt + 1, sc + 3);
        MDZ_LAUNCHED(ctx);
        k_energy_update<<<blocks, EN_THREADS, 0, st>>>(n, tags, diag, sc, sc + 3, p, q, x, r, z, part + 2048,
                                                        cnt + 2, sc + 4);
        MDZ_LAUNCHED(ctx);
        k_energy_dir<<<blocks, EN_THREADS, 0, st>>>(n, sc + 4, sc, z, p);
        MDZ_LAUNCHED(ctx);
        MDZ_CUDA(ctx, cudaMemcpyAsync(sc, sc + 4, sizeof(double), cudaMemcpyDeviceToDevice, st));
        double u[2];
        MDZ_CUDA(ctx, cudaMemcpyAsync(u, sc + 4, sizeof u, cudaMemcpyDeviceToHost, st));
        MDZ_CUDA(ctx, cudaStreamSynchronize(st));
        rel = bnorm > 0.0 ? std::sqrt(u[1]) / bnorm : 0.0;
        it++;
        if (!std::isfinite(rel)) return mdz_fail(ctx, MDZ_ERR_NAN, "EnergyDirectSolve: NaN residual");
    }
    if (iterations) *iterations = it;
    if (rel_residual) *rel_residual = rel;
    k_energy_finish<<<mdz_blocks(n), MDZ_THREADS, 0, st>>>(n, tags, x, d.T, d.dT, ZEROC_K / scale_T, neg);
    MDZ_LAUNCHED(ctx);
    static const char *const names[] = {"T", "dT"};
    if ((s = mdz_download_fields(ctx, f, names, 2, st)) != MDZ_OK) return s;
    int nneg = 0;
    MDZ_CUDA(ctx, cudaMemcpyAsync(&nneg, neg, sizeof(int), cudaMemcpyDeviceToHost, st));
    MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    if (rel > rel_tol)
        return mdz_fail(ctx, MDZ_ERR_NOT_CONVERGED, "EnergyDirectSolve: relative residual %.3e after %d iterations",
                        rel, it);
    if (nneg) return mdz_fail(ctx, MDZ_ERR_STATE, "EnergyDirectSolve: negative temperature in %d cells", nneg);
    return MDZ_OK;
}
