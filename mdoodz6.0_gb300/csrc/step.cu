// One time step of the reference's main loop on the resident state
// (SOURCE/Main_DOODZ.c:459-1320), restricted to the mechanical hot path:
//   1. marker->grid projections (P2Mastah calls of Main_DOODZ.c:501-594) as two
//      batched gathers (centroids, vertices), plus the grid properties of
//      ShearModCompExpGrid / CohesionFrictionDilationGrid
//      (SOURCE/RheologyDensity.c:1422-1791);
//   2. the non-linear loop (Main_DOODZ.c:733-940): UpdateNonLinearity, residual
//      and convergence test, Jacobian, defect solve, LineSearchDecoupled
//      (SOURCE/StokesRoutines.c:396-626) and ExtractSolutions2 (:187-234);
//   3. final rheology update with p = p_corr (Main_DOODZ.c:950-951);
//   4. marker updates: UpdateParticleStress without rotation and subgrid
//      diffusion (SOURCE/RheologyParticles.c:1124-1447), AccumulatedStrainII
//      (:191-537) and RogerGuntherII (SOURCE/AdvectionRoutines.c:569-628).
#include <cmath>
#include <cstdio>
#include <cstring>
#include "stokes.cuh"
#include "solver.cuh"
#include "mlp.cuh"

// ---------------------------------------------------------------------------
// Grid properties from phase fractions (one thread per node).
// centroid = 1: writes mu_n, bet_n, rho_n, d0_n, C_n, fric_n, dil_n
// centroid = 0: writes mu_s, bet_s, rho_s, C_s, fric_s, dil_s
__device__ __forceinline__ void softened(const mdz_materials &m, int p, double strain, int law, double &fric,
                                         double &dil, double &C) {
    fric = m.phi[p];
    dil = m.psi[p];
    C = m.C[p];
    double ds = m.pls_end[p] - m.pls_start[p];
    if (law == 0) {   // smooth law (RheologyDensity.c:1466-1488)
        double mu = 0.5 * (m.pls_end[p] + m.pls_start[p]);
        if (m.phi_soft[p] == 1) {
            double d = m.phi[p] - m.phi_end[p];
            double f = m.phi[p] - d / 2.0 * erfc(-(strain - mu) / ds) - m.phi_end[p];
            double f0 = m.phi[p] - d / 2.0 * erfc(-(0.0 - mu) / ds) - m.phi_end[p];
            fric = f * d / f0 + m.phi_end[p];
        }
        if (m.psi_soft[p] == 1) {
            double d = m.psi[p] - m.psi_end[p];
            double f = m.psi[p] - d / 2.0 * erfc(-(strain - mu) / ds) - m.psi_end[p];
            double f0 = m.psi[p] - d / 2.0 * erfc(-(0.0 - mu) / ds) - m.psi_end[p];
            dil = f * d / f0 + m.psi_end[p];
        }
        if (m.coh_soft[p] == 1) {
            double d = m.C[p] - m.C_end[p];
            double f = m.C[p] - d / 2.0 * erfc(-(strain - mu) / ds) - m.C_end[p];
            double f0 = m.C[p] - d / 2.0 * erfc(-(0.0 - mu) / ds) - m.C_end[p];
            C = f * d / f0 + m.C_end[p];
        }
    } else {          // linear law (RheologyDensity.c:1490-1512)
        if (strain >= m.pls_end[p]) {
            if (m.phi_soft[p] == 1) fric = m.phi_end[p];
            if (m.psi_soft[p] == 1) dil = m.psi_end[p];
            if (m.coh_soft[p] == 1) C = m.C_end[p];
        } else if (strain >= m.pls_start[p]) {
            if (m.phi_soft[p] == 1) fric = m.phi[p] + (m.phi_end[p] - m.phi[p]) / ds * strain;
            if (m.psi_soft[p] == 1) dil = m.psi[p] + (m.psi_end[p] - m.psi[p]) / ds * strain;
            if (m.coh_soft[p] == 1) C = m.C[p] + (m.C_end[p] - m.C[p]) / ds * strain;
        }
    }
}

__global__ void k_grid_props(int n, int nph, mdz_materials m, int law, const signed char *__restrict__ tag, int air31,
                             const double *__restrict__ pp, const double *__restrict__ strain,
                             const double *__restrict__ cmul, double *__restrict__ mu, double *__restrict__ bet,
                             double *__restrict__ rho, double *__restrict__ d0, double *__restrict__ C,
                             double *__restrict__ fric, double *__restrict__ dil) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    double imu = 0, ibet = 0, r = 0, d = 0, Cs = 0, fs = 0, ds = 0;
    bool active = tag[c] != 30 && !(air31 && tag[c] == 31);
    if (active) {
        for (int p = 0; p < nph; p++) {
            double w = pp[(size_t)p * n + c];
            imu += w / m.mu[p];
            ibet += w / m.bet[p];
            r += w * m.rho[p];
            d += w * m.gs_ref[p];
            double f_, di_, C_;
            softened(m, p, strain[c], law, f_, di_, C_);
            fs += w * f_;
            ds += w * di_;
            Cs += w * C_;
        }
        imu = 1.0 / imu;
        ibet = 1.0 / ibet;
        if (cmul) Cs *= cmul[c];
    }
    mu[c] = imu; bet[c] = ibet; rho[c] = r;
    if (d0) d0[c] = d;
    C[c] = Cs; fric[c] = fs; dil[c] = ds;
}

// Dirichlet values on boundary nodes and free-slip ghost mirrors (ApplyBC,
// SOURCE/StokesRoutines.c:51-135) for u and v.
__global__ void k_apply_bc(mdz_dgrid g, double *__restrict__ u, double *__restrict__ v) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int Nx = g.Nx, Nz = g.Nz;
    if (i < Nx * (Nz + 1)) {
        signed char t = g.BCu[i];
        if (t == 0) u[i] = g.BCu_val[i];
    }
    if (i < (Nx + 1) * Nz) {
        signed char t = g.BCv[i];
        if (t == 0) v[i] = g.BCv_val[i];
    }
}

__global__ void k_mirror_ghosts(mdz_dgrid g, double *__restrict__ u, double *__restrict__ v) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int Nx = g.Nx, Nz = g.Nz, nxvz = Nx + 1;
    if (i < Nx) {
        if (g.BCu[i] == 13) u[i] = u[i + Nx];
        int top = i + Nz * Nx;
        if (g.BCu[top] == 13) u[top] = u[top - Nx];
    }
    if (i < Nz) {
        int w = i * nxvz, e = i * nxvz + Nx;
        if (g.BCv[w] == 13) v[w] = v[w + 1];
        if (g.BCv[e] == 13) v[e] = v[e - 1];
    }
}

// x = x0 + alpha * dx on the equations (ExtractSolutions2)
__global__ void k_trial(mdz_dgrid g, const double *__restrict__ u0, const double *__restrict__ v0,
                        const double *__restrict__ p0, const double *__restrict__ dx, double alpha,
                        double *__restrict__ u, double *__restrict__ v, double *__restrict__ p) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int nu = g.Nx * (g.Nz + 1), nv = (g.Nx + 1) * g.Nz, np = g.ncx * g.ncz;
    if (i < nu) u[i] = g.BCu[i] == -1 ? u0[i] + alpha * dx[i] : u0[i];
    if (i < nv) v[i] = g.BCv[i] == -1 ? v0[i] + alpha * dx[nu + i] : v0[i];
    if (i < np) p[i] = g.BCp[i] == -1 ? p0[i] + alpha * dx[nu + nv + i] : p0[i];
}

__global__ void k_copy3(int nu, int nv, int np, const double *__restrict__ a, const double *__restrict__ b,
                        const double *__restrict__ c, double *__restrict__ A, double *__restrict__ B,
                        double *__restrict__ Cc) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nu) A[i] = a[i];
    if (i < nv) B[i] = b[i];
    if (i < np) Cc[i] = c[i];
}

// stress increments on the grid (UpdateParticleStress, no-subgrid branch :1397-1420)
// and strain increments (AccumulatedStrainII :205-219)
// and the pressure increment of UpdateParticlePressure (RheologyParticles.c:
// 1004-1030, Plith_trick = 0: p_in - p0_n where the tag is not 30)
__global__ void k_increments(mdz_dgrid g, double dt, mdz_fields f, double *__restrict__ dsxx,
                             double *__restrict__ dszz, double *__restrict__ dsxz, double *__restrict__ dstrain,
                             double *__restrict__ dstrain_pl, double *__restrict__ dp) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int nc = g.ncx * g.ncz, nv = g.Nx * g.Nz;
    if (i < nc) {
        bool act = g.BCp[i] != 30 && g.BCp[i] != 31;
        dp[i] = g.BCp[i] != 30 ? f.p[i] - f.p0_n[i] : 0.0;
        dsxx[i] = act ? f.sxxd[i] - f.sxxd0[i] : 0.0;
        dszz[i] = act ? f.szzd[i] - f.szzd0[i] : 0.0;
        dstrain[i] = dt * (f.eII_pl[i] + f.eII_pwl[i] + f.eII_lin[i] + f.eII_el[i] + f.eII_cst[i]);
        dstrain_pl[i] = dt * f.eII_pl[i];
    }
    if (i < nv) dsxz[i] = g.BCg[i] != 30 ? f.sxz[i] - f.sxz0[i] : 0.0;
}

__device__ __forceinline__ bool is_air(signed char t) { return t == 30 || t == 31; }

// Marker updates: stress += G2P(increments) (centroids in the ghosted frame,
// shear on vertices), strain(_pl) += AccumulatedStrainII interpolation.
__global__ void k_marker_update(int n, mdz_dgrid g, const double *__restrict__ mx, const double *__restrict__ mz,
                                const int *__restrict__ mph, const double *__restrict__ dsxx,
                                const double *__restrict__ dszz, const double *__restrict__ dsxz,
                                const double *__restrict__ dstrain, const double *__restrict__ dstrain_pl,
                                const double *__restrict__ dp, double *__restrict__ sxx, double *__restrict__ szz,
                                double *__restrict__ sxz, double *__restrict__ strain, double *__restrict__ strain_pl,
                                double *__restrict__ P, int what) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n || mph[k] == -1) return;
    const double x = mx[k], z = mz[k], dx = g.dx, dz = g.dz, idx = g.idx, idz = g.idz;
    const int ncx = g.ncx, ncz = g.ncz, Nx = g.Nx, Nz = g.Nz;
    // what & 1: stress increments (UpdateParticleStress, before the advection);
    // what & 2: strain increments (AccumulatedStrainII, after it, at the
    // advected positions; markers that left the box are skipped);
    // what & 4: pressure increment (UpdateParticlePressure, before the advection)
    // centroids, ghosted frame (Interp_Grid2P_centroids2, non-periodic)
    if (what & 5) {
        int jp = (int)ceil_quot(x - g.xvz[0], dx, idx, 0.0) - 1, ip = (int)ceil_quot(z - g.zvx[0], dz, idz, 0.0) - 1;
        int jw = jp - 1, je = jp, is = ip - 1, in_ = ip;
        if (jp <= 0) { jw = 0; je = 0; }
        if (jp >= ncx) { jw = ncx - 1; je = ncx - 1; }
        if (ip <= 0) { is = 0; in_ = 0; }
        if (ip >= ncz) { is = ncz - 1; in_ = ncz - 1; }
        int jx = jp < 0 ? 0 : (jp > ncx ? ncx : jp), iz = ip < 0 ? 0 : (ip > ncz ? ncz : ip);
        double dxm = x - g.xvz[jx], dzm = z - g.zvx[iz];
        int SW = jw + is * ncx, SE = je + is * ncx, NW = jw + in_ * ncx, NE = je + in_ * ncx;
        const double wx = dxm * idx, wz = dzm * idz;
        double wSW = (1.0 - wx) * (1.0 - wz), wSE = wx * (1.0 - wz);
        double wNW = (1.0 - wx) * wz, wNE = wx * wz;
        const signed char *t = g.BCp;
        int sSW = is_air(t[SW]) ? NW : SW, sSE = is_air(t[SE]) ? NE : SE;
        int sNW = is_air(t[NW]) ? SW : NW, sNE = is_air(t[NE]) ? SE : NE;
        if (what & 1) {
            sxx[k] += wSW * dsxx[sSW] + wSE * dsxx[sSE] + wNW * dsxx[sNW] + wNE * dsxx[sNE];
            szz[k] += wSW * dszz[sSW] + wSE * dszz[sSE] + wNW * dszz[sNW] + wNE * dszz[sNE];
        }
        if (what & 4) P[k] += wSW * dp[sSW] + wSE * dp[sSE] + wNW * dp[sNW] + wNE * dp[sNE];
    }
    // vertices (Interp_Grid2P)
    if (what & 1) {
        int jp = (int)ceil_quot(x - g.xg[0], dx, idx, 0.0) - 1, ip = (int)ceil_quot(z - g.zg[0], dz, idz, 0.0) - 1;
        jp = jp < 0 ? 0 : (jp > Nx - 2 ? Nx - 2 : jp);
        ip = ip < 0 ? 0 : (ip > Nz - 2 ? Nz - 2 : ip);
        double dxm = fabs(x - g.xg[jp]), dzm = fabs(z - g.zg[ip]);
        int SW = jp + ip * Nx, SE = SW + 1, NW = jp + (ip + 1) * Nx, NE = NW + 1;
        const signed char *t = g.BCg;
        double v = 0.0;
        const double wx = dxm * idx, wz = dzm * idz;
        v += (1.0 - wx) * (1.0 - wz) * dsxz[is_air(t[SW]) ? NW : SW];
        v += wx * (1.0 - wz) * dsxz[is_air(t[SE]) ? NE : SE];
        v += (1.0 - wx) * wz * dsxz[is_air(t[NW]) ? SW : NW];
        v += wx * wz * dsxz[is_air(t[NE]) ? SE : NE];
        sxz[k] += v;
    }
    // strain increments on centroid lines (AccumulatedStrainII :235-350)
    if (what & 2) {
        int jp = (int)ceil_quot(x - g.xc[0], dx, idx, 0.0) - 1, ip = (int)ceil_quot(z - g.zc[0], dz, idz, 0.0) - 1;
        jp = jp < 0 ? 0 : (jp > ncx - 2 ? ncx - 2 : jp);
        ip = ip < 0 ? 0 : (ip > ncz - 2 ? ncz - 2 : ip);
        double dxm = x - g.xc[jp], dzm = z - g.zc[ip];
        int SW = jp + ip * ncx, SE = SW + 1, NW = jp + (ip + 1) * ncx, NE = NW + 1;
        const signed char *t = g.BCp;
        double e = 0, ep = 0, s = 0, w;
        const double wx = dxm * idx, wz = dzm * idz;
        if (!is_air(t[SW])) { w = (1.0 - wx) * (1.0 - wz); e += w * dstrain[SW]; ep += w * dstrain_pl[SW]; s += w; }
        if (!is_air(t[SE])) { w = wx * (1.0 - wz); e += w * dstrain[SE]; ep += w * dstrain_pl[SE]; s += w; }
        if (!is_air(t[NW])) { w = (1.0 - wx) * wz; e += w * dstrain[NW]; ep += w * dstrain_pl[NW]; s += w; }
        if (!is_air(t[NE])) { w = wx * wz; e += w * dstrain[NE]; ep += w * dstrain_pl[NE]; s += w; }
        if (s > 1e-13) { e /= s; ep /= s; }
        strain[k] += e;
        strain_pl[k] += ep;
    }
}

// ---------------------------------------------------------------------------
struct step_timer {
    cudaEvent_t a, b;
    cudaStream_t st;
    bool on;
    double *acc;
    step_timer(cudaStream_t s, double *acc_) : st(s), on(acc_ != nullptr), acc(acc_) {
        if (on) { cudaEventCreate(&a); cudaEventCreate(&b); cudaEventRecord(a, st); }
    }
    ~step_timer() {
        if (on) {
            cudaEventRecord(b, st);
            cudaEventSynchronize(b);
            float ms = 0;
            cudaEventElapsedTime(&ms, a, b);
            *acc += ms;
            cudaEventDestroy(a);
            cudaEventDestroy(b);
        }
    }
};

// Local rheology + RHS + Picard operators of the current state (UpdateNonLinearity).
// labels: whether an FP64 evaluation of this time step recorded its converged
// local solves (learned_guess = 1 then starts the next one from them instead
// of the MLP: the phase fractions are those of the step's projection).
static mdz_status update_nonlinearity(mdz_ctx *ctx, const mdz_materials *mat, const mdz_model *M,
                                      bool &labels, cudaStream_t st, bool fp32 = false) {
    mdz_fields &f = ctx->d;
    mdz_status s;
    if ((s = mdz_dev_strain_rates(ctx, f, st)) != MDZ_OK) return s;
    if (fp32) {
        if ((s = mdz_dev_viscosity(ctx, mat, &M->rheo, f, ctx->d_counters, st, false, true)) != MDZ_OK) return s;
    } else if (M->learned_guess) {
        const int warm = M->learned_guess == 1 ? (labels ? 2 : 1) : 0;
        if ((s = mdz_dev_viscosity_learned(ctx, mat, &M->rheo, f, ctx->d_counters, st, warm)) != MDZ_OK) return s;
        labels = warm >= 1;
    } else {
        if ((s = mdz_dev_viscosity(ctx, mat, &M->rheo, f, ctx->d_counters, st)) != MDZ_OK) return s;
    }
    if ((s = mdz_dev_rhs(ctx, &M->rheo, M->gx, M->gz, f, st)) != MDZ_OK) return s;
    if ((s = mdz_dev_operators(ctx, &M->rheo, f, 0, st)) != MDZ_OK) return s;
    return MDZ_OK;
}

static mdz_status residual_norms(mdz_ctx *ctx, double *norms3, cudaStream_t st) {
    double *dn = (double *)(ctx->d_counters + 8);
    mdz_status s = mdz_dev_residual(ctx, ctx->d, dn, st);
    if (s != MDZ_OK) return s;
    double h[6];
    MDZ_CUDA(ctx, cudaMemcpyAsync(h, dn, sizeof h, cudaMemcpyDeviceToHost, st));
    MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    for (int q = 0; q < 3; q++) norms3[q] = sqrt(h[q] / (h[q + 3] > 0 ? h[q + 3] : 1.0));
    if (!std::isfinite(norms3[0]) || !std::isfinite(norms3[1]) || !std::isfinite(norms3[2]))
        return mdz_fail(ctx, MDZ_ERR_NAN, "time step: NaN residual");
    return MDZ_OK;
}

// Main_DOODZ.c:830: each block converged in absolute or relative terms; a
// block whose first residual is exactly zero (e.g. continuity of a
// divergence-free initial guess) is measured against the largest first residual.
// Each block converges on its absolute or relative tolerance; a block whose
// first residual is negligible next to the largest one (an initially
// divergence-free velocity makes resp0 round-off) is measured against that one.
// the largest block residual relative to its first value, with the block
// selection of converged(): the distance still to go to rel_tol
static double relative_residual(const double *r, const double *r0) {
    double rmax = fmax(r0[0], fmax(r0[1], r0[2])), out = 0.0;
    for (int q = 0; q < 3; q++) {
        double ref = r0[q] > 1e-6 * rmax ? r0[q] : rmax;
        if (ref > 0) out = fmax(out, r[q] / ref);
    }
    return out;
}

static bool converged(const mdz_model *M, const double *r, const double *r0) {
    double rmax = fmax(r0[0], fmax(r0[1], r0[2]));
    for (int q = 0; q < 3; q++) {
        double ref = r0[q] > 1e-6 * rmax ? r0[q] : rmax;
        bool ok = r[q] < M->abs_tol || (ref > 0 && r[q] / ref < M->rel_tol);
        if (!ok) return false;
    }
    return true;
}

struct step_buffers {
    double *F = nullptr, *dx = nullptr, *u0 = nullptr, *v0 = nullptr, *p0 = nullptr;
    double *cmul_n = nullptr, *cmul_s = nullptr;
    double *dsxx = nullptr, *dszz = nullptr, *dsxz = nullptr, *dstr = nullptr, *dstr_pl = nullptr, *dp = nullptr;
};

static mdz_status step_buffers_get(mdz_ctx *ctx, step_buffers &B) {
    const mdz_dgrid &g = ctx->g;
    size_t nu = (size_t)g.Nx * (g.Nz + 1), nv = (size_t)(g.Nx + 1) * g.Nz, np = (size_t)g.ncx * g.ncz;
    size_t ng = (size_t)g.Nx * g.Nz, n = nu + nv + np;
    size_t total = 2 * n + nu + nv + np + np + ng + 3 * np + ng + np + np;
    double *b = (double *)mdz_stage(ctx, 5, sizeof(double) * total);
    if (!b) return mdz_fail(ctx, MDZ_ERR_CUDA, "time step: workspace allocation failed");
    B.F = b; b += n;
    B.dx = b; b += n;
    B.u0 = b; b += nu;
    B.v0 = b; b += nv;
    B.p0 = b; b += np;
    B.cmul_n = b; b += np;
    B.cmul_s = b; b += ng;
    B.dsxx = b; b += np;
    B.dszz = b; b += np;
    B.dstr = b; b += np;
    B.dsxz = b; b += ng;
    B.dstr_pl = b; b += np;
    B.dp = b; b += np;
    return MDZ_OK;
}

mdz_status mdz_dev_time_step(mdz_ctx *ctx, const mdz_materials *mat, const mdz_model *M, mdz_step_report *rep,
                             cudaStream_t st) {
    mdz_status s;
    mdz_step_report R{};
    bool labels = false;
    const mdz_dgrid &g = ctx->g;
    mdz_fields &f = ctx->d;
    const int nu = g.Nx * (g.Nz + 1), nv = (g.Nx + 1) * g.Nz, np = g.ncx * g.ncz, nvert = g.Nx * g.Nz;
    const int nmax = (g.Nx + 1) * (g.Nz + 1);
    step_buffers B;
    if ((s = step_buffers_get(ctx, B)) != MDZ_OK) return s;
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    cudaEventRecord(t0, st);
    // ---- 1. projections ------------------------------------------------------
    // Active nodes that receive no marker weight (cells emptied by the flow when
    // reseeding is off) would get zero phase fractions, a zero viscosity and a
    // NaN later in the Krylov solve; the phase-fraction projections count them
    // and the step refuses such a state here.
    int *d_empty = ctx->d_counters + 3;
    MDZ_CUDA(ctx, cudaMemsetAsync(d_empty, 0, sizeof(int), st));
    ctx->p2g_empty = d_empty;
    {
        step_timer T(st, &R.ms_projection);
        // centroids: old stresses, T, plastic strain, cohesion multiplier and the
        // markers' pressure (p0_n, Main_DOODZ.c:593)
        const double *cv[6] = {ctx->m.attr[MDZ_M_SXXD], ctx->m.attr[MDZ_M_SZZD], ctx->m.attr[MDZ_M_T],
                               ctx->m.attr[MDZ_M_STRAIN_PL], ctx->m.attr[MDZ_M_CMUL], ctx->m.attr[MDZ_M_P]};
        double *co[6] = {f.sxxd0, f.szzd0, f.T, f.strain_n, B.cmul_n, f.p0_n};
        int avg[6] = {0, 0, 0, 0, 0, 0};
        if ((s = mdz_dev_p2g(ctx, 6, cv, avg, co, f.phase_perc_n, MDZ_NODES_CENTROIDS, M->itp_stencil, st)) != MDZ_OK)
            return s;
        // vertices: the softening reads the plastic strain as Interp_P2N gives it
        // (RheologyDensity.c:1545, the one-cell stencil whatever itp_stencil),
        // and the cohesion multiplier travels with it
        const double *vv[3] = {ctx->m.attr[MDZ_M_SXZ], ctx->m.attr[MDZ_M_STRAIN_PL], ctx->m.attr[MDZ_M_CMUL]};
        double *vo[3] = {f.sxz0, f.strain_s, B.cmul_s};
        const int nv1 = M->itp_stencil == 1 ? 3 : 1;
        if ((s = mdz_dev_p2g(ctx, nv1, vv, avg, vo, f.phase_perc_s, MDZ_NODES_VERTICES, M->itp_stencil, st)) != MDZ_OK)
            return s;
        if (nv1 == 1 && (s = mdz_dev_p2g(ctx, 2, vv + 1, avg, vo + 1, nullptr, MDZ_NODES_VERTICES, 1, st)) != MDZ_OK)
            return s;
        if ((s = mdz_dev_c2v(ctx, f.sxxd0, f.sxxd0_s, st)) != MDZ_OK) return s;
        if ((s = mdz_dev_c2v(ctx, f.szzd0, f.szzd0_s, st)) != MDZ_OK) return s;
        if ((s = mdz_dev_v2c(ctx, f.sxz0_n, f.sxz0, st)) != MDZ_OK) return s;
        k_grid_props<<<mdz_blocks(np), MDZ_THREADS, 0, st>>>(np, mat->n_phases, *mat, M->softening, g.BCp, 1,
                                                             f.phase_perc_n, f.strain_n, B.cmul_n, f.mu_n, f.bet_n,
                                                             f.rho_n, f.d0_n, f.C_n, f.fric_n, f.dil_n);
        MDZ_LAUNCHED(ctx);
        k_grid_props<<<mdz_blocks(nvert), MDZ_THREADS, 0, st>>>(nvert, mat->n_phases, *mat, M->softening, g.BCg, 0,
                                                                f.phase_perc_s, f.strain_s, B.cmul_s, f.mu_s,
                                                                f.bet_s, f.rho_s, nullptr, f.C_s, f.fric_s, f.dil_s);
        MDZ_LAUNCHED(ctx);
        k_apply_bc<<<mdz_blocks(nmax), MDZ_THREADS, 0, st>>>(g, f.u, f.v);
        MDZ_LAUNCHED(ctx);
        k_mirror_ghosts<<<mdz_blocks(g.Nx > g.Nz ? g.Nx : g.Nz), MDZ_THREADS, 0, st>>>(g, f.u, f.v);
        MDZ_LAUNCHED(ctx);
    }
    ctx->p2g_empty = nullptr;
    {
        int empty = 0;
        MDZ_CUDA(ctx, cudaMemcpyAsync(&empty, d_empty, sizeof(int), cudaMemcpyDeviceToHost, st));
        MDZ_CUDA(ctx, cudaStreamSynchronize(st));
        if (empty > 0)
            return mdz_fail(ctx, MDZ_ERR_STATE,
                            "time step: %d active centroids/vertices received no marker weight (emptied cells: "
                            "enable reseeding, mdz_model.reseed = 1)", empty);
    }
    // ---- 2. non-linear iterations -----------------------------------------------
    double r0[3] = {0, 0, 0}, r[3] = {0, 0, 0};
    int nit = 0;
    bool use_newton = M->newton && !M->picard2newton;
    double rel_prev = -1.0, eta_prev = 0.1;   // forcing-term history (adaptive_lin_tol)
    MDZ_CUDA(ctx, cudaMemsetAsync(ctx->d_counters, 0, sizeof(int) * 4, st));
    MDZ_CUDA(ctx, cudaMemsetAsync(ctx->d_counters + 48, 0, sizeof(unsigned long long), st));
    for (nit = 0; nit <= M->nit_max; nit++) {
        // inexact FP32 rheology in the first iterations (fp32_rheology_its)
        bool fp32 = nit < M->fp32_rheology_its;
        {
            step_timer T(st, &R.ms_rheology);
            if ((s = update_nonlinearity(ctx, mat, M, labels, st, fp32)) != MDZ_OK) return s;
        }
        {
            step_timer T(st, &R.ms_residual);
            if ((s = residual_norms(ctx, r, st)) != MDZ_OK) return s;
        }
        if (nit == 0) memcpy(r0, r, sizeof r0);
        bool conv = converged(M, r, r0) && (nit > 0 || (r[0] < M->abs_tol && r[1] < M->abs_tol && r[2] < M->abs_tol));
        if (conv && fp32) {   // convergence is only decided on an FP64 evaluation
            {
                step_timer T(st, &R.ms_rheology);
                if ((s = update_nonlinearity(ctx, mat, M, labels, st, false)) != MDZ_OK) return s;
            }
            {
                step_timer T(st, &R.ms_residual);
                if ((s = residual_norms(ctx, r, st)) != MDZ_OK) return s;
            }
            conv = converged(M, r, r0);
        }
        if (nit < MDZ_HISTORY) memcpy(R.res_history[nit], r, sizeof r);
        if (conv) {
            R.converged = 1;
            break;
        }
        if (nit == M->nit_max) break;
        // Picard -> Newton switch (Main_DOODZ.c:735-743)
        if (M->newton && !use_newton && nit > 0 &&
            (r[0] < M->pic2newt_cond * r0[0] || r[1] < M->pic2newt_cond * r0[1] || nit >= M->nit_pic_max))
            use_newton = true;
        // defect F (grid layout) and the linear operator
        k_copy3<<<mdz_blocks(nmax), MDZ_THREADS, 0, st>>>(nu, nv, np, f.ru, f.rv, f.rp, B.F, B.F + nu, B.F + nu + nv);
        MDZ_LAUNCHED(ctx);
        if (use_newton) {
            if ((s = mdz_dev_operators(ctx, &M->rheo, f, 1, st)) != MDZ_OK) return s;
        }
        mdz_solve_stats ss{};
        bool newton_step = use_newton;
        // tolerance of this defect solve: lin_rtol, or the Eisenstat-Walker
        // forcing term (choice 2, gamma 0.9, alpha 2, with its safeguard) kept
        // within [lin_rtol, 0.1] and no tighter than half the way to rel_tol
        double eta = M->lin_rtol;
        const bool reuse_mg = M->mg_reuse_below > 0.0 && nit > 0 && relative_residual(r, r0) < M->mg_reuse_below;
        if (M->adaptive_lin_tol) {
            const double rel = relative_residual(r, r0);
            double e = rel_prev > 0.0 ? 0.9 * (rel / rel_prev) * (rel / rel_prev) : 0.1;
            if (rel_prev > 0.0 && 0.9 * eta_prev * eta_prev > 0.1) e = fmax(e, 0.9 * eta_prev * eta_prev);
            e = fmin(e, 0.1);
            if (rel > 0.0) e = fmax(e, 0.5 * M->rel_tol / rel);
            e = fmin(e, 0.1);
            eta = fmax(e, M->lin_rtol);
            rel_prev = rel;
            eta_prev = eta;
        }
        {
            step_timer T(st, &R.ms_solve);
            const int maxit = use_newton && M->newton_maxit > 0 ? M->newton_maxit : M->lin_maxit;
            s = mdz_dev_solve(ctx, f, use_newton, M->precision, eta, maxit, B.F, B.dx, &ss, st, reuse_mg);
            if (s != MDZ_OK) return s;
            R.linear_its += ss.iterations;
            R.newton_its += use_newton ? 1 : 0;
            // an FP32-refined solve that stopped short of the tolerance (its
            // refinement stagnates where FP32 cannot resolve the correction) is
            // redone in FP64, so a missed digit never reaches the Newton update;
            // one that did not even halve the defect always is
            if (M->precision == 32 && !(ss.rel_residual <= fmin(10.0 * eta, 0.5))) {
                s = mdz_dev_solve(ctx, f, use_newton, 64, eta, maxit, B.F, B.dx, &ss, st);
                if (s != MDZ_OK) return s;
                R.linear_its += ss.iterations;
                R.precision_fallbacks++;
            }
            // A Newton system whose pressure Schur complement the Picard-based
            // preconditioner cannot follow (strong pressure-dependent plasticity)
            // stalls the Krylov solve: take a Picard step for this iteration.
            if (use_newton && !(ss.rel_residual <= fmax(1e-2, 2.0 * eta))) {
                if ((s = mdz_dev_operators(ctx, &M->rheo, f, 0, st)) != MDZ_OK) return s;
                s = mdz_dev_solve(ctx, f, false, M->precision, eta, M->lin_maxit, B.F, B.dx, &ss, st);
                if (s != MDZ_OK) return s;
                R.linear_its += ss.iterations;
                R.picard_fallbacks++;
                R.newton_its--;
                newton_step = false;
            }
            if (nit < MDZ_HISTORY) {
                R.lin_its_history[nit] = ss.iterations;
                R.lin_rel_history[nit] = ss.rel_residual;
                R.newton_history[nit] = newton_step ? 1 : 0;
            }
        }
        // line search / update
        k_copy3<<<mdz_blocks(nmax), MDZ_THREADS, 0, st>>>(nu, nv, np, f.u, f.v, f.p, B.u0, B.v0, B.p0);
        MDZ_LAUNCHED(ctx);
        double alpha = -1.0;
        if (M->line_search) {
            step_timer T(st, &R.ms_line_search);
            const int ntry = 6;
            double amin = newton_step ? -1.0 : -2.5, amax = newton_step ? -M->line_search_min : -0.0;
            double da = fabs(amax - amin) / (ntry - 1), a = amax;
            double best = 1e300, rx[6], rz[6], rp[6], av[6];
            int ibest = 0;
            for (int kk = 0; kk < ntry; kk++) {
                if (kk > 0) a -= da;
                av[kk] = a;
                k_trial<<<mdz_blocks(nmax), MDZ_THREADS, 0, st>>>(g, B.u0, B.v0, B.p0, B.dx, a, f.u, f.v, f.p);
                MDZ_LAUNCHED(ctx);
                k_mirror_ghosts<<<mdz_blocks(g.Nx > g.Nz ? g.Nx : g.Nz), MDZ_THREADS, 0, st>>>(g, f.u, f.v);
                MDZ_LAUNCHED(ctx);
                if ((s = update_nonlinearity(ctx, mat, M, labels, st)) != MDZ_OK) return s;
                double t[3];
                if ((s = residual_norms(ctx, t, st)) != MDZ_OK) return s;
                rx[kk] = t[0]; rz[kk] = t[1]; rp[kk] = t[2];
                double fxzp = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
                if (fxzp < best) { best = fxzp; ibest = kk; }
            }
            double f0 = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
            bool ok = best < f0;
            if (!ok) {   // the reference's fall-backs on the x/z residuals
                int ixz = 0, ix = 0, iz = 0;
                for (int kk = 1; kk < ntry; kk++) {
                    if (sqrt(rx[kk] * rx[kk] + rz[kk] * rz[kk]) < sqrt(rx[ixz] * rx[ixz] + rz[ixz] * rz[ixz])) ixz = kk;
                    if (rx[kk] < rx[ix]) ix = kk;
                    if (rz[kk] < rz[iz]) iz = kk;
                }
                if (rx[ixz] < r[0] && rz[ixz] < r[1]) { ok = true; ibest = ixz; }
                else if (rx[ix] < r[0]) { ok = true; ibest = ix; }
                else if (rz[iz] < r[1]) { ok = true; ibest = iz; }
            }
            (void)rp;
            if (!ok || fabs(av[ibest]) < 1e-13) {
                R.stagnated = 1;
                alpha = 0.0;
            } else {
                alpha = av[ibest];
            }
        }
        k_trial<<<mdz_blocks(nmax), MDZ_THREADS, 0, st>>>(g, B.u0, B.v0, B.p0, B.dx, alpha, f.u, f.v, f.p);
        MDZ_LAUNCHED(ctx);
        k_mirror_ghosts<<<mdz_blocks(g.Nx > g.Nz ? g.Nx : g.Nz), MDZ_THREADS, 0, st>>>(g, f.u, f.v);
        MDZ_LAUNCHED(ctx);
        if (R.stagnated) { nit++; break; }
    }
    R.nonlinear_its = nit;
    memcpy(R.res0, r0, sizeof r0);
    memcpy(R.res, r, sizeof r);
    // ---- 3. final rheology update, p <- p_corr ----------------------------------
    {
        step_timer T(st, &R.ms_rheology);
        if ((s = update_nonlinearity(ctx, mat, M, labels, st)) != MDZ_OK) return s;
        MDZ_CUDA(ctx, cudaMemcpyAsync(f.p, f.p_corr, sizeof(double) * np, cudaMemcpyDeviceToDevice, st));
    }
    // ---- 4. markers ---------------------------------------------------------------
    if (M->advect) {
        step_timer T(st, &R.ms_markers);
        int nn = np > nvert ? np : nvert;
        k_increments<<<mdz_blocks(nn), MDZ_THREADS, 0, st>>>(g, M->rheo.dt, f, B.dsxx, B.dszz, B.dsxz, B.dstr,
                                                            B.dstr_pl, B.dp);
        MDZ_LAUNCHED(ctx);
        int n = ctx->m.n;
        if (n > 0) {
            // UpdateParticleStress and UpdateParticlePressure (Main_DOODZ.c:1010-1013)
            k_marker_update<<<mdz_blocks(n), MDZ_THREADS, 0, st>>>(
                n, g, ctx->m.x, ctx->m.z, ctx->m.phase, B.dsxx, B.dszz, B.dsxz, B.dstr, B.dstr_pl, B.dp,
                ctx->m.attr[MDZ_M_SXXD], ctx->m.attr[MDZ_M_SZZD], ctx->m.attr[MDZ_M_SXZ], ctx->m.attr[MDZ_M_STRAIN],
                ctx->m.attr[MDZ_M_STRAIN_PL], ctx->m.attr[MDZ_M_P], 1 | 4);
            MDZ_LAUNCHED(ctx);
        }
        // PureShearALE before the marker advection (Main_DOODZ.c:1107-1109): the
        // markers then move through the velocities on the new grid lines
        if (M->ispureshear_ale == 1)
            if ((s = mdz_dev_pure_shear_ale(ctx, f.u, f.v, M->rheo.dt, st)) != MDZ_OK) return s;
        if ((s = mdz_dev_rk4(ctx, f.u, f.v, M->rheo.dt, st)) != MDZ_OK) return s;
        // AccumulatedStrainII after the advection (Main_DOODZ.c:1134-1140)
        if (n > 0) {
            k_marker_update<<<mdz_blocks(n), MDZ_THREADS, 0, st>>>(
                n, g, ctx->m.x, ctx->m.z, ctx->m.phase, B.dsxx, B.dszz, B.dsxz, B.dstr, B.dstr_pl, B.dp,
                ctx->m.attr[MDZ_M_SXXD], ctx->m.attr[MDZ_M_SZZD], ctx->m.attr[MDZ_M_SXZ], ctx->m.attr[MDZ_M_STRAIN],
                ctx->m.attr[MDZ_M_STRAIN_PL], nullptr, 2);
            MDZ_LAUNCHED(ctx);
        }
        // reseeding after the advection (Main_DOODZ.c:1233-1236)
        if (M->reseed)
            if ((s = mdz_dev_reseed(ctx, M->min_part_cell, M->direct_neighbour, f.T, f.sxxd, f.szzd, f.sxz, f.p, st,
                                    &R.markers_added)) != MDZ_OK)
                return s;
    }
    cudaEventRecord(t1, st);
    MDZ_CUDA(ctx, cudaEventSynchronize(t1));
    float ms = 0;
    cudaEventElapsedTime(&ms, t0, t1);
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    R.ms_total = ms;
    int cnt[4];
    MDZ_CUDA(ctx, cudaMemcpy(cnt, ctx->d_counters, sizeof cnt, cudaMemcpyDeviceToHost));
    R.local_failures = cnt[0];
    R.local_fallbacks = cnt[1];
    R.local_solves = cnt[2];
    unsigned long long li = 0;
    MDZ_CUDA(ctx, cudaMemcpy(&li, ctx->d_counters + 48, sizeof li, cudaMemcpyDeviceToHost));
    R.local_iterations = (long long)li;
    R.xmin = ctx->host_desc.xmin; R.xmax = ctx->host_desc.xmax;
    R.zmin = ctx->host_desc.zmin; R.zmax = ctx->host_desc.zmax;
    if (rep) *rep = R;
    return MDZ_OK;
}

extern "C" mdz_status mdz_time_step(mdz_ctx *ctx, const mdz_materials *mat, const mdz_model *model,
                                    mdz_step_report *rep) {
    if (!ctx || !mat || !model) return ctx ? mdz_fail(ctx, MDZ_ERR_ARG, "mdz_time_step: null argument") : MDZ_ERR_ARG;
    mdz_status s = mdz_check_materials(ctx, mat);
    if (s != MDZ_OK) return s;
    if (model->precision != 64 && model->precision != 32)
        return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_time_step: precision must be 64 or 32");
    if (model->itp_stencil != 1 && model->itp_stencil != 9)
        return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_time_step: itp_stencil must be 1 or 9");
    if (model->rheo.dt <= 0) return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_time_step: dt must be > 0");
    if (model->ispureshear_ale != 0 && model->ispureshear_ale != 1)
        return mdz_fail(ctx, MDZ_ERR_ARG, "mdz_time_step: ispureshear_ale must be 0 or 1");
    if (model->learned_guess && !mdz_mlp_ready(ctx))
        return mdz_fail(ctx, MDZ_ERR_STATE, "mdz_time_step: learned guess requested but no MLP weights loaded");
    if ((s = mdz_ensure_fields(ctx)) != MDZ_OK) return s;
    if ((s = mdz_solver_ensure(ctx)) != MDZ_OK) return s;
    if ((s = mdz_ensure_bins(ctx, ctx->stream)) != MDZ_OK) return s;
    s = mdz_dev_time_step(ctx, mat, model, rep, ctx->stream);
    ctx->p2g_empty = nullptr;
    ctx->bins.valid = false;
    return s;
}

// ShearModCompExpGrid (SOURCE/RheologyDensity.c:1666-1791): harmonic shear
// modulus and compressibility at centroids and vertices from the phase
// fractions f->phase_perc_n / phase_perc_s (host); writes f->mu_n, mu_s,
// bet_n, bet_s.  Air nodes (tag 30, and 31 at centroids) get 0.
// CohesionFrictionDilationGrid (:1422-1665): the resident markers' plastic
// strain projected to the centroids (P2Mastah with itp_stencil) and to the
// vertices (Interp_P2N: nearest vertex, one-cell tent), the smooth softening
// law per phase, arithmetic phase average; writes f->C_n, C_s, fric_n, fric_s,
// dil_n, dil_s (and strain_n, strain_s).  Both run on the device mirrors and
// copy the outputs back (synchronous).
static mdz_status grid_props_host(mdz_ctx *ctx, const mdz_materials *mat, int itp_stencil, mdz_fields *h,
                                  bool cohesion) {
    if (!ctx || !mat || !h || !h->phase_perc_n || !h->phase_perc_s)
        return ctx ? mdz_fail(ctx, MDZ_ERR_ARG, "grid properties: null argument") : MDZ_ERR_ARG;
    mdz_status s = mdz_check_materials(ctx, mat);
    if (s != MDZ_OK) return s;
    if (itp_stencil != 1 && itp_stencil != 9)
        return mdz_fail(ctx, MDZ_ERR_ARG, "CohesionFrictionDilationGrid: itp_stencil must be 1 or 9");
    if ((s = mdz_ensure_fields(ctx)) != MDZ_OK) return s;
    const mdz_dgrid &g = ctx->g;
    mdz_fields &f = ctx->d;
    cudaStream_t st = ctx->stream;
    const int np = g.ncx * g.ncz, nvert = g.Nx * g.Nz, nph = mat->n_phases;
    MDZ_CUDA(ctx, cudaMemcpyAsync(f.phase_perc_n, h->phase_perc_n, sizeof(double) * np * nph, cudaMemcpyHostToDevice,
                                  st));
    MDZ_CUDA(ctx, cudaMemcpyAsync(f.phase_perc_s, h->phase_perc_s, sizeof(double) * nvert * nph,
                                  cudaMemcpyHostToDevice, st));
    if (cohesion) {
        const double *val[1] = {ctx->m.attr[MDZ_M_STRAIN_PL]};
        int avg[1] = {0};
        double *on[1] = {f.strain_n}, *os[1] = {f.strain_s};
        if ((s = mdz_dev_p2g(ctx, 1, val, avg, on, nullptr, MDZ_NODES_CENTROIDS, itp_stencil, st)) != MDZ_OK) return s;
        if ((s = mdz_dev_p2g(ctx, 1, val, avg, os, nullptr, MDZ_NODES_VERTICES, 1, st)) != MDZ_OK) return s;
    }
    k_grid_props<<<mdz_blocks(np), MDZ_THREADS, 0, st>>>(np, nph, *mat, 0, g.BCp, 1, f.phase_perc_n, f.strain_n,
                                                         nullptr, f.mu_n, f.bet_n, f.rho_n, f.d0_n, f.C_n, f.fric_n,
                                                         f.dil_n);
    MDZ_LAUNCHED(ctx);
    k_grid_props<<<mdz_blocks(nvert), MDZ_THREADS, 0, st>>>(nvert, nph, *mat, 0, g.BCg, 0, f.phase_perc_s,
                                                            f.strain_s, nullptr, f.mu_s, f.bet_s, f.rho_s, nullptr,
                                                            f.C_s, f.fric_s, f.dil_s);
    MDZ_LAUNCHED(ctx);
    if (cohesion) {
        static const char *const names[] = {"C_n", "C_s", "fric_n", "fric_s", "dil_n", "dil_s", "strain_n", "strain_s"};
        return mdz_download_fields(ctx, h, names, 8, st);
    }
    static const char *const names[] = {"mu_n", "mu_s", "bet_n", "bet_s"};
    return mdz_download_fields(ctx, h, names, 4, st);
}

// Host drop-ins of the marker updates on the resident markers: the grid
// fields named are uploaded from h, the increments formed on the device and
// interpolated to the markers (what: 1 stresses, 2 strains, 4 pressure).
static mdz_status marker_update_host(mdz_ctx *ctx, mdz_fields *h, const char *const *need, int nneed, int what,
                                     double dt) {
    mdz_status s = mdz_ensure_fields(ctx);
    if (s != MDZ_OK) return s;
    mdz_fields up{};   // upload exactly the fields this update reads
    for (int i = 0; i < nneed; i++) {
#define PICK(name, kind)                                                                         \
        if (!strcmp(need[i], #name)) {                                                          \
            if (!h->name) return mdz_fail(ctx, MDZ_ERR_ARG, "marker update: needs %s", #name);  \
            up.name = h->name;                                                                  \
        }
        MDZ_FIELD_LIST(PICK)
#undef PICK
    }
    cudaStream_t st = ctx->stream;
    if ((s = mdz_upload_fields(ctx, &up, st)) != MDZ_OK) return s;
    const mdz_dgrid &g = ctx->g;
    const int np = g.ncx * g.ncz, nvert = g.Nx * g.Nz, nn = np > nvert ? np : nvert;
    step_buffers B;
    if ((s = step_buffers_get(ctx, B)) != MDZ_OK) return s;
    k_increments<<<mdz_blocks(nn), MDZ_THREADS, 0, st>>>(g, dt, ctx->d, B.dsxx, B.dszz, B.dsxz, B.dstr, B.dstr_pl,
                                                          B.dp);
    MDZ_LAUNCHED(ctx);
    const int n = ctx->m.n;
    if (n > 0) {
        k_marker_update<<<mdz_blocks(n), MDZ_THREADS, 0, st>>>(
            n, g, ctx->m.x, ctx->m.z, ctx->m.phase, B.dsxx, B.dszz, B.dsxz, B.dstr, B.dstr_pl, B.dp,
            ctx->m.attr[MDZ_M_SXXD], ctx->m.attr[MDZ_M_SZZD], ctx->m.attr[MDZ_M_SXZ], ctx->m.attr[MDZ_M_STRAIN],
            ctx->m.attr[MDZ_M_STRAIN_PL], ctx->m.attr[MDZ_M_P], what);
        MDZ_LAUNCHED(ctx);
    }
    MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    return MDZ_OK;
}

extern "C" mdz_status mdz_UpdateParticlePressure(mdz_ctx *ctx, mdz_fields *h) {
    if (!ctx || !h) return ctx ? mdz_fail(ctx, MDZ_ERR_ARG, "UpdateParticlePressure: null argument") : MDZ_ERR_ARG;
    static const char *const need[] = {"p", "p0_n"};
    return marker_update_host(ctx, h, need, 2, 4, 1.0);
}

extern "C" mdz_status mdz_UpdateParticleStress(mdz_ctx *ctx, mdz_fields *h) {
    if (!ctx || !h) return ctx ? mdz_fail(ctx, MDZ_ERR_ARG, "UpdateParticleStress: null argument") : MDZ_ERR_ARG;
    static const char *const need[] = {"sxxd", "szzd", "sxz", "sxxd0", "szzd0", "sxz0"};
    return marker_update_host(ctx, h, need, 6, 1, 1.0);
}

extern "C" mdz_status mdz_AccumulatedStrainII(mdz_ctx *ctx, mdz_fields *h, double dt) {
    if (!ctx || !h) return ctx ? mdz_fail(ctx, MDZ_ERR_ARG, "AccumulatedStrainII: null argument") : MDZ_ERR_ARG;
    static const char *const need[] = {"eII_pl", "eII_pwl", "eII_lin", "eII_el", "eII_cst"};
    return marker_update_host(ctx, h, need, 5, 2, dt);
}

extern "C" mdz_status mdz_ShearModCompExpGrid(mdz_ctx *ctx, const mdz_materials *mat, mdz_fields *f) {
    return grid_props_host(ctx, mat, 1, f, false);
}

extern "C" mdz_status mdz_CohesionFrictionDilationGrid(mdz_ctx *ctx, const mdz_materials *mat, int itp_stencil,
                                                       mdz_fields *f) {
    return grid_props_host(ctx, mat, itp_stencil, f, true);
}

extern "C" mdz_status mdz_sync_fields(mdz_ctx *ctx, mdz_fields *f, int to_device) {
    if (!ctx || !f) return ctx ? mdz_fail(ctx, MDZ_ERR_ARG, "mdz_sync_fields: null") : MDZ_ERR_ARG;
    mdz_status s = mdz_ensure_fields(ctx);
    if (s != MDZ_OK) return s;
    if (to_device) {
        if ((s = mdz_upload_fields(ctx, f, ctx->stream)) != MDZ_OK) return s;
        MDZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        return MDZ_OK;
    }
    static const char *const all[] = {
#define NAME(name, kind) #name,
        MDZ_FIELD_LIST(NAME)
#undef NAME
    };
    return mdz_download_fields(ctx, f, all, (int)(sizeof(all) / sizeof(all[0])), ctx->stream);
}

extern "C" mdz_status mdz_get_velocity(mdz_ctx *ctx, double *u, double *v, double *p) {
    if (!ctx) return MDZ_ERR_ARG;
    mdz_status s = mdz_ensure_fields(ctx);
    if (s != MDZ_OK) return s;
    const mdz_dgrid &g = ctx->g;
    cudaStream_t st = ctx->stream;
    if (u) MDZ_CUDA(ctx, cudaMemcpyAsync(u, ctx->d.u, sizeof(double) * g.Nx * (g.Nz + 1), cudaMemcpyDeviceToHost, st));
    if (v) MDZ_CUDA(ctx, cudaMemcpyAsync(v, ctx->d.v, sizeof(double) * (g.Nx + 1) * g.Nz, cudaMemcpyDeviceToHost, st));
    if (p) MDZ_CUDA(ctx, cudaMemcpyAsync(p, ctx->d.p, sizeof(double) * g.ncx * g.ncz, cudaMemcpyDeviceToHost, st));
    MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    return MDZ_OK;
}
