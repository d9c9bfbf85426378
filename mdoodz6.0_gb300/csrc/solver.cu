// Linear solver for the decoupled Stokes correction  K dx = F  (K = Picard
// operator or Newton Jacobian, applied matrix-free): right-preconditioned,
// restarted GCR with classical Gram-Schmidt applied twice, FP64 dot products
// (warp-shuffle block reductions), and an upper block-triangular
// preconditioner [[A, B], [0, S]]:
//   S^-1 = eta_n / cell volume            (viscosity-scaled pressure mass)
//   A^-1 = one geometric-multigrid V-cycle on the velocity block (Picard,
//          or optionally the Newton Jacobian's): damped Jacobi smoothing,
//          cell-doubling coarsening, bilinear prolongation with R = P^T,
//          Galerkin coarse operators R A P as 31-point stencils, and an
//          explicit inverse (or a single-CTA Jacobi-PCG solve) on the
//          coarsest level.
// The same code runs in FP64 (plain form) and with FP32 storage and FP32
// stencil / V-cycle arithmetic (T = float) inside an FP64 defect-correction
// loop (iterative refinement); all inner products accumulate in FP64.
//
// This replaces the reference's CHOLMOD-preconditioned GCR with
// Powell-Hestenes iterations (KillerSolver, SOURCE/Solvers.c:2226-2755 and
// kspgcr, SOURCE/Solvers.c:100-228): same defect-correction equation, solved to
// a relative tolerance, without assembling a matrix.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>
#include <cooperative_groups.h>
#include "stokes.cuh"
#include "solver.cuh"

#define MG_MAX_LEVELS 16
#define MG_DENSE_MAX 256
#define MG_DENSE_SMEM (96 * 1024)   // [A | I] of the coarsest level in shared memory up to this size (n <= 78)
#define MG_NST 31        // stencil coefficients per velocity row (15 same-component + 16 cross)
#define MG_CENTER 7      // plane of the diagonal entry in both layouts
#define GCR_MAX_M 48

// ---------------------------------------------------------------------------
template <typename T>
struct mg_level {
    int Nx = 0, Nz = 0, ncx = 0, ncz = 0;
    double dx = 0, dz = 0;
    signed char *BCu = nullptr, *BCv = nullptr, *BCp = nullptr, *BCg = nullptr;
    bool own_tags = false;
    T *D11 = nullptr, *D33 = nullptr;           // level 0 (Picard): D11 = D22 = 2 eta_n; D33 = eta_s
    // 31-point stencils of the velocity block (MG_NST coefficient planes per
    // component, structure of arrays): level 0 probed from the re-discretised
    // operator, coarser levels the Galerkin product R A P of the level above.
    T *su = nullptr, *sv = nullptr;
    T *pz = nullptr;                            // level 0: zero pressure vector for Newton probes
    T *xu = nullptr, *xv = nullptr, *yu = nullptr, *yv = nullptr;
    T *fu = nullptr, *fv = nullptr, *ru = nullptr, *rv = nullptr;
    T *idu = nullptr, *idv = nullptr;
    T *cg[8] = {nullptr};                       // coarsest-level CG workspace
    // coarsest level with at most MG_DENSE_MAX unknowns: explicit inverse
    int ndense = 0;
    int *dmap = nullptr;                        // dense index -> u index, or nu + v index
    double *Awork = nullptr;                    // 2 ndense^2 FP64: [A | I] for Gauss-Jordan
    T *AinvT = nullptr;                         // inverse, column-major
    size_t nu() const { return (size_t)Nx * (Nz + 1); }
    size_t nv() const { return (size_t)(Nx + 1) * Nz; }
    stokes_geom geom() const { return make_geom(Nx, Nz, dx, dz, BCu, BCv, BCp, BCg); }
    stokes_coefs<T> coefs() const {
        return stokes_coefs<T>{D11, nullptr, nullptr, nullptr, nullptr, D11, nullptr, nullptr,
                               nullptr, nullptr, D33, nullptr};
    }
};

template <typename T>
struct gcr_space {
    size_t nu = 0, nv = 0, np = 0, n = 0;
    int m = 0;
    T *Z = nullptr, *W = nullptr;       // m basis vectors each (u, v, p contiguous)
    T *x = nullptr, *r = nullptr, *z = nullptr, *w = nullptr, *t = nullptr;
    T *pin = nullptr;                   // the preconditioner's input (graph-captured pointer)
    double *tri = nullptr;              // Gram-Schmidt triangle U (column q at q * GCR_MAX_M), then gamma
    const T **dA0 = nullptr, **dA1 = nullptr, **dA2 = nullptr;   // dot-product pointer tables (k_dots uses dA0)
    double *dots = nullptr;             // device scalars
    // FP32 copies of the operator (only used for T = float)
    T *Dc[12] = {nullptr};
};

template <typename T>
struct mg_hier {
    int nlev = 0;
    bool newton = false;          // level 0 is the probed Newton block (smoothed by its stencil)
    bool built = false;           // mg_setup has filled the levels at least once
    double *pmean = nullptr;      // preconditioner scratch: pressure sum and count
    mg_level<T> L[MG_MAX_LEVELS];
};

#define MDZ_PRE_SLOTS 8
struct mdz_solver {
    mg_hier<double> mg64;
    mg_hier<float> mg32;
    gcr_space<double> g64;
    gcr_space<float> g32;
    double *sc = nullptr;        // host-pinned scalars
    bool ready = false;
    int nu1 = 2, nu2 = 1;        // fewer sweeps, a few more Krylov iterations: faster overall at 1025x513
    double omega = 0.7;
    int check = 1;               // GCR iterations between host convergence checks (one read-back
                                 // each: cheaper at 1025x513 than the iterations a sparser check overshoots)
    int restart = 30;            // GCR basis size
    int mg_jacobian = 0;         // 1: multigrid on the Newton Jacobian's velocity block (else Picard)
    int schur = 0;               // pressure block of Newton solves: 0 eta_n / cell volume, 1 the Jacobian's
                                 // D11 / 2 (tangent viscosity) where positive
    int bottom_cs[2] = {1, 1};   // cluster size of the V-cycle bottom kernel ([0] FP64, [1] FP32)
    // preconditioner application captured as a CUDA graph, per precision
    // ([0] FP64, [1] FP32): one graph launch per Krylov iteration
    // [precision (0 FP64, 1 FP32) * 2 + newton hierarchy + 4 * tangent Schur]
    cudaGraphExec_t pre[MDZ_PRE_SLOTS] = {};
    long long pre_launches[MDZ_PRE_SLOTS] = {};
    const double *pre_eta[MDZ_PRE_SLOTS] = {};
    double pre_bytes[MDZ_PRE_SLOTS] = {};   // algorithmic bytes of one application
};

// ---------------------------------------------------------------------------
// Tag rule of the free-slip pure-shear box on any level (the fine level must
// follow it too): Vx Dirichlet on the W/E lines, free-slip ghosts on the S/N
// rows; Vz Dirichlet on the S/N lines, ghosts on W/E; everything else inner.
__global__ void k_level_tags(int Nx, int Nz, signed char *BCu, signed char *BCv, signed char *BCp, signed char *BCg) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int nu = Nx * (Nz + 1), nv = (Nx + 1) * Nz, np = (Nx - 1) * (Nz - 1), ng = Nx * Nz;
    if (i < nu) {
        int k = i % Nx, l = i / Nx;
        signed char t = -1;
        if (k == 0 || k == Nx - 1) t = 0;
        if (l == 0 || l == Nz) t = 13;
        BCu[i] = t;
    }
    if (i < nv) {
        int k = i % (Nx + 1), l = i / (Nx + 1);
        signed char t = -1;
        if (l == 0 || l == Nz - 1) t = 0;
        if (k == 0 || k == Nx) t = 13;
        BCv[i] = t;
    }
    if (i < np) BCp[i] = -1;
    if (i < ng) BCg[i] = -1;
}

static bool fine_tags_follow_rule(const mdz_grid_desc &d) {
    int Nx = d.Nx, Nz = d.Nz;
    for (int l = 0; l <= Nz; l++)
        for (int k = 0; k < Nx; k++) {
            signed char t = -1;
            if (k == 0 || k == Nx - 1) t = 0;
            if (l == 0 || l == Nz) t = 13;
            if (d.BCu_type[k + l * Nx] != t) return false;
        }
    for (int l = 0; l < Nz; l++)
        for (int k = 0; k <= Nx; k++) {
            signed char t = -1;
            if (l == 0 || l == Nz - 1) t = 0;
            if (k == 0 || k == Nx) t = 13;
            if (d.BCv_type[k + l * (Nx + 1)] != t) return false;
        }
    return true;
}

// ---------------------------------------------------------------------------
// Multigrid kernels (velocity block, Picard, homogeneous boundaries).
template <typename T>
__global__ void k_mg_diag(stokes_geom G, const T *__restrict__ D11, const T *__restrict__ D33, T *__restrict__ idu,
                          T *__restrict__ idv) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int Nx = G.Nx, Nz = G.Nz, ncx = G.ncx, nu = Nx * (Nz + 1), nv = (Nx + 1) * Nz;
    // in the level's precision, with 1/dx^2, 1/dz^2 precomputed (FP64
    // divisions are long instruction sequences on this part)
    const T celvol = gc<T>(G, GC_CELVOL), idx2 = gc<T>(G, GC_IXX), idz2 = gc<T>(G, GC_IZZ);
    if (i < nu) {
        int k = i % Nx, l = i / Nx;
        T d = 0;
        if (G.BCu[i] == -1) {
            int c2 = k - 1 + (l - 1) * ncx;
            T inS = G.BCu[i - Nx] != 13 ? T(1) : T(0), inN = G.BCu[i + Nx] != 13 ? T(1) : T(0);
            T a = (inN * D33[i] + inS * D33[i - Nx]) * idz2 + T(2.0 / 3.0) * (D11[c2 + 1] + D11[c2]) * idx2;
            d = T(1) / (a * celvol);
        }
        idu[i] = d;
    }
    if (i < nv) {
        int k = i % (Nx + 1), l = i / (Nx + 1);
        T d = 0;
        if (G.BCv[i] == -1) {
            int c1 = k + l * Nx, c2 = k - 1 + (l - 1) * ncx;
            T inW = G.BCv[i - 1] != 13 ? T(1) : T(0), inE = G.BCv[i + 1] != 13 ? T(1) : T(0);
            T a = T(2.0 / 3.0) * (D11[c2 + ncx] + D11[c2]) * idz2 + (inE * D33[c1] + inW * D33[c1 - 1]) * idx2;
            d = T(1) / (a * celvol);
        }
        idv[i] = d;
    }
}

// out = x + omega * D^-1 (f - A x)  (x == nullptr: x = 0)
template <typename T>
__global__ void __launch_bounds__(256) k_mg_smooth(stokes_geom G, stokes_coefs<T> D, const T *__restrict__ xu,
                                                   const T *__restrict__ xv, const T *__restrict__ fu,
                                                   const T *__restrict__ fv, const T *__restrict__ idu,
                                                   const T *__restrict__ idv, T omega, T *__restrict__ ou,
                                                   T *__restrict__ ov) {
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int Nx = G.Nx, Nz = G.Nz;
    const T celvol = gc<T>(G, GC_CELVOL);
    stokes_cvec<T> x{xu, xv, nullptr};
    if (i < Nx && j <= Nz) {
        int c = i + j * Nx;
        T r = 0;
        if (G.BCu[c] == -1) {
            T ax = xu ? xrow<T, false>(G, D, x, i, j) * celvol : T(0);
            r = (xu ? xu[c] : T(0)) + omega * idu[c] * (fu[c] - ax);
        }
        ou[c] = r;
    }
    if (i <= Nx && j < Nz) {
        int c = i + j * (Nx + 1);
        T r = 0;
        if (G.BCv[c] == -1) {
            T ax = xv ? zrow<T, false>(G, D, x, i, j) * celvol : T(0);
            r = (xv ? xv[c] : T(0)) + omega * idv[c] * (fv[c] - ax);
        }
        ov[c] = r;
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_mg_residual(stokes_geom G, stokes_coefs<T> D, const T *__restrict__ xu,
                                                     const T *__restrict__ xv, const T *__restrict__ fu,
                                                     const T *__restrict__ fv, T *__restrict__ ru,
                                                     T *__restrict__ rv) {
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int Nx = G.Nx, Nz = G.Nz;
    const T celvol = gc<T>(G, GC_CELVOL);
    stokes_cvec<T> x{xu, xv, nullptr};
    if (i < Nx && j <= Nz) {
        int c = i + j * Nx;
        ru[c] = G.BCu[c] == -1 ? fu[c] - xrow<T, false>(G, D, x, i, j) * celvol : T(0);
    }
    if (i <= Nx && j < Nz) {
        int c = i + j * (Nx + 1);
        rv[c] = G.BCv[c] == -1 ? fv[c] - zrow<T, false>(G, D, x, i, j) * celvol : T(0);
    }
}

// Prolongation weights along the "cell-centred" direction of a staggered
// component: fine line j (1..ncf) -> main coarse line and neighbour, with the
// ghost neighbour mirrored onto the main line (free slip).
__device__ __forceinline__ void cc_weights(int j, int ncc, int &J0, float &w0, int &J1, float &w1) {
    int r = j - 1, R = r >> 1;
    J0 = R + 1;
    J1 = (r & 1) ? J0 + 1 : J0 - 1;
    w0 = 0.75f; w1 = 0.25f;
    if (J1 < 1 || J1 > ncc) { w0 = 1.0f; w1 = 0.0f; J1 = J0; }
}

// Weight of coarse vertex line I for fine vertex line i (node-centred direction).
__device__ __forceinline__ float nc_weight(int i, int I) {
    if ((i & 1) == 0) return i == 2 * I ? 1.0f : 0.0f;
    return (i == 2 * I - 1 || i == 2 * I + 1) ? 0.5f : 0.0f;
}

// Unknowns under the tag rule of k_level_tags (every level of a hierarchy
// follows it; the fine level is checked before the hierarchy is built).
__device__ __forceinline__ bool u_unknown(int k, int l, int Nx, int Nz) {
    return k >= 1 && k <= Nx - 2 && l >= 1 && l <= Nz - 1;
}
__device__ __forceinline__ bool v_unknown(int i, int j, int Nx, int Nz) {
    return i >= 1 && i <= Nx - 1 && j >= 1 && j <= Nz - 2;
}

// fine x += P xc at fine point (i, j) of the (Nx+1) x (Nz+1) box (both components)
template <typename T>
__device__ __forceinline__ void mg_prolong_pt(const stokes_geom &F, const stokes_geom &Cg, const T *__restrict__ cu,
                                              const T *__restrict__ cv, T *__restrict__ fu, T *__restrict__ fv,
                                              int i, int j) {
    const int Nx = F.Nx, Nz = F.Nz, Nxc = Cg.Nx;
    if (i < Nx && j <= Nz && u_unknown(i, j, Nx, Nz)) {   // Vx: x node-centred, z cell-centred
        const int c = i + j * Nx;
        int J0, J1;
        float w0, w1;
        cc_weights(j, Cg.ncz, J0, w0, J1, w1);
        const int Ia = i >> 1, Ib = (i + 1) >> 1;
        const float wa = (i & 1) ? 0.5f : 1.0f, wb = (i & 1) ? 0.5f : 0.0f;
        const T a0 = cu[Ia + J0 * Nxc], a1 = cu[Ia + J1 * Nxc], b0 = cu[Ib + J0 * Nxc], b1 = cu[Ib + J1 * Nxc];
        fu[c] += (T)(wa * w0) * a0 + (T)(wa * w1) * a1 + (T)(wb * w0) * b0 + (T)(wb * w1) * b1;
    }
    if (i <= Nx && j < Nz && v_unknown(i, j, Nx, Nz)) {   // Vz: x cell-centred, z node-centred
        const int c = i + j * (Nx + 1);
        int I0, I1;
        float w0, w1;
        cc_weights(i, Cg.ncx, I0, w0, I1, w1);
        const int Ja = j >> 1, Jb = (j + 1) >> 1;
        const float wa = (j & 1) ? 0.5f : 1.0f, wb = (j & 1) ? 0.5f : 0.0f;
        const int W = Nxc + 1;
        const T a0 = cv[I0 + Ja * W], a1 = cv[I1 + Ja * W], b0 = cv[I0 + Jb * W], b1 = cv[I1 + Jb * W];
        fv[c] += (T)(wa * w0) * a0 + (T)(wa * w1) * a1 + (T)(wb * w0) * b0 + (T)(wb * w1) * b1;
    }
}

template <typename T>
__global__ void k_mg_prolong_add(stokes_geom F, stokes_geom Cg, const T *__restrict__ cu, const T *__restrict__ cv,
                                 T *__restrict__ fu, T *__restrict__ fv) {
    mg_prolong_pt<T>(F, Cg, cu, cv, fu, fv, blockIdx.x * blockDim.x + threadIdx.x,
                     blockIdx.y * blockDim.y + threadIdx.y);
}

// coarse f = P^T fine r at coarse point (I, J): the 12 fine values of each
// component are loaded together (indices clamped into the box, weights of
// points outside the unknowns zero)
template <typename T>
__device__ __forceinline__ void mg_restrict_pt(const stokes_geom &F, const stokes_geom &Cg, const T *__restrict__ ru,
                                               const T *__restrict__ rv, T *__restrict__ cu, T *__restrict__ cv,
                                               int I, int J) {
    const int Nxf = F.Nx, Nzf = F.Nz, Nx = Cg.Nx, Nz = Cg.Nz;
    if (I < Nx && J <= Nz) {
        T s = 0;
        if (u_unknown(I, J, Nx, Nz)) {
#pragma unroll
            for (int a = 0; a < 4; a++) {
                const int j = 2 * J - 2 + a;
                int J0, J1;
                float w0, w1;
                cc_weights(j, Cg.ncz, J0, w0, J1, w1);
                const float wz = (J0 == J ? w0 : 0.0f) + (J1 == J && J1 != J0 ? w1 : 0.0f);
                const int jc = min(max(j, 0), Nzf);
#pragma unroll
                for (int b = 0; b < 3; b++) {
                    const int i = 2 * I - 1 + b;
                    const float w = (j >= 1 && j <= F.ncz && u_unknown(i, j, Nxf, Nzf)) ? nc_weight(i, I) * wz : 0.0f;
                    s += (T)w * ru[min(max(i, 0), Nxf - 1) + jc * Nxf];
                }
            }
        }
        cu[I + J * Nx] = s;
    }
    if (I <= Nx && J < Nz) {
        T s = 0;
        if (v_unknown(I, J, Nx, Nz)) {
#pragma unroll
            for (int a = 0; a < 4; a++) {
                const int i = 2 * I - 2 + a;
                int I0, I1;
                float w0, w1;
                cc_weights(i, Cg.ncx, I0, w0, I1, w1);
                const float wx = (I0 == I ? w0 : 0.0f) + (I1 == I && I1 != I0 ? w1 : 0.0f);
                const int ic = min(max(i, 0), Nxf);
#pragma unroll
                for (int b = 0; b < 3; b++) {
                    const int j = 2 * J - 1 + b;
                    const float w = (i >= 1 && i <= F.ncx && v_unknown(i, j, Nxf, Nzf)) ? wx * nc_weight(j, J) : 0.0f;
                    s += (T)w * rv[ic + min(max(j, 0), Nzf - 1) * (Nxf + 1)];
                }
            }
        }
        cv[I + J * (Nx + 1)] = s;
    }
}

template <typename T>
__global__ void k_mg_restrict(stokes_geom F, stokes_geom Cg, const T *__restrict__ ru, const T *__restrict__ rv,
                              T *__restrict__ cu, T *__restrict__ cv) {
    mg_restrict_pt<T>(F, Cg, ru, rv, cu, cv, blockIdx.x * blockDim.x + threadIdx.x,
                      blockIdx.y * blockDim.y + threadIdx.y);
}

// ---------------------------------------------------------------------------
// Galerkin coarse operators.  Re-discretised coarse levels (averaged
// viscosities) lose the coupling across layers of 1e5 viscosity contrast and
// the V-cycle stops converging; R A P keeps it.  With this P (bilinear in the
// staggered sense) and R = P^T the coarse stencils close on a fixed footprint:
//   u-row (K, L):  uu  dK in [-1, 1], dL in [-2, 2]   planes  0..14: (dK+1) + 3 (dL+2)
//                  uv  I-K in [-1, 2], J-L in [-2, 1]  planes 15..30: 15 + (dI+1) + 4 (dJ+2)
//   v-row (I, J):  vv  dI in [-2, 2], dJ in [-1, 1]   planes  0..14: (dI+2) + 5 (dJ+1)
//                  vu  K-I in [-2, 1], L-J in [-1, 2]  planes 15..30: 15 + (dK+2) + 4 (dL+1)
// (u index (k, l) of the Nx x (Nz+1) box, v index (i, j) of the (Nx+1) x Nz box).
// The level-0 stencil is a subset of this footprint.

// y = A x for a stencil level, one u-row / v-row.  All 31 coefficients and
// neighbour values are loaded before the first multiply (neighbour indices
// clamped into the box, out-of-box terms masked to zero) so that the loads
// overlap instead of waiting on each other behind the bounds tests.
template <typename T>
__device__ __forceinline__ T st_urow(int Nx, int Nz, const T *__restrict__ su, size_t nu, const T *__restrict__ xu,
                                     const T *__restrict__ xv, int k, int l) {
    const size_t c = (size_t)k + (size_t)l * Nx;
    T cf[MG_NST], xn[MG_NST];
#pragma unroll
    for (int q = 0; q < 15; q++) {   // uu: (dk, dl) = (q % 3 - 1, q / 3 - 2)
        const int kk = k + q % 3 - 1, ll = l + q / 3 - 2;
        const bool in = kk >= 0 && kk < Nx && ll >= 0 && ll <= Nz;
        const int kc = min(max(kk, 0), Nx - 1), lc = min(max(ll, 0), Nz);
        cf[q] = su[(size_t)q * nu + c];
        xn[q] = xu[kc + lc * Nx];
        if (!in) cf[q] = T(0);
    }
#pragma unroll
    for (int q = 0; q < 16; q++) {   // uv: (dI, dJ) = (q % 4 - 1, q / 4 - 2)
        const int i = k + q % 4 - 1, j = l + q / 4 - 2;
        const bool in = i >= 0 && i <= Nx && j >= 0 && j < Nz;
        const int ic = min(max(i, 0), Nx), jc = min(max(j, 0), Nz - 1);
        cf[15 + q] = su[(size_t)(15 + q) * nu + c];
        xn[15 + q] = xv[ic + jc * (Nx + 1)];
        if (!in) cf[15 + q] = T(0);
    }
    T s = 0;
#pragma unroll
    for (int q = 0; q < MG_NST; q++) s += cf[q] * xn[q];
    return s;
}

template <typename T>
__device__ __forceinline__ T st_vrow(int Nx, int Nz, const T *__restrict__ sv, size_t nv, const T *__restrict__ xu,
                                     const T *__restrict__ xv, int i, int j) {
    const size_t c = (size_t)i + (size_t)j * (Nx + 1);
    T cf[MG_NST], xn[MG_NST];
#pragma unroll
    for (int q = 0; q < 15; q++) {   // vv: (dI, dJ) = (q % 5 - 2, q / 5 - 1)
        const int ii = i + q % 5 - 2, jj = j + q / 5 - 1;
        const bool in = ii >= 0 && ii <= Nx && jj >= 0 && jj < Nz;
        const int ic = min(max(ii, 0), Nx), jc = min(max(jj, 0), Nz - 1);
        cf[q] = sv[(size_t)q * nv + c];
        xn[q] = xv[ic + jc * (Nx + 1)];
        if (!in) cf[q] = T(0);
    }
#pragma unroll
    for (int q = 0; q < 16; q++) {   // vu: (dK, dL) = (q % 4 - 2, q / 4 - 1)
        const int k = i + q % 4 - 2, l = j + q / 4 - 1;
        const bool in = k >= 0 && k < Nx && l >= 0 && l <= Nz;
        const int kc = min(max(k, 0), Nx - 1), lc = min(max(l, 0), Nz);
        cf[15 + q] = sv[(size_t)(15 + q) * nv + c];
        xn[15 + q] = xu[kc + lc * Nx];
        if (!in) cf[15 + q] = T(0);
    }
    T s = 0;
#pragma unroll
    for (int q = 0; q < MG_NST; q++) s += cf[q] * xn[q];
    return s;
}

// out = x + omega D^-1 (f - A x) on a stencil level, one u-row (i, j) or
// v-row (i, j) (x == nullptr: x = 0)
template <typename T>
__device__ __forceinline__ void st_smooth_u(const stokes_geom &G, const T *__restrict__ su, const T *__restrict__ sv,
                                            const T *__restrict__ xu, const T *__restrict__ xv,
                                            const T *__restrict__ fu, const T *__restrict__ idu, T omega,
                                            T *__restrict__ ou, int i, int j) {
    const int Nx = G.Nx, Nz = G.Nz;
    const size_t nu = (size_t)Nx * (Nz + 1);
    const int c = i + j * Nx;
    T r = 0;
    if (u_unknown(i, j, Nx, Nz)) {
        if (xu) r = xu[c] + omega * idu[c] * (fu[c] - st_urow<T>(Nx, Nz, su, nu, xu, xv, i, j));
        else r = omega * idu[c] * fu[c];
    }
    ou[c] = r;
}

template <typename T>
__device__ __forceinline__ void st_smooth_v(const stokes_geom &G, const T *__restrict__ su, const T *__restrict__ sv,
                                            const T *__restrict__ xu, const T *__restrict__ xv,
                                            const T *__restrict__ fv, const T *__restrict__ idv, T omega,
                                            T *__restrict__ ov, int i, int j) {
    const int Nx = G.Nx, Nz = G.Nz;
    const size_t nv = (size_t)(Nx + 1) * Nz;
    const int c = i + j * (Nx + 1);
    T r = 0;
    if (v_unknown(i, j, Nx, Nz)) {
        if (xv) r = xv[c] + omega * idv[c] * (fv[c] - st_vrow<T>(Nx, Nz, sv, nv, xu, xv, i, j));
        else r = omega * idv[c] * fv[c];
    }
    ov[c] = r;
}

// both rows at point (i, j) of the (Nx+1) x (Nz+1) box
template <typename T>
__device__ __forceinline__ void st_smooth_pt(const stokes_geom &G, const T *__restrict__ su, const T *__restrict__ sv,
                                             const T *__restrict__ xu, const T *__restrict__ xv,
                                             const T *__restrict__ fu, const T *__restrict__ fv,
                                             const T *__restrict__ idu, const T *__restrict__ idv, T omega,
                                             T *__restrict__ ou, T *__restrict__ ov, int i, int j) {
    if (i < G.Nx && j <= G.Nz) st_smooth_u<T>(G, su, sv, xu, xv, fu, idu, omega, ou, i, j);
    if (i <= G.Nx && j < G.Nz) st_smooth_v<T>(G, su, sv, xu, xv, fv, idv, omega, ov, i, j);
}

// one thread per row (u rows first, then v rows): twice the threads of a
// point-per-thread launch, so that the fine stencil levels fill the machine
template <typename T>
__global__ void __launch_bounds__(128) k_st_smooth(stokes_geom G, const T *__restrict__ su, const T *__restrict__ sv,
                                                   const T *__restrict__ xu, const T *__restrict__ xv,
                                                   const T *__restrict__ fu, const T *__restrict__ fv,
                                                   const T *__restrict__ idu, const T *__restrict__ idv, T omega,
                                                   T *__restrict__ ou, T *__restrict__ ov) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int Nx = G.Nx, nu = Nx * (G.Nz + 1), nv = (Nx + 1) * G.Nz;
    if (t < nu) st_smooth_u<T>(G, su, sv, xu, xv, fu, idu, omega, ou, t % Nx, t / Nx);
    else if (t < nu + nv) st_smooth_v<T>(G, su, sv, xu, xv, fv, idv, omega, ov, (t - nu) % (Nx + 1), (t - nu) / (Nx + 1));
}

template <typename T>
__device__ __forceinline__ void st_residual_u(const stokes_geom &G, const T *__restrict__ su, const T *__restrict__ xu,
                                              const T *__restrict__ xv, const T *__restrict__ fu, T *__restrict__ ru,
                                              int i, int j) {
    const int Nx = G.Nx, Nz = G.Nz, c = i + j * Nx;
    ru[c] = u_unknown(i, j, Nx, Nz) ? fu[c] - st_urow<T>(Nx, Nz, su, (size_t)Nx * (Nz + 1), xu, xv, i, j) : T(0);
}

template <typename T>
__device__ __forceinline__ void st_residual_v(const stokes_geom &G, const T *__restrict__ sv, const T *__restrict__ xu,
                                              const T *__restrict__ xv, const T *__restrict__ fv, T *__restrict__ rv,
                                              int i, int j) {
    const int Nx = G.Nx, Nz = G.Nz, c = i + j * (Nx + 1);
    rv[c] = v_unknown(i, j, Nx, Nz) ? fv[c] - st_vrow<T>(Nx, Nz, sv, (size_t)(Nx + 1) * Nz, xu, xv, i, j) : T(0);
}

template <typename T>
__device__ __forceinline__ void st_residual_pt(const stokes_geom &G, const T *__restrict__ su,
                                               const T *__restrict__ sv, const T *__restrict__ xu,
                                               const T *__restrict__ xv, const T *__restrict__ fu,
                                               const T *__restrict__ fv, T *__restrict__ ru, T *__restrict__ rv,
                                               int i, int j) {
    if (i < G.Nx && j <= G.Nz) st_residual_u<T>(G, su, xu, xv, fu, ru, i, j);
    if (i <= G.Nx && j < G.Nz) st_residual_v<T>(G, sv, xu, xv, fv, rv, i, j);
}

template <typename T>
__global__ void __launch_bounds__(128) k_st_residual(stokes_geom G, const T *__restrict__ su,
                                                     const T *__restrict__ sv, const T *__restrict__ xu,
                                                     const T *__restrict__ xv, const T *__restrict__ fu,
                                                     const T *__restrict__ fv, T *__restrict__ ru,
                                                     T *__restrict__ rv) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int Nx = G.Nx, nu = Nx * (G.Nz + 1), nv = (Nx + 1) * G.Nz;
    if (t < nu) st_residual_u<T>(G, su, xu, xv, fu, ru, t % Nx, t / Nx);
    else if (t < nu + nv) st_residual_v<T>(G, sv, xu, xv, fv, rv, (t - nu) % (Nx + 1), (t - nu) / (Nx + 1));
}

template <typename T>
__global__ void k_st_diag(stokes_geom G, const T *__restrict__ su, const T *__restrict__ sv, T *__restrict__ idu,
                          T *__restrict__ idv) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    const size_t nu = (size_t)G.Nx * (G.Nz + 1), nv = (size_t)(G.Nx + 1) * G.Nz;
    if (i < (long long)nu) idu[i] = G.BCu[i] == -1 ? T(1) / su[(size_t)MG_CENTER * nu + i] : T(0);
    if (i < (long long)nv) idv[i] = G.BCv[i] == -1 ? T(1) / sv[(size_t)MG_CENTER * nv + i] : T(0);
}

// Level-0 probing: x = indicator of the unknowns of component comp with
// (k mod 4, l mod 4) = (cx, cz); y = A x.  The level-0 operator (Picard or
// Newton) couples a row to same-component nodes within [-1, 1]^2 and to
// other-component nodes within a 4 x 4 window, so each colour class holds at
// most one node of a row's footprint and y at the row is one coefficient.
#define MG_PROBE 4
template <typename T>
__global__ void k_probe_vec(stokes_geom G, int comp, int cx, int cz, T *__restrict__ xu, T *__restrict__ xv) {
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int Nx = G.Nx, Nz = G.Nz;
    if (i < Nx && j <= Nz) {
        int c = i + j * Nx;
        xu[c] = (comp == 0 && G.BCu[c] == -1 && i % MG_PROBE == cx && j % MG_PROBE == cz) ? T(1) : T(0);
    }
    if (i <= Nx && j < Nz) {
        int c = i + j * (Nx + 1);
        xv[c] = (comp == 1 && G.BCv[c] == -1 && i % MG_PROBE == cx && j % MG_PROBE == cz) ? T(1) : T(0);
    }
}

// velocity rows of the Picard (NEWTON = false, p0 unused) or Newton operator
// (p0 = a zero pressure vector) applied to (xu, xv, 0)
template <typename T, bool NEWTON>
__global__ void __launch_bounds__(256) k_mg_apply(stokes_geom G, stokes_coefs<T> D, const T *__restrict__ xu,
                                                  const T *__restrict__ xv, const T *__restrict__ p0,
                                                  T *__restrict__ yu, T *__restrict__ yv) {
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int Nx = G.Nx, Nz = G.Nz;
    const T celvol = gc<T>(G, GC_CELVOL);
    stokes_cvec<T> x{xu, xv, NEWTON ? p0 : nullptr};
    if (i < Nx && j <= Nz) {
        int c = i + j * Nx;
        yu[c] = G.BCu[c] == -1 ? xrow<T, NEWTON>(G, D, x, i, j) * celvol : T(0);
    }
    if (i <= Nx && j < Nz) {
        int c = i + j * (Nx + 1);
        yv[c] = G.BCv[c] == -1 ? zrow<T, NEWTON>(G, D, x, i, j) * celvol : T(0);
    }
}

// offset of the colour-cx node from position p along one direction inside the
// window [lo, hi] (at most MG_PROBE wide): returns 1 and the offset, or 0
__device__ __forceinline__ int colour_offset(int p, int cx, int lo, int hi, int *d) {
    for (int o = lo; o <= hi; o++)
        if ((((p + o) % MG_PROBE) + MG_PROBE) % MG_PROBE == cx) { *d = o; return 1; }
    return 0;
}

template <typename T>
__global__ void k_probe_collect(stokes_geom G, int comp, int cx, int cz, const T *__restrict__ yu,
                                const T *__restrict__ yv, T *__restrict__ su, T *__restrict__ sv) {
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int Nx = G.Nx, Nz = G.Nz;
    const size_t nu = (size_t)Nx * (Nz + 1), nv = (size_t)(Nx + 1) * Nz;
    int a, b;
    if (i < Nx && j <= Nz) {
        int c = i + j * Nx;
        if (G.BCu[c] == -1) {
            if (comp == 0) {   // uu within [-1, 1]^2
                if (colour_offset(i, cx, -1, 1, &a) && colour_offset(j, cz, -1, 1, &b))
                    su[(size_t)((a + 1) + 3 * (b + 2)) * nu + c] = yu[c];
            } else {           // uv: I - k in [-1, 2], J - l in [-2, 1]
                if (colour_offset(i, cx, -1, 2, &a) && colour_offset(j, cz, -2, 1, &b))
                    su[(size_t)(15 + (a + 1) + 4 * (b + 2)) * nu + c] = yu[c];
            }
        }
    }
    if (i <= Nx && j < Nz) {
        int c = i + j * (Nx + 1);
        if (G.BCv[c] == -1) {
            if (comp == 1) {   // vv within [-1, 1]^2
                if (colour_offset(i, cx, -1, 1, &a) && colour_offset(j, cz, -1, 1, &b))
                    sv[(size_t)((a + 2) + 5 * (b + 1)) * nv + c] = yv[c];
            } else {           // vu: K - i in [-2, 1], L - j in [-1, 2]
                if (colour_offset(i, cx, -2, 1, &a) && colour_offset(j, cz, -1, 2, &b))
                    sv[(size_t)(15 + (a + 2) + 4 * (b + 1)) * nv + c] = yv[c];
            }
        }
    }
}

// Level-0 stencils of the Picard velocity block written out directly from
// the viscosities (the composition strain rate -> D11 / D33 stress ->
// divergence of xrow / zrow with the same row flags, times the cell volume),
// one thread per (i, j), in the level's precision; every plane of every row
// is written, zeros outside the unknowns.  Equal to probing the Picard
// operator, in one pass.
//   u-row (k, l), aE = inE D11[E], aW = inW D11[W], bN = inN D33[N], bS = inS D33[S]:
//     u(k+-1, l): -2/3 aE|aW / dx^2   u(k, l+-1): -bN|bS / dz^2   u(k, l): the sum of their negatives
//     v(k+1, l): aE/3 - bN   v(k+1, l-1): bS - aE/3   v(k, l): bN - aW/3   v(k, l-1): aW/3 - bS   (/ dx dz)
//   v-row (i, j), cN = inN D22[N], cS = inS D22[S], dE = inE D33[E], dW = inW D33[W]:
//     v(i, j+-1): -2/3 cN|cS / dz^2   v(i+-1, j): -dE|dW / dx^2   v(i, j): the sum of their negatives
//     u(i, j+1): cN/3 - dE   u(i-1, j+1): dW - cN/3   u(i, j): dE - cS/3   u(i-1, j): cS/3 - dW   (/ dx dz)
template <typename T>
__global__ void __launch_bounds__(256) k_picard_stencil(stokes_geom G, const T *__restrict__ D11,
                                                        const T *__restrict__ D33, T *__restrict__ su,
                                                        T *__restrict__ sv) {
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int Nx = G.Nx, Nz = G.Nz, nx = Nx, ncx = G.ncx, nxvz = Nx + 1;
    const size_t nu = (size_t)Nx * (Nz + 1), nv = (size_t)(Nx + 1) * Nz;
    const T celvol = gc<T>(G, GC_CELVOL), ixx = gc<T>(G, GC_IXX), izz = gc<T>(G, GC_IZZ),
            ixz = gc<T>(G, GC_IXZ);
    if (i < Nx && j <= Nz) {   // u-row (k, l) = (i, j)
        const int k = i, l = j, c1 = k + l * nx;
        T a[MG_NST];
#pragma unroll
        for (int q = 0; q < MG_NST; q++) a[q] = T(0);
        if (G.BCu[c1] == -1) {
            const int c2 = k - 1 + (l - 1) * ncx, iPrW = c2, iPrE = c2 + 1, ixyN = c1, ixyS = c1 - nx;
            const T inW = G.BCp[iPrW] == -1 ? T(1) : T(0), inE = G.BCp[iPrE] == -1 ? T(1) : T(0);
            const T inS = (G.BCg[ixyS] != 30 && G.BCu[c1 - nx] != 13) ? T(1) : T(0);
            const T inN = (G.BCg[ixyN] != 30 && G.BCu[c1 + nx] != 13) ? T(1) : T(0);
            const T aE = inE * D11[iPrE], aW = inW * D11[iPrW];
            const T bN = inN * D33[ixyN], bS = inS * D33[ixyS];
            const T uE = -T(2.0 * T(1.0 / 3.0)) * aE * ixx, uW = -T(2.0 * T(1.0 / 3.0)) * aW * ixx;
            const T uN = -bN * izz, uS = -bS * izz;
            auto isu = [&](int kk, int ll) { return G.BCu[kk + ll * nx] == -1 ? T(1) : T(0); };
            auto isv = [&](int ii, int jj) { return G.BCv[ii + jj * nxvz] == -1 ? T(1) : T(0); };
            a[(0 + 1) + 3 * (0 + 2)] = -(uE + uW + uN + uS);
            a[(1 + 1) + 3 * (0 + 2)] = uE * isu(k + 1, l);
            a[(-1 + 1) + 3 * (0 + 2)] = uW * isu(k - 1, l);
            a[(0 + 1) + 3 * (1 + 2)] = uN * isu(k, l + 1);
            a[(0 + 1) + 3 * (-1 + 2)] = uS * isu(k, l - 1);
            a[15 + (1 + 1) + 4 * (0 + 2)] = (aE * T(1.0 / 3.0) - bN) * ixz * isv(k + 1, l);
            a[15 + (1 + 1) + 4 * (-1 + 2)] = (bS - aE * T(1.0 / 3.0)) * ixz * isv(k + 1, l - 1);
            a[15 + (0 + 1) + 4 * (0 + 2)] = (bN - aW * T(1.0 / 3.0)) * ixz * isv(k, l);
            a[15 + (0 + 1) + 4 * (-1 + 2)] = (aW * T(1.0 / 3.0) - bS) * ixz * isv(k, l - 1);
        }
#pragma unroll
        for (int q = 0; q < MG_NST; q++) su[(size_t)q * nu + c1] = a[q] * celvol;
    }
    if (i <= Nx && j < Nz) {   // v-row (k, l) = (i, j)
        const int k = i, l = j, c3 = k + l * nxvz;
        T a[MG_NST];
#pragma unroll
        for (int q = 0; q < MG_NST; q++) a[q] = T(0);
        if (G.BCv[c3] == -1) {
            const int c1 = k + l * nx, c2 = k - 1 + (l - 1) * ncx;
            const int iPrS = c2, iPrN = c2 + ncx, ixyW = c1 - 1, ixyE = c1;
            T inS = 0, inN = 0;
            const bool s30 = G.BCv[c3 - nxvz] == 30, n30 = G.BCv[c3 + nxvz] == 30;
            if (!s30 && !n30) { inS = 1; inN = 1; }
            if (s30 && !n30) inN = 1;
            if (!s30 && n30) inS = 1;
            if (G.BCp[iPrS] == -1) inS = 1;
            if (G.BCp[iPrN] == -1) inN = 1;
            const T inW = (G.BCg[ixyW] != 30 && G.BCv[c3 - 1] != 13) ? T(1) : T(0);
            const T inE = (G.BCg[ixyE] != 30 && G.BCv[c3 + 1] != 13) ? T(1) : T(0);
            const T cN = inN * D11[iPrN], cS = inS * D11[iPrS];
            const T dE = inE * D33[ixyE], dW = inW * D33[ixyW];
            const T vN = -T(2.0 * T(1.0 / 3.0)) * cN * izz, vS = -T(2.0 * T(1.0 / 3.0)) * cS * izz;
            const T vE = -dE * ixx, vW = -dW * ixx;
            auto isu = [&](int kk, int ll) { return G.BCu[kk + ll * nx] == -1 ? T(1) : T(0); };
            auto isv = [&](int ii, int jj) { return G.BCv[ii + jj * nxvz] == -1 ? T(1) : T(0); };
            a[(0 + 2) + 5 * (0 + 1)] = -(vN + vS + vE + vW);
            a[(0 + 2) + 5 * (1 + 1)] = vN * isv(k, l + 1);
            a[(0 + 2) + 5 * (-1 + 1)] = vS * isv(k, l - 1);
            a[(1 + 2) + 5 * (0 + 1)] = vE * isv(k + 1, l);
            a[(-1 + 2) + 5 * (0 + 1)] = vW * isv(k - 1, l);
            a[15 + (0 + 2) + 4 * (1 + 1)] = (cN * T(1.0 / 3.0) - dE) * ixz * isu(k, l + 1);
            a[15 + (-1 + 2) + 4 * (1 + 1)] = (dW - cN * T(1.0 / 3.0)) * ixz * isu(k - 1, l + 1);
            a[15 + (0 + 2) + 4 * (0 + 1)] = (dE - cS * T(1.0 / 3.0)) * ixz * isu(k, l);
            a[15 + (-1 + 2) + 4 * (0 + 1)] = (cS * T(1.0 / 3.0) - dW) * ixz * isu(k - 1, l);
        }
#pragma unroll
        for (int q = 0; q < MG_NST; q++) sv[(size_t)q * nv + c3] = a[q] * celvol;
    }
}

// Coarse stencils = R A P, four threads per coarse row (one fine line of the
// restriction each, summed in shared memory at the end), accumulated in the
// level's precision (FP64 throughput is a small fraction of FP32 on this
// part) in shared memory (plane-major, one column per thread).  Every level of the
// hierarchy follows the tag rule (u_unknown / v_unknown), so the kernel
// reads no tags.  Each fine row's 31 coefficients are loaded in
// one batch before use: loaded one at a time behind the zero test they
// serialise on memory latency.  An entry landing outside the footprint
// (impossible with this P) sets *bad.
// parents of fine u node (i, j) / v node (i, j) as coarse (I, J) pairs
__device__ __forceinline__ void u_parents_ij(int i, int j, int nczc, int *I, int *J, float *w) {
    int J0, J1;
    float w0, w1;
    cc_weights(j, nczc, J0, w0, J1, w1);
    const int Ia = i >> 1, Ib = (i + 1) >> 1;
    const float wa = (i & 1) ? 0.5f : 1.0f, wb = (i & 1) ? 0.5f : 0.0f;
    I[0] = Ia; J[0] = J0; w[0] = wa * w0;
    I[1] = Ia; J[1] = J1; w[1] = wa * w1;
    I[2] = Ib; J[2] = J0; w[2] = wb * w0;
    I[3] = Ib; J[3] = J1; w[3] = wb * w1;
}
__device__ __forceinline__ void v_parents_ij(int i, int j, int ncxc, int *I, int *J, float *w) {
    int I0, I1;
    float w0, w1;
    cc_weights(i, ncxc, I0, w0, I1, w1);
    const int Ja = j >> 1, Jb = (j + 1) >> 1;
    const float wa = (j & 1) ? 0.5f : 1.0f, wb = (j & 1) ? 0.5f : 0.0f;
    I[0] = I0; J[0] = Ja; w[0] = wa * w0;
    I[1] = I1; J[1] = Ja; w[1] = wa * w1;
    I[2] = I0; J[2] = Jb; w[2] = wb * w0;
    I[3] = I1; J[3] = Jb; w[3] = wb * w1;
}

#define GAL_THREADS 128
#define GAL_SPLIT 4   // threads per coarse row: each takes one of the 4 fine lines of the restriction
template <typename T>
__global__ void __launch_bounds__(GAL_THREADS) k_galerkin(stokes_geom F, const T *__restrict__ suF,
                                                          const T *__restrict__ svF, stokes_geom Cg,
                                                          T *__restrict__ suC, T *__restrict__ svC, int *bad) {
    __shared__ T acc_sh[MG_NST * GAL_THREADS];
    T *acc = acc_sh + threadIdx.x;
#define ACC(q) acc[(q) * GAL_THREADS]
    const long long gt = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int t = (int)(gt / GAL_SPLIT), sub = (int)(gt % GAL_SPLIT);   // coarse row, fine line of it
    const int col0 = threadIdx.x - sub;                                  // the row's first column here
    const int Nxf = F.Nx, Nzf = F.Nz, Nxc = Cg.Nx, Nzc = Cg.Nz;
    const size_t nuf = (size_t)Nxf * (Nzf + 1), nvf = (size_t)(Nxf + 1) * Nzf;
    const int nuc = Nxc * (Nzc + 1), nvc = (Nxc + 1) * Nzc;
    int PI[4], PJ[4];
    float pw[4];
    T a[MG_NST];
    if (t < nuc) {   // coarse u-row (K, L)
        const int K = t % Nxc, L = t / Nxc;
        for (int q = 0; q < MG_NST; q++) ACC(q) = T(0);
        if (u_unknown(K, L, Nxc, Nzc)) {
            for (int lf = 2 * L - 2 + sub; lf <= 2 * L - 2 + sub; lf++) {
                if (lf < 1 || lf > F.ncz) continue;
                int J0, J1;
                float w0, w1;
                cc_weights(lf, Cg.ncz, J0, w0, J1, w1);
                const float wz = (J0 == L ? w0 : 0.0f) + (J1 == L && J1 != J0 ? w1 : 0.0f);
                if (wz == 0.0f) continue;
                for (int k = 2 * K - 1; k <= 2 * K + 1; k++) {
                    if (!u_unknown(k, lf, Nxf, Nzf)) continue;
                    const size_t f = (size_t)k + (size_t)lf * Nxf;
                    const T R = (T)(nc_weight(k, K) * wz);
#pragma unroll
                    for (int q = 0; q < MG_NST; q++) a[q] = __ldg(suF + (size_t)q * nuf + f);
#pragma unroll
                    for (int q = 0; q < 15; q++) {   // uu entries of the fine row
                        if (a[q] == T(0)) continue;
                        u_parents_ij(k + q % 3 - 1, lf + q / 3 - 2, Cg.ncz, PI, PJ, pw);
                        const T ra = R * a[q];
#pragma unroll
                        for (int s = 0; s < 4; s++) {
                            if (pw[s] == 0.0f || !u_unknown(PI[s], PJ[s], Nxc, Nzc)) continue;
                            const int dK = PI[s] - K, dL = PJ[s] - L;
                            if (dK < -1 || dK > 1 || dL < -2 || dL > 2) { *bad = 1; continue; }
                            ACC((dK + 1) + 3 * (dL + 2)) += ra * (T)pw[s];
                        }
                    }
#pragma unroll
                    for (int q = 0; q < 16; q++) {   // uv entries of the fine row
                        if (a[15 + q] == T(0)) continue;
                        v_parents_ij(k + q % 4 - 1, lf + q / 4 - 2, Cg.ncx, PI, PJ, pw);
                        const T ra = R * a[15 + q];
#pragma unroll
                        for (int s = 0; s < 4; s++) {
                            if (pw[s] == 0.0f || !v_unknown(PI[s], PJ[s], Nxc, Nzc)) continue;
                            const int dI = PI[s] - K, dJ = PJ[s] - L;
                            if (dI < -1 || dI > 2 || dJ < -2 || dJ > 1) { *bad = 1; continue; }
                            ACC(15 + (dI + 1) + 4 * (dJ + 2)) += ra * (T)pw[s];
                        }
                    }
                }
            }
        }
    }
    __syncthreads();
    if (t < nuc)
        for (int q = sub; q < MG_NST; q += GAL_SPLIT) {
            const T *c = acc_sh + q * GAL_THREADS + col0;
            suC[(size_t)q * nuc + t] = (c[0] + c[1]) + (c[2] + c[3]);
        }
    __syncthreads();
    if (t < nvc) {   // coarse v-row (I, J)
        const int I = t % (Nxc + 1), J = t / (Nxc + 1);
        for (int q = 0; q < MG_NST; q++) ACC(q) = T(0);
        if (v_unknown(I, J, Nxc, Nzc)) {
            for (int i = 2 * I - 2 + sub; i <= 2 * I - 2 + sub; i++) {
                if (i < 1 || i > F.ncx) continue;
                int I0, I1;
                float w0, w1;
                cc_weights(i, Cg.ncx, I0, w0, I1, w1);
                const float wx = (I0 == I ? w0 : 0.0f) + (I1 == I && I1 != I0 ? w1 : 0.0f);
                if (wx == 0.0f) continue;
                for (int j = 2 * J - 1; j <= 2 * J + 1; j++) {
                    if (!v_unknown(i, j, Nxf, Nzf)) continue;
                    const size_t f = (size_t)i + (size_t)j * (Nxf + 1);
                    const T R = (T)(wx * nc_weight(j, J));
#pragma unroll
                    for (int q = 0; q < MG_NST; q++) a[q] = __ldg(svF + (size_t)q * nvf + f);
#pragma unroll
                    for (int q = 0; q < 15; q++) {   // vv entries
                        if (a[q] == T(0)) continue;
                        v_parents_ij(i + q % 5 - 2, j + q / 5 - 1, Cg.ncx, PI, PJ, pw);
                        const T ra = R * a[q];
#pragma unroll
                        for (int s = 0; s < 4; s++) {
                            if (pw[s] == 0.0f || !v_unknown(PI[s], PJ[s], Nxc, Nzc)) continue;
                            const int dI = PI[s] - I, dJ = PJ[s] - J;
                            if (dI < -2 || dI > 2 || dJ < -1 || dJ > 1) { *bad = 1; continue; }
                            ACC((dI + 2) + 5 * (dJ + 1)) += ra * (T)pw[s];
                        }
                    }
#pragma unroll
                    for (int q = 0; q < 16; q++) {   // vu entries
                        if (a[15 + q] == T(0)) continue;
                        u_parents_ij(i + q % 4 - 2, j + q / 4 - 1, Cg.ncz, PI, PJ, pw);
                        const T ra = R * a[15 + q];
#pragma unroll
                        for (int s = 0; s < 4; s++) {
                            if (pw[s] == 0.0f || !u_unknown(PI[s], PJ[s], Nxc, Nzc)) continue;
                            const int dK = PI[s] - I, dL = PJ[s] - J;
                            if (dK < -2 || dK > 1 || dL < -1 || dL > 2) { *bad = 1; continue; }
                            ACC(15 + (dK + 2) + 4 * (dL + 1)) += ra * (T)pw[s];
                        }
                    }
                }
            }
        }
    }
    __syncthreads();
    if (t < nvc)
        for (int q = sub; q < MG_NST; q += GAL_SPLIT) {
            const T *c = acc_sh + q * GAL_THREADS + col0;
            svC[(size_t)q * nvc + t] = (c[0] + c[1]) + (c[2] + c[3]);
        }
#undef ACC
}

template <typename T>
__global__ void k_fill_D11_D33(int nc, int nv, const double *__restrict__ eta_n, const double *__restrict__ eta_s,
                               T *__restrict__ D11, T *__restrict__ D33) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nc) D11[i] = (T)(2.0 * eta_n[i]);
    if (i < nv) D33[i] = (T)eta_s[i];
}

// ---------------------------------------------------------------------------
// Coarsest level: one CTA runs Jacobi-preconditioned CG on the whole level.
template <typename T>
__device__ double cta_dot(const T *a, const T *b, int n0, int n1, const T *a1, const T *b1, double *sh) {
    double s = 0.0;
    for (int i = threadIdx.x; i < n0; i += blockDim.x) s += (double)a[i] * (double)b[i];
    for (int i = threadIdx.x; i < n1; i += blockDim.x) s += (double)a1[i] * (double)b1[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = s;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) sh[32] = t;
    }
    __syncthreads();
    return sh[32];
}

template <typename T>
__device__ void cta_apply(const stokes_geom &G, const T *su, const T *sv, const T *xu, const T *xv, T *yu, T *yv) {
    const int Nx = G.Nx, Nz = G.Nz;
    const size_t nu = (size_t)Nx * (Nz + 1), nv = (size_t)(Nx + 1) * Nz;
    for (int c = threadIdx.x; c < (int)nu; c += blockDim.x)
        yu[c] = G.BCu[c] == -1 ? st_urow<T>(Nx, Nz, su, nu, xu, xv, c % Nx, c / Nx) : T(0);
    for (int c = threadIdx.x; c < (int)nv; c += blockDim.x)
        yv[c] = G.BCv[c] == -1 ? st_vrow<T>(Nx, Nz, sv, nv, xu, xv, c % (Nx + 1), c / (Nx + 1)) : T(0);
}

template <typename T>
__global__ void __launch_bounds__(1024) k_mg_coarse_cg(stokes_geom G, const T *su, const T *sv, const T *__restrict__ fu,
                                                       const T *__restrict__ fv, const T *__restrict__ idu,
                                                       const T *__restrict__ idv, T *xu, T *xv, T *ru, T *rv, T *zu,
                                                       T *zv, T *pu, T *pv, T *qu, T *qv, int maxit, double rtol) {
    __shared__ double sh[34];
    const int nu = G.Nx * (G.Nz + 1), nv = (G.Nx + 1) * G.Nz;
    for (int i = threadIdx.x; i < nu; i += blockDim.x) { xu[i] = 0; ru[i] = fu[i]; zu[i] = idu[i] * fu[i]; pu[i] = zu[i]; }
    for (int i = threadIdx.x; i < nv; i += blockDim.x) { xv[i] = 0; rv[i] = fv[i]; zv[i] = idv[i] * fv[i]; pv[i] = zv[i]; }
    __syncthreads();
    double rz = cta_dot<T>(ru, zu, nu, nv, rv, zv, sh);
    double r0 = cta_dot<T>(ru, ru, nu, nv, rv, rv, sh);
    if (r0 == 0.0) return;
    for (int it = 0; it < maxit; it++) {
        cta_apply<T>(G, su, sv, pu, pv, qu, qv);
        __syncthreads();
        double pq = cta_dot<T>(pu, qu, nu, nv, pv, qv, sh);
        if (pq <= 0.0) break;
        T a = (T)(rz / pq);
        for (int i = threadIdx.x; i < nu; i += blockDim.x) { xu[i] += a * pu[i]; ru[i] -= a * qu[i]; zu[i] = idu[i] * ru[i]; }
        for (int i = threadIdx.x; i < nv; i += blockDim.x) { xv[i] += a * pv[i]; rv[i] -= a * qv[i]; zv[i] = idv[i] * rv[i]; }
        __syncthreads();
        double rz1 = cta_dot<T>(ru, zu, nu, nv, rv, zv, sh);
        double rr = cta_dot<T>(ru, ru, nu, nv, rv, rv, sh);
        if (rr <= rtol * rtol * r0) break;
        T b = (T)(rz1 / rz);
        rz = rz1;
        for (int i = threadIdx.x; i < nu; i += blockDim.x) pu[i] = zu[i] + b * pu[i];
        for (int i = threadIdx.x; i < nv; i += blockDim.x) pv[i] = zv[i] + b * pv[i];
        __syncthreads();
    }
}

// Small coarsest level: the velocity block is gathered from the level's
// stencils into a dense matrix (one CTA) and inverted by Gauss-Jordan
// elimination with partial pivoting in FP64 (a zero pivot column sets
// *status).  AinvT is stored column-major so that the solve's threads read it
// coalesced.  Dense numbering: u unknowns (k, l), k in 1..Nx-2, l in 1..Nz-1,
// row by row, then v unknowns (i, j), i in 1..Nx-1, j in 1..Nz-2.
__device__ __forceinline__ int dense_u(int Nx, int Nz, int k, int l) {
    return (k >= 1 && k <= Nx - 2 && l >= 1 && l <= Nz - 1) ? (k - 1) + (l - 1) * (Nx - 2) : -1;
}
__device__ __forceinline__ int dense_v(int Nx, int Nz, int i, int j) {
    return (i >= 1 && i <= Nx - 1 && j >= 1 && j <= Nz - 2) ? (Nx - 2) * (Nz - 1) + (i - 1) + (j - 1) * (Nx - 1) : -1;
}

template <typename T>
__global__ void __launch_bounds__(512) k_coarse_dense_setup(stokes_geom G, const T *__restrict__ su,
                                                            const T *__restrict__ sv, int n,
                                                            const int *__restrict__ map, double *Ag,
                                                            T *__restrict__ AinvT, int *status) {
    // [A | I] in shared memory when it fits (the launch passes the dynamic
    // size), else in the global work array: each of the n elimination steps
    // reads and writes all of it between barriers
    // in the hierarchy's precision: the FP32 hierarchy's inverse is stored in
    // FP32 and only corrects a V-cycle; FP64 elimination runs at a small
    // fraction of the FP32 rate on this part (one CTA: ~300 us per set-up)
    extern __shared__ double dsm[];
    T *A = (size_t)2 * n * n * sizeof(T) <= MG_DENSE_SMEM ? reinterpret_cast<T *>(dsm) : reinterpret_cast<T *>(Ag);
    __shared__ T col[MG_DENSE_MAX];
    __shared__ int bad;
    const int Nx = G.Nx, Nz = G.Nz;
    const size_t nu = (size_t)Nx * (Nz + 1), nv = (size_t)(Nx + 1) * Nz;
    if (threadIdx.x == 0) bad = 0;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) A[e] = T(0);
    __syncthreads();
    for (int r = threadIdx.x; r < n; r += blockDim.x) {
        const int m = map[r];
        if (m < (int)nu) {
            const int k = m % Nx, l = m / Nx;
            for (int q = 0; q < 15; q++) {
                int c = dense_u(Nx, Nz, k + q % 3 - 1, l + q / 3 - 2);
                if (c >= 0) A[(size_t)r * n + c] += su[(size_t)q * nu + m];
            }
            for (int q = 0; q < 16; q++) {
                int c = dense_v(Nx, Nz, k + q % 4 - 1, l + q / 4 - 2);
                if (c >= 0) A[(size_t)r * n + c] += su[(size_t)(15 + q) * nu + m];
            }
        } else {
            const int mv = m - (int)nu, i = mv % (Nx + 1), j = mv / (Nx + 1);
            for (int q = 0; q < 15; q++) {
                int c = dense_v(Nx, Nz, i + q % 5 - 2, j + q / 5 - 1);
                if (c >= 0) A[(size_t)r * n + c] += sv[(size_t)q * nv + mv];
            }
            for (int q = 0; q < 16; q++) {
                int c = dense_u(Nx, Nz, i + q % 4 - 2, j + q / 4 - 1);
                if (c >= 0) A[(size_t)r * n + c] += sv[(size_t)(15 + q) * nv + mv];
            }
        }
    }
    __syncthreads();
    // Gauss-Jordan on [A | I] with partial pivoting (the Newton block is
    // neither symmetric nor definite); B ends as A^-1
    T *B = A + (size_t)n * n;
    __shared__ T red_v[32];
    __shared__ int red_i[32];
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) B[e] = (e / n == e % n) ? T(1) : T(0);
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    for (int k = 0; k < n; k++) {
        T bv = T(-1);
        int bi = k;
        for (int i = k + threadIdx.x; i < n; i += blockDim.x) {
            const T v = fabs(A[(size_t)i * n + k]);
            if (v > bv) { bv = v; bi = i; }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const T ov = __shfl_xor_sync(0xffffffffu, bv, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
        }
        if (lane == 0) { red_v[wid] = bv; red_i[wid] = bi; }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int w = 1; w < nw; w++)
                if (red_v[w] > red_v[0] || (red_v[w] == red_v[0] && red_i[w] < red_i[0])) {
                    red_v[0] = red_v[w];
                    red_i[0] = red_i[w];
                }
        }
        __syncthreads();
        const T pmax = red_v[0];
        const int pr = red_i[0];
        if (!(pmax > T(0)) || !isfinite(pmax)) { if (threadIdx.x == 0) bad = 1; break; }   // uniform
        if (pr != k)
            for (int j = threadIdx.x; j < n; j += blockDim.x) {
                T t = A[(size_t)k * n + j]; A[(size_t)k * n + j] = A[(size_t)pr * n + j]; A[(size_t)pr * n + j] = t;
                t = B[(size_t)k * n + j]; B[(size_t)k * n + j] = B[(size_t)pr * n + j]; B[(size_t)pr * n + j] = t;
            }
        __syncthreads();
        const T inv = T(1) / A[(size_t)k * n + k];
        __syncthreads();
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
            A[(size_t)k * n + j] *= inv;
            B[(size_t)k * n + j] *= inv;
        }
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += blockDim.x) col[i] = A[(size_t)i * n + k];
        __syncthreads();
        for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
            const int i = e / n, j = e % n;
            if (i == k) continue;
            A[(size_t)i * n + j] -= col[i] * A[(size_t)k * n + j];
            B[(size_t)i * n + j] -= col[i] * B[(size_t)k * n + j];
        }
        __syncthreads();
    }
    __syncthreads();
    if (bad) { if (threadIdx.x == 0) *status = 1; return; }
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        int i = e / n, j = e % n;
        AinvT[(size_t)j * n + i] = (T)B[(size_t)i * n + j];
    }
}

// x = A^-1 f on the small coarsest level (zero outside the unknowns)
template <typename T>
__global__ void __launch_bounds__(256) k_coarse_dense_solve(int n, int nu, int nv, const int *__restrict__ map,
                                                            const T *__restrict__ AinvT, const T *__restrict__ fu,
                                                            const T *__restrict__ fv, T *__restrict__ xu,
                                                            T *__restrict__ xv) {
    __shared__ T fs[MG_DENSE_MAX];
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        int m = map[i];
        fs[i] = m < nu ? fu[m] : fv[m - nu];
    }
    for (int i = threadIdx.x; i < nu; i += blockDim.x) xu[i] = T(0);
    for (int i = threadIdx.x; i < nv; i += blockDim.x) xv[i] = T(0);
    __syncthreads();
    for (int r = threadIdx.x; r < n; r += blockDim.x) {
        T s = 0;
        for (int j = 0; j < n; j++) s += AinvT[(size_t)j * n + r] * fs[j];
        int m = map[r];
        if (m < nu) xu[m] = s; else xv[m - nu] = s;
    }
}


// ---------------------------------------------------------------------------
// Bottom of the V-cycle in one thread-block cluster.  The small levels (a few
// thousand points each) cost one launch per sweep, residual and transfer when
// run as grid kernels, and each such launch is several microseconds of
// latency for little work; here the whole descent from level `first` to the
// dense coarsest level and the ascent back run in one launch of one cluster
// (up to 16 CTAs of 1024 threads on 16 SMs; a single CTA where clusters are
// not available), with a cluster barrier between phases.  Same arithmetic
// as the grid kernels (the same point functions), so the result is
// identical.  The first level's result ends in its xu / xv buffers like the
// grid path's.
#define MG_BOTTOM_MAX 6
#define MG_BOTTOM_THREADS 1024
template <typename T>
struct mg_bottom_level {
    stokes_geom G;
    const T *su, *sv, *idu, *idv;
    T *xu, *xv, *yu, *yv, *fu, *fv, *ru, *rv;
};

template <typename T>
struct mg_bottom_args {
    int nlev, nu1, nu2, ndense;   // nlev levels, the last one the dense coarsest
    int lsplit;                   // first level run by CTA 0 alone (nlev: none)
    T omega;
    const int *dmap;
    const T *AinvT;
    mg_bottom_level<T> L[MG_BOTTOM_MAX];
};

// points a bottom launch of `cs` CTAs takes on per level
static inline long long mg_bottom_points(int cs) { return (long long)cs * MG_BOTTOM_THREADS * (cs == 1 ? 4 : 2); }

template <typename T>
__global__ void __launch_bounds__(MG_BOTTOM_THREADS) k_mg_bottom(const __grid_constant__ mg_bottom_args<T> A) {
    __shared__ T fs[MG_DENSE_MAX];
    T *xu[MG_BOTTOM_MAX], *xv[MG_BOTTOM_MAX], *yu[MG_BOTTOM_MAX], *yv[MG_BOTTOM_MAX];
    for (int l = 0; l < A.nlev; l++) { xu[l] = A.L[l].xu; xv[l] = A.L[l].xv; yu[l] = A.L[l].yu; yv[l] = A.L[l].yv; }
    // barrier over every thread of the launch: the grid is one cluster (or one CTA);
    // release / acquire at cluster scope orders the global-memory phases
    auto cbar = [&]() {
        if (gridDim.x > 1) cooperative_groups::this_cluster().sync();
        else __syncthreads();
    };
    auto tbar = [&]() { __syncthreads(); };
    auto swap_xy = [&](int l) {
        T *t = xu[l]; xu[l] = yu[l]; yu[l] = t;
        t = xv[l]; xv[l] = yv[l]; yv[l] = t;
    };
    // one smoothing sweep / residual over a level's rows, one row per thread
    // (u rows, then v rows: twice the threads of a point per thread, so that
    // each phase's critical path is one 31-point row)
    auto smooth_rows = [&](const mg_bottom_level<T> &L, const T *ixu, const T *ixv, T *ou, T *ov, int t0, int nt) {
        const int Nx = L.G.Nx, nuL = Nx * (L.G.Nz + 1), nvL = (Nx + 1) * L.G.Nz;
        for (int r = t0; r < nuL + nvL; r += nt) {
            if (r < nuL) st_smooth_u<T>(L.G, L.su, L.sv, ixu, ixv, L.fu, L.idu, A.omega, ou, r % Nx, r / Nx);
            else st_smooth_v<T>(L.G, L.su, L.sv, ixu, ixv, L.fv, L.idv, A.omega, ov, (r - nuL) % (Nx + 1),
                                (r - nuL) / (Nx + 1));
        }
    };
    auto residual_rows = [&](const mg_bottom_level<T> &L, const T *ixu, const T *ixv, int t0, int nt) {
        const int Nx = L.G.Nx, nuL = Nx * (L.G.Nz + 1), nvL = (Nx + 1) * L.G.Nz;
        for (int r = t0; r < nuL + nvL; r += nt) {
            if (r < nuL) st_residual_u<T>(L.G, L.su, ixu, ixv, L.fu, L.ru, r % Nx, r / Nx);
            else st_residual_v<T>(L.G, L.sv, ixu, ixv, L.fv, L.rv, (r - nuL) % (Nx + 1), (r - nuL) / (Nx + 1));
        }
    };
    // One level's descent (pre-smoothing, residual, restriction) or ascent
    // (prolongation, post-smoothing) by a team of threads t0, t0 + nt, ...
    // (act = false: the thread only keeps its pointer swaps in step) with the
    // team's barrier after each phase.
    auto down = [&](int l, bool act, int t0, int nt, auto &&sync) {
        const mg_bottom_level<T> &L = A.L[l];
        if (act) smooth_rows(L, nullptr, nullptr, xu[l], xv[l], t0, nt);
        sync();
        for (int s = 1; s < A.nu1; s++) {
            if (act) smooth_rows(L, xu[l], xv[l], yu[l], yv[l], t0, nt);
            sync();
            swap_xy(l);
        }
        if (act) residual_rows(L, xu[l], xv[l], t0, nt);
        sync();
        const mg_bottom_level<T> &C = A.L[l + 1];
        const int Wc = C.G.Nx + 1, nptc = Wc * (C.G.Nz + 1);
        for (int p = t0; act && p < nptc; p += nt)
            mg_restrict_pt<T>(L.G, C.G, L.ru, L.rv, C.fu, C.fv, p % Wc, p / Wc);
        sync();
    };
    auto up = [&](int l, bool act, int t0, int nt, auto &&sync) {
        const mg_bottom_level<T> &L = A.L[l];
        const mg_bottom_level<T> &C = A.L[l + 1];
        const int W = L.G.Nx + 1, npt = W * (L.G.Nz + 1);
        for (int p = t0; act && p < npt; p += nt)
            mg_prolong_pt<T>(L.G, C.G, xu[l + 1], xv[l + 1], xu[l], xv[l], p % W, p / W);
        sync();
        for (int s = 0; s < A.nu2; s++) {
            if (act) smooth_rows(L, xu[l], xv[l], yu[l], yv[l], t0, nt);
            sync();
            swap_xy(l);
        }
    };
    auto dense = [&](bool act, int t0, int nt, auto &&sync) {   // x = A^-1 f on the coarsest level
        const int lc = A.nlev - 1, n = A.ndense;
        const mg_bottom_level<T> &C = A.L[lc];
        const int nu = C.G.Nx * (C.G.Nz + 1), nv = (C.G.Nx + 1) * C.G.Nz;
        for (int i = threadIdx.x; act && i < n; i += blockDim.x) {   // every active CTA gathers f for itself
            const int m = A.dmap[i];
            fs[i] = m < nu ? C.fu[m] : C.fv[m - nu];
        }
        for (int i = t0; act && i < nu; i += nt) xu[lc][i] = T(0);
        for (int i = t0; act && i < nv; i += nt) xv[lc][i] = T(0);
        sync();
        for (int r = t0; act && r < n; r += nt) {
            T s = 0;
            for (int j = 0; j < n; j++) s += A.AinvT[(size_t)j * n + r] * fs[j];
            const int m = A.dmap[r];
            if (m < nu) xu[lc][m] = s; else xv[lc][m - nu] = s;
        }
        sync();
    };
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nthr = gridDim.x * blockDim.x;
    // levels lsplit .. nlev-1 are small enough for CTA 0 alone: their phases end
    // in CTA barriers instead of cluster barriers (the other CTAs wait once)
    const int ls = A.lsplit;
    for (int l = 0; l < ls && l < A.nlev - 1; l++) down(l, true, tid, nthr, cbar);
    if (ls < A.nlev) {
        const bool act = blockIdx.x == 0;
        for (int l = ls; l < A.nlev - 1; l++) down(l, act, threadIdx.x, blockDim.x, tbar);
        dense(act, threadIdx.x, blockDim.x, tbar);
        for (int l = A.nlev - 2; l >= ls; l--) up(l, act, threadIdx.x, blockDim.x, tbar);
        cbar();
    } else {
        dense(true, tid, nthr, cbar);
    }
    for (int l = (ls < A.nlev - 1 ? ls : A.nlev - 1) - 1; l >= 0; l--) up(l, true, tid, nthr, cbar);
    if (xu[0] != A.L[0].xu) {   // odd number of swaps on the first level: copy back
        const mg_bottom_level<T> &L = A.L[0];
        const int nu = L.G.Nx * (L.G.Nz + 1), nv = (L.G.Nx + 1) * L.G.Nz;
        for (int i = tid; i < nu; i += nthr) L.xu[i] = xu[0][i];
        for (int i = tid; i < nv; i += nthr) L.xv[i] = xv[0][i];
    }
}

// Largest cluster (16, 8 or 4 CTAs of 1024 threads) the device can place for
// the bottom kernel, else 1 (a single CTA).
template <typename T>
static int mg_bottom_cluster_size() {
    if (cudaFuncSetAttribute(k_mg_bottom<T>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
        cudaGetLastError();
    const int sizes[3] = {16, 8, 4};
    for (int q = 0; q < 3; q++) {
        const int cs = sizes[q];
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(cs);
        cfg.blockDim = dim3(MG_BOTTOM_THREADS);
        cudaLaunchAttribute at;
        at.id = cudaLaunchAttributeClusterDimension;
        at.val.clusterDim.x = cs;
        at.val.clusterDim.y = 1;
        at.val.clusterDim.z = 1;
        cfg.attrs = &at;
        cfg.numAttrs = 1;
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, k_mg_bottom<T>, &cfg) == cudaSuccess && n >= 1) return cs;
        cudaGetLastError();
    }
    return 1;
}

// ---------------------------------------------------------------------------
template <typename T>
static cudaError_t alloc0(T **p, size_t n) {
    cudaError_t e = cudaMalloc((void **)p, sizeof(T) * (n ? n : 1));
    if (e == cudaSuccess) e = cudaMemset(*p, 0, sizeof(T) * (n ? n : 1));
    return e;
}

template <typename T>
static mdz_status build_hierarchy(mdz_ctx *ctx, mg_hier<T> &H) {
    const mdz_dgrid &g = ctx->g;
    int Nx = g.Nx, Nz = g.Nz;
    double dx = g.dx, dz = g.dz;
    cudaError_t e = cudaSuccess;
    int lev = 0;
    while (lev < MG_MAX_LEVELS) {
        mg_level<T> &L = H.L[lev];
        L.Nx = Nx; L.Nz = Nz; L.ncx = Nx - 1; L.ncz = Nz - 1; L.dx = dx; L.dz = dz;
        if (lev == 0) {
            L.BCu = g.BCu; L.BCv = g.BCv; L.BCp = g.BCp; L.BCg = g.BCg; L.own_tags = false;
        } else {
            L.own_tags = true;
            if (e == cudaSuccess) e = alloc0(&L.BCu, L.nu());
            if (e == cudaSuccess) e = alloc0(&L.BCv, L.nv());
            if (e == cudaSuccess) e = alloc0(&L.BCp, (size_t)L.ncx * L.ncz);
            if (e == cudaSuccess) e = alloc0(&L.BCg, (size_t)Nx * Nz);
            if (e == cudaSuccess) {
                k_level_tags<<<mdz_blocks((size_t)(Nx + 1) * (Nz + 1)), MDZ_THREADS>>>(Nx, Nz, L.BCu, L.BCv, L.BCp, L.BCg);
                e = cudaGetLastError();
            }
        }
        if (lev == 0) {
            if (e == cudaSuccess) e = alloc0(&L.D11, (size_t)L.ncx * L.ncz);
            if (e == cudaSuccess) e = alloc0(&L.D33, (size_t)Nx * Nz);
            if (e == cudaSuccess) e = alloc0(&L.pz, (size_t)L.ncx * L.ncz);
            if (e == cudaSuccess) e = alloc0(&H.pmean, 2);
        }
        if (e == cudaSuccess) e = alloc0(&L.su, (size_t)MG_NST * L.nu());
        if (e == cudaSuccess) e = alloc0(&L.sv, (size_t)MG_NST * L.nv());
        T **bufs[] = {&L.xu, &L.yu, &L.fu, &L.ru, &L.idu};
        for (T **b : bufs) if (e == cudaSuccess) e = alloc0(b, L.nu());
        T **bufv[] = {&L.xv, &L.yv, &L.fv, &L.rv, &L.idv};
        for (T **b : bufv) if (e == cudaSuccess) e = alloc0(b, L.nv());
        lev++;
        // halve while both cell counts are even and the coarse level keeps >= 4 cells a side
        bool can = (L.ncx % 2 == 0) && (L.ncz % 2 == 0) && L.ncx / 2 >= 4 && L.ncz / 2 >= 4;
        if (!can) break;
        Nx = L.ncx / 2 + 1; Nz = L.ncz / 2 + 1; dx *= 2; dz *= 2;
    }
    H.nlev = lev;
    mg_level<T> &C = H.L[lev - 1];
    // unknowns of the coarsest level (tag rule of the free-slip box)
    std::vector<int> map;
    for (int l = 1; l <= C.Nz - 1; l++)
        for (int k = 1; k <= C.Nx - 2; k++) map.push_back(k + l * C.Nx);
    for (int l = 1; l <= C.Nz - 2; l++)
        for (int k = 1; k <= C.Nx - 1; k++) map.push_back((int)C.nu() + k + l * (C.Nx + 1));
    if ((int)map.size() <= MG_DENSE_MAX) {
        C.ndense = (int)map.size();
        size_t n2 = (size_t)C.ndense * C.ndense;
        if (e == cudaSuccess) e = alloc0(&C.dmap, map.size());
        if (e == cudaSuccess) e = cudaMemcpy(C.dmap, map.data(), sizeof(int) * map.size(), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = alloc0(&C.Awork, 2 * n2);
        if (e == cudaSuccess) e = alloc0(&C.AinvT, n2);
    } else {
        for (int q = 0; q < 4; q++) {
            if (e == cudaSuccess) e = alloc0(&C.cg[2 * q], C.nu());
            if (e == cudaSuccess) e = alloc0(&C.cg[2 * q + 1], C.nv());
        }
    }
    if (e != cudaSuccess) return mdz_cuda_check(ctx, e, "multigrid allocation");
    return MDZ_OK;
}

template <typename T>
static void free_hierarchy(mg_hier<T> &H) {
    for (int l = 0; l < H.nlev; l++) {
        mg_level<T> &L = H.L[l];
        if (L.own_tags) { cudaFree(L.BCu); cudaFree(L.BCv); cudaFree(L.BCp); cudaFree(L.BCg); }
        void *p[] = {L.D11, L.D33, L.xu, L.xv, L.yu, L.yv, L.fu, L.fv, L.ru, L.rv, L.idu, L.idv,
                     L.cg[0], L.cg[1], L.cg[2], L.cg[3], L.cg[4], L.cg[5], L.cg[6], L.cg[7],
                     L.dmap, L.Awork, L.AinvT, L.su, L.sv, L.pz};
        for (void *q : p) if (q) cudaFree(q);
    }
    if (H.pmean) cudaFree(H.pmean);
    H.pmean = nullptr;
    H.nlev = 0;
}

template <typename T>
static mdz_status alloc_gcr(mdz_ctx *ctx, gcr_space<T> &S, int m) {
    const mdz_dgrid &g = ctx->g;
    S.nu = (size_t)g.Nx * (g.Nz + 1); S.nv = (size_t)(g.Nx + 1) * g.Nz; S.np = (size_t)g.ncx * g.ncz;
    S.n = S.nu + S.nv + S.np;
    S.m = m;
    cudaError_t e = alloc0(&S.Z, S.n * m);
    if (e == cudaSuccess) e = alloc0(&S.W, S.n * m);
    T **v[] = {&S.x, &S.r, &S.z, &S.w, &S.t, &S.pin};
    for (T **b : v) if (e == cudaSuccess) e = alloc0(b, S.n);
    if (e == cudaSuccess) e = cudaMalloc((void **)&S.dA0, sizeof(T *) * (GCR_MAX_M + 4));
    if (e == cudaSuccess) e = cudaMalloc((void **)&S.dA1, sizeof(T *) * (GCR_MAX_M + 4));
    if (e == cudaSuccess) e = cudaMalloc((void **)&S.dA2, sizeof(T *) * (GCR_MAX_M + 4));
    if (e == cudaSuccess) e = alloc0(&S.dots, 8 * (GCR_MAX_M + 8));   // see the layout in gcr_solve
    if (e == cudaSuccess) e = alloc0(&S.tri, (size_t)GCR_MAX_M * GCR_MAX_M + GCR_MAX_M);
    if (e != cudaSuccess) return mdz_cuda_check(ctx, e, "GCR allocation");
    // pointer tables: rows 0..m-1 = W_i, row m = w, row m+1 = r
    std::vector<const T *> a0(m + 2), a1(m + 2), a2(m + 2);
    for (int i = 0; i < m + 2; i++) {
        const T *base = i < m ? S.W + S.n * i : (i == m ? S.w : S.r);
        a0[i] = base; a1[i] = base + S.nu; a2[i] = base + S.nu + S.nv;
    }
    cudaMemcpy(S.dA0, a0.data(), sizeof(T *) * (m + 2), cudaMemcpyHostToDevice);
    cudaMemcpy(S.dA1, a1.data(), sizeof(T *) * (m + 2), cudaMemcpyHostToDevice);
    cudaMemcpy(S.dA2, a2.data(), sizeof(T *) * (m + 2), cudaMemcpyHostToDevice);
    if (sizeof(T) == 4) {
        for (int q = 0; q < 12; q++) {
            size_t n = (q < 8) ? S.np : (size_t)g.Nx * g.Nz;
            if (alloc0(&S.Dc[q], n) != cudaSuccess) return mdz_cuda_check(ctx, cudaGetLastError(), "GCR allocation");
        }
    }
    return MDZ_OK;
}

template <typename T>
static void free_gcr(gcr_space<T> &S) {
    void *p[] = {S.Z, S.W, S.x, S.r, S.z, S.w, S.t, S.pin, S.tri, S.dA0, S.dA1, S.dA2, S.dots};
    for (void *q : p) if (q) cudaFree(q);
    for (int q = 0; q < 12; q++) if (S.Dc[q]) cudaFree(S.Dc[q]);
}

mdz_status mdz_solver_ensure(mdz_ctx *ctx) {
    if (ctx->solver && ctx->solver->ready) return MDZ_OK;
    mdz_status s = mdz_check_stokes_bcs(ctx);
    if (s != MDZ_OK) return s;
    if (!fine_tags_follow_rule(ctx->host_desc))
        return mdz_fail(ctx, MDZ_ERR_UNSUPPORTED, "solver: boundary tags must be the free-slip box pattern");
    if (!ctx->solver) ctx->solver = new mdz_solver();
    mdz_solver *S = ctx->solver;
    if ((s = build_hierarchy<double>(ctx, S->mg64)) != MDZ_OK) return s;
    if ((s = build_hierarchy<float>(ctx, S->mg32)) != MDZ_OK) return s;
    if ((s = alloc_gcr<double>(ctx, S->g64, S->restart)) != MDZ_OK) return s;
    if ((s = alloc_gcr<float>(ctx, S->g32, S->restart)) != MDZ_OK) return s;
    MDZ_CUDA(ctx, cudaMallocHost((void **)&S->sc, 64 * sizeof(double)));
    memset(S->sc, 0, 64 * sizeof(double));
    S->bottom_cs[0] = mg_bottom_cluster_size<double>();
    S->bottom_cs[1] = mg_bottom_cluster_size<float>();
    MDZ_CUDA(ctx, cudaFuncSetAttribute(k_coarse_dense_setup<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       MG_DENSE_SMEM));
    MDZ_CUDA(ctx, cudaFuncSetAttribute(k_coarse_dense_setup<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       MG_DENSE_SMEM));
    MDZ_CUDA(ctx, cudaDeviceSynchronize());
    S->ready = true;
    return MDZ_OK;
}

template <typename T>
static mdz_status copy_stencils(mdz_ctx *ctx, const mg_hier<T> &H, int level, int *Nx, int *Nz, double *su,
                                double *sv) {
    if (level < 0 || level >= H.nlev) return mdz_fail(ctx, MDZ_ERR_ARG, "mg_stencils: level %d of %d", level, H.nlev);
    const mg_level<T> &L = H.L[level];
    *Nx = L.Nx;
    *Nz = L.Nz;
    MDZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const T *src[2] = {L.su, L.sv};
    double *dst[2] = {su, sv};
    size_t cnt[2] = {MG_NST * L.nu(), MG_NST * L.nv()};
    for (int q = 0; q < 2; q++) {
        if (!dst[q]) continue;
        std::vector<T> h(cnt[q]);
        MDZ_CUDA(ctx, cudaMemcpy(h.data(), src[q], sizeof(T) * cnt[q], cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < cnt[q]; i++) dst[q][i] = (double)h[i];
    }
    return MDZ_OK;
}

extern "C" mdz_status mdz_mg_stencils(mdz_ctx *ctx, int precision, int level, int *levels, int *Nx, int *Nz,
                                      double *su, double *sv) {
    if (!ctx || !Nx || !Nz || !levels) return ctx ? mdz_fail(ctx, MDZ_ERR_ARG, "mg_stencils: null argument") : MDZ_ERR_ARG;
    if (!ctx->solver || !ctx->solver->ready)
        return mdz_fail(ctx, MDZ_ERR_STATE, "mg_stencils: no multigrid hierarchy (run a solve first)");
    if (precision == 64) {
        *levels = ctx->solver->mg64.nlev;
        return copy_stencils<double>(ctx, ctx->solver->mg64, level, Nx, Nz, su, sv);
    }
    if (precision == 32) {
        *levels = ctx->solver->mg32.nlev;
        return copy_stencils<float>(ctx, ctx->solver->mg32, level, Nx, Nz, su, sv);
    }
    return mdz_fail(ctx, MDZ_ERR_ARG, "mg_stencils: precision 64 or 32");
}

extern "C" mdz_status mdz_set_solver_options(mdz_ctx *ctx, int nu1, int nu2, double omega, int restart, int check,
                                             int mg_jacobian) {
    if (!ctx) return MDZ_ERR_ARG;
    if (nu1 < 1 || nu1 > 16 || nu2 < 0 || nu2 > 16 || !(omega > 0.0 && omega < 2.0) || restart < 2 ||
        restart > GCR_MAX_M || check < 1 || check > 64 || (mg_jacobian != 0 && mg_jacobian != 1))
        return mdz_fail(ctx, MDZ_ERR_ARG, "solver options: nu1 1..16, nu2 0..16, omega in (0, 2), restart 2..%d, "
                                          "check 1..64, mg_jacobian 0/1", GCR_MAX_M);
    if (!ctx->solver) ctx->solver = new mdz_solver();
    mdz_solver *S = ctx->solver;
    MDZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int q = 0; q < MDZ_PRE_SLOTS; q++)
        if (S->pre[q]) { cudaGraphExecDestroy(S->pre[q]); S->pre[q] = nullptr; }
    S->nu1 = nu1; S->nu2 = nu2; S->omega = omega; S->check = check; S->mg_jacobian = mg_jacobian;
    if (S->ready && restart != S->restart) {
        free_gcr(S->g64);
        free_gcr(S->g32);
        S->g64 = gcr_space<double>();
        S->g32 = gcr_space<float>();
        S->restart = restart;
        mdz_status s;
        if ((s = alloc_gcr<double>(ctx, S->g64, restart)) != MDZ_OK) return s;
        if ((s = alloc_gcr<float>(ctx, S->g32, restart)) != MDZ_OK) return s;
    }
    S->restart = restart;
    return MDZ_OK;
}

extern "C" mdz_status mdz_set_schur_scaling(mdz_ctx *ctx, int mode) {
    if (!ctx) return MDZ_ERR_ARG;
    if (mode != 0 && mode != 1) return mdz_fail(ctx, MDZ_ERR_ARG, "Schur scaling: mode 0 or 1");
    if (!ctx->solver) ctx->solver = new mdz_solver();
    ctx->solver->schur = mode;   // graphs of both kinds have their own slots
    return MDZ_OK;
}

// The grid spacing changed (PureShearALE): every level's spacing follows the
// fine one (doubling per level, as the hierarchy was built) and the captured
// preconditioner graphs, which hold the old spacings as kernel arguments, are
// dropped (recaptured on their next use).
mdz_status mdz_solver_regrid(mdz_ctx *ctx) {
    mdz_solver *S = ctx->solver;
    if (!S) return MDZ_OK;
    MDZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int q = 0; q < MDZ_PRE_SLOTS; q++)
        if (S->pre[q]) { cudaGraphExecDestroy(S->pre[q]); S->pre[q] = nullptr; S->pre_eta[q] = nullptr; }
    S->mg64.built = false;   // no solve may keep operators of the old spacing
    S->mg32.built = false;
    double dx = ctx->g.dx, dz = ctx->g.dz;
    for (int lev = 0; lev < S->mg64.nlev; lev++, dx *= 2, dz *= 2) { S->mg64.L[lev].dx = dx; S->mg64.L[lev].dz = dz; }
    dx = ctx->g.dx; dz = ctx->g.dz;
    for (int lev = 0; lev < S->mg32.nlev; lev++, dx *= 2, dz *= 2) { S->mg32.L[lev].dx = dx; S->mg32.L[lev].dz = dz; }
    return MDZ_OK;
}

void mdz_solver_free(mdz_ctx *ctx) {
    if (!ctx->solver) return;
    mdz_solver *S = ctx->solver;
    for (int q = 0; q < MDZ_PRE_SLOTS; q++)
        if (S->pre[q]) cudaGraphExecDestroy(S->pre[q]);
    free_hierarchy(S->mg64);
    free_hierarchy(S->mg32);
    free_gcr(S->g64);
    free_gcr(S->g32);
    if (S->sc) cudaFreeHost(S->sc);
    delete S;
    ctx->solver = nullptr;
}

int mdz_solver_levels(const mdz_ctx *ctx) { return ctx->solver ? ctx->solver->mg64.nlev : 0; }

// ---------------------------------------------------------------------------
// Multigrid setup (coefficients) and V-cycle.
template <typename T>
static mdz_status mg_setup(mdz_ctx *ctx, mg_hier<T> &H, const double *eta_n, const double *eta_s,
                           const stokes_coefs<T> &K, bool newton, cudaStream_t st) {
    mg_level<T> &F = H.L[0];
    int nc = F.ncx * F.ncz, nv = F.Nx * F.Nz;
    H.newton = newton;
    H.built = true;
    cudaEvent_t ev;
    mdz_prof_begin(ctx, MDZ_PROF_MG_SETUP, st, &ev);
    k_fill_D11_D33<T><<<mdz_blocks(nv > nc ? nv : nc), MDZ_THREADS, 0, st>>>(nc, nv, eta_n, eta_s, F.D11, F.D33);
    MDZ_LAUNCHED(ctx);
    // level-0 stencils: the Picard block written out from eta, or the Newton
    // Jacobian's velocity block probed with 2 x 16 colour classes
    const dim3 bl(32, 8), gr0((F.Nx + 1 + 31) / 32, (F.Nz + 1 + 7) / 8);
    if (!newton) {
        k_picard_stencil<T><<<gr0, bl, 0, st>>>(F.geom(), F.D11, F.D33, F.su, F.sv);
        MDZ_LAUNCHED(ctx);
    } else {
    MDZ_CUDA(ctx, cudaMemsetAsync(F.su, 0, sizeof(T) * MG_NST * F.nu(), st));
    MDZ_CUDA(ctx, cudaMemsetAsync(F.sv, 0, sizeof(T) * MG_NST * F.nv(), st));
    for (int comp = 0; comp < 2; comp++)
        for (int cz = 0; cz < MG_PROBE; cz++)
            for (int cx = 0; cx < MG_PROBE; cx++) {
                k_probe_vec<T><<<gr0, bl, 0, st>>>(F.geom(), comp, cx, cz, F.xu, F.xv);
                MDZ_LAUNCHED(ctx);
                if (newton) k_mg_apply<T, true><<<gr0, bl, 0, st>>>(F.geom(), K, F.xu, F.xv, F.pz, F.ru, F.rv);
                else k_mg_apply<T, false><<<gr0, bl, 0, st>>>(F.geom(), F.coefs(), F.xu, F.xv, nullptr, F.ru, F.rv);
                MDZ_LAUNCHED(ctx);
                k_probe_collect<T><<<gr0, bl, 0, st>>>(F.geom(), comp, cx, cz, F.ru, F.rv, F.su, F.sv);
                MDZ_LAUNCHED(ctx);
            }
    }
    {   // Jacobi diagonal of level 0: the viscosity formula (Picard) or the probed stencil (Newton)
        size_t n = F.nu() > F.nv() ? F.nu() : F.nv();
        if (newton) k_st_diag<T><<<mdz_blocks(n), MDZ_THREADS, 0, st>>>(F.geom(), F.su, F.sv, F.idu, F.idv);
        else k_mg_diag<T><<<mdz_blocks(n), MDZ_THREADS, 0, st>>>(F.geom(), F.D11, F.D33, F.idu, F.idv);
        MDZ_LAUNCHED(ctx);
    }
    int *status = ctx->d_counters + 40;   // [0] coarse inverse, [1] Galerkin footprint
    MDZ_CUDA(ctx, cudaMemsetAsync(status, 0, 2 * sizeof(int), st));
    for (int l = 1; l < H.nlev; l++) {
        mg_level<T> &P = H.L[l - 1], &L = H.L[l];
        size_t n = L.nu() > L.nv() ? L.nu() : L.nv();
        k_galerkin<T><<<mdz_blocks((long long)n * GAL_SPLIT, GAL_THREADS), GAL_THREADS, 0, st>>>(P.geom(), P.su, P.sv, L.geom(), L.su, L.sv, status + 1);
        MDZ_LAUNCHED(ctx);
        k_st_diag<T><<<mdz_blocks(n), MDZ_THREADS, 0, st>>>(L.geom(), L.su, L.sv, L.idu, L.idv);
        MDZ_LAUNCHED(ctx);
    }
    mg_level<T> &C = H.L[H.nlev - 1];
    if (C.ndense) {
        const size_t smem = (size_t)2 * C.ndense * C.ndense * sizeof(T);
        k_coarse_dense_setup<T><<<1, 512, smem <= MG_DENSE_SMEM ? smem : 0, st>>>(C.geom(), C.su, C.sv, C.ndense,
                                                                              C.dmap, C.Awork, C.AinvT, status);
        MDZ_LAUNCHED(ctx);
    }
    {   // algorithmic bytes: viscosities in, D11 / D33 out; level-0 stencils
        // written once; each Galerkin level reads the finer stencils once and
        // writes its own plus the inverse diagonal
        double b = 8.0 * (nc + nv) + sizeof(T) * (nc + nv) + sizeof(T) * MG_NST * (double)(F.nu() + F.nv());
        for (int l = 1; l < H.nlev; l++)
            b += sizeof(T) * (MG_NST * (double)(H.L[l - 1].nu() + H.L[l - 1].nv()) +
                              (MG_NST + 1.0) * (double)(H.L[l].nu() + H.L[l].nv()));
        mdz_prof_end(ctx, MDZ_PROF_MG_SETUP, b, st, ev);
    }
    MDZ_CUDA(ctx, cudaMemcpyAsync((int *)(ctx->solver->sc + 20), status, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
    return MDZ_OK;
}

static inline dim3 box_grid(int Nx, int Nz) { return dim3((Nx + 1 + 31) / 32, (Nz + 1 + 7) / 8); }

// Whether vcycle() smooths level l with its own sweeps (not the dense
// coarsest solve, the coarse CG, nor the one-launch bottom kernel).
template <typename T>
static bool vcycle_smoothed(const mdz_ctx *ctx, const mg_hier<T> &H, int l) {
    const mg_level<T> &L = H.L[l];
    if (l == H.nlev - 1) return false;
    const bool viscous = l == 0 && !H.newton;
    const mg_level<T> &Cd = H.L[H.nlev - 1];
    const int cs = ctx->solver->bottom_cs[sizeof(T) == 8 ? 0 : 1];
    return !(!viscous && Cd.ndense && H.nlev - l <= MG_BOTTOM_MAX &&
             (long long)(L.Nx + 1) * (L.Nz + 1) <= mg_bottom_points(cs));
}

// One V-cycle: H.L[l].x <- approx A^-1 H.L[l].f.  Level 0 smooths with the
// re-discretised stencil (viscosities read directly), coarser levels with the
// Galerkin stencils.  x0_done: the first sweep from x = 0 (x = omega D^-1 f)
// was already written into L.xu / L.xv with the right-hand side
// (k_precond_rhs); out_u / out_v: where the last post-smoothing sweep writes
// (the caller's vector), else the level's own buffers.  Both only for a level
// that vcycle_smoothed() accepts.
template <typename T>
static mdz_status vcycle(mdz_ctx *ctx, mg_hier<T> &H, int l, int nu1, int nu2, T omega, cudaStream_t st,
                         bool x0_done = false, T *out_u = nullptr, T *out_v = nullptr) {
    mg_level<T> &L = H.L[l];
    stokes_geom G = L.geom();
    stokes_coefs<T> D = L.coefs();
    dim3 bl(32, 8), gr = box_grid(L.Nx, L.Nz);
    if (l == H.nlev - 1 && L.ndense) {
        k_coarse_dense_solve<T><<<1, 256, 0, st>>>(L.ndense, (int)L.nu(), (int)L.nv(), L.dmap, L.AinvT, L.fu, L.fv,
                                                   L.xu, L.xv);
        MDZ_LAUNCHED(ctx);
        return MDZ_OK;
    }
    if (l == H.nlev - 1) {
        int maxit = 4 * (L.ncx > L.ncz ? L.ncx : L.ncz) + 50;
        k_mg_coarse_cg<T><<<1, 1024, 0, st>>>(G, L.su, L.sv, L.fu, L.fv, L.idu, L.idv, L.xu, L.xv, L.ru, L.rv,
                                              L.cg[0], L.cg[1], L.cg[2], L.cg[3], L.cg[4], L.cg[5], maxit, 1e-6);
        MDZ_LAUNCHED(ctx);
        return MDZ_OK;
    }
    const bool viscous = l == 0 && !H.newton;   // level 0 of a Picard hierarchy: stencil from eta directly
    const mg_level<T> &Cd = H.L[H.nlev - 1];
    const int cs = ctx->solver->bottom_cs[sizeof(T) == 8 ? 0 : 1];
    if (!viscous && Cd.ndense && H.nlev - l <= MG_BOTTOM_MAX &&
        (long long)(L.Nx + 1) * (L.Nz + 1) <= mg_bottom_points(cs)) {   // this level and all below in one launch
        mg_bottom_args<T> A;
        A.nlev = H.nlev - l; A.nu1 = nu1; A.nu2 = nu2; A.ndense = Cd.ndense; A.omega = omega;
        A.lsplit = A.nlev;
        for (int q = 0; q < A.nlev; q++)   // levels of at most one point per thread of one CTA
            if ((long long)(H.L[l + q].Nx + 1) * (H.L[l + q].Nz + 1) <= MG_BOTTOM_THREADS) { A.lsplit = q; break; }
        A.dmap = Cd.dmap; A.AinvT = Cd.AinvT;
        for (int q = 0; q < A.nlev; q++) {
            const mg_level<T> &B = H.L[l + q];
            A.L[q] = mg_bottom_level<T>{B.geom(), B.su, B.sv, B.idu, B.idv, B.xu, B.xv, B.yu, B.yv,
                                        B.fu, B.fv, B.ru, B.rv};
        }
        if (cs > 1) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(cs);
            cfg.blockDim = dim3(MG_BOTTOM_THREADS);
            cfg.stream = st;
            cudaLaunchAttribute at;
            at.id = cudaLaunchAttributeClusterDimension;
            at.val.clusterDim.x = cs;
            at.val.clusterDim.y = 1;
            at.val.clusterDim.z = 1;
            cfg.attrs = &at;
            cfg.numAttrs = 1;
            MDZ_CUDA(ctx, cudaLaunchKernelEx(&cfg, k_mg_bottom<T>, A));
        } else {
            k_mg_bottom<T><<<1, MG_BOTTOM_THREADS, 0, st>>>(A);
        }
        MDZ_LAUNCHED(ctx);
        return MDZ_OK;
    }
    const int rows_grid = mdz_blocks(L.nu() + L.nv(), 128);
    auto smooth = [&](const T *xu, const T *xv, T *ou, T *ov) {
        if (viscous) k_mg_smooth<T><<<gr, bl, 0, st>>>(G, D, xu, xv, L.fu, L.fv, L.idu, L.idv, omega, ou, ov);
        else k_st_smooth<T><<<rows_grid, 128, 0, st>>>(G, L.su, L.sv, xu, xv, L.fu, L.fv, L.idu, L.idv, omega, ou, ov);
    };
    // pre-smoothing from x = 0
    if (!x0_done) {
        smooth(nullptr, nullptr, L.xu, L.xv);
        MDZ_LAUNCHED(ctx);
    }
    for (int s = 1; s < nu1; s++) {
        smooth(L.xu, L.xv, L.yu, L.yv);
        MDZ_LAUNCHED(ctx);
        std::swap(L.xu, L.yu); std::swap(L.xv, L.yv);
    }
    if (viscous) k_mg_residual<T><<<gr, bl, 0, st>>>(G, D, L.xu, L.xv, L.fu, L.fv, L.ru, L.rv);
    else k_st_residual<T><<<rows_grid, 128, 0, st>>>(G, L.su, L.sv, L.xu, L.xv, L.fu, L.fv, L.ru, L.rv);
    MDZ_LAUNCHED(ctx);
    mg_level<T> &C = H.L[l + 1];
    k_mg_restrict<T><<<box_grid(C.Nx, C.Nz), bl, 0, st>>>(G, C.geom(), L.ru, L.rv, C.fu, C.fv);
    MDZ_LAUNCHED(ctx);
    mdz_status s = vcycle<T>(ctx, H, l + 1, nu1, nu2, omega, st);
    if (s != MDZ_OK) return s;
    k_mg_prolong_add<T><<<gr, bl, 0, st>>>(G, C.geom(), C.xu, C.xv, L.xu, L.xv);
    MDZ_LAUNCHED(ctx);
    for (int q = 0; q < nu2; q++) {
        if (q == nu2 - 1 && out_u) {   // the last sweep straight into the caller's vector
            smooth(L.xu, L.xv, out_u, out_v);
            MDZ_LAUNCHED(ctx);
            break;
        }
        smooth(L.xu, L.xv, L.yu, L.yv);
        MDZ_LAUNCHED(ctx);
        std::swap(L.xu, L.yu); std::swap(L.xv, L.yv);
    }
    return MDZ_OK;
}

// ---------------------------------------------------------------------------
// Pressure mean over the pressure equations (sum, count) and its removal.
// (sum in the vector's precision and an integer count per thread, warp sums
// in that precision, then a fixed-order FP64 sum of the block partials:
// reduce.cuh)
template <typename T>
__global__ void __launch_bounds__(256) k_psum(int np, const signed char *__restrict__ tp, const T *__restrict__ p,
                                              double *part, unsigned int *counter, double *out) {
    T acc = 0;
    int cnt = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x)
        if (tp[i] == -1) { acc += p[i]; cnt++; }
    const T v[2] = {acc, (T)cnt};   // (counts per thread are small integers: exact in T)
    mdz_grid_sum<2, T>(v, part, counter, out);
}

// (the mean in the vector's precision: an FP64 division per thread is a long
// instruction sequence on this part)
template <typename T>
__global__ void k_psub(int np, const signed char *__restrict__ tp, const double *__restrict__ sum, T *__restrict__ p) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < np && tp[i] == -1 && sum[1] > 0) p[i] -= (T)sum[0] / (T)sum[1];
}

// ---------------------------------------------------------------------------
// Block preconditioner: zp = (eta_n / celvol) rp ; zu = V-cycle(ru - B zp).
// (eta_n / celvol from the level-0 copy D11 = 2 eta_n in precision T), and
// the sum and count of zp over the pressure equations (as k_psum) for the
// zero-mean projection applied by k_copy_out
template <typename T>
__global__ void __launch_bounds__(256) k_precond_p(stokes_geom G, const T *__restrict__ D11, const T *__restrict__ Dt,
                                                   const T *__restrict__ rp, T *__restrict__ zp, double *part,
                                                   unsigned int *counter, double *psum) {
    const int np = G.ncx * G.ncz;
    const T c = T(0.5) * gc<T>(G, GC_IXZ);
    T acc = 0;
    int cnt = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
        T v = 0;
        if (G.BCp[i] == -1) {
            T d = D11[i];
            if (Dt) {   // the Jacobian's tangent D11 where it is positive
                const T t = Dt[i];
                if (t > T(0)) d = t;
            }
            v = c * d * rp[i];
            acc += v;
            cnt++;
        }
        zp[i] = v;
    }
    const T v[2] = {acc, (T)cnt};
    mdz_grid_sum<2, T>(v, part, counter, psum);
}

// f = r_vel - B zp  on the fine MG level (B: celvol-scaled pressure gradient);
// with xu non-null also the V-cycle's first sweep from x = 0, x = omega D^-1 f
// (the smoother's own arithmetic for a zero x), in the same pass
template <typename T>
__global__ void k_precond_rhs(stokes_geom G, const T *__restrict__ ru, const T *__restrict__ rv,
                              const T *__restrict__ zp, T *__restrict__ fu, T *__restrict__ fv,
                              const T *__restrict__ idu, const T *__restrict__ idv, T omega, T *__restrict__ xu,
                              T *__restrict__ xv) {
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int Nx = G.Nx, Nz = G.Nz, ncx = G.ncx;
    if (i < Nx && j <= Nz) {
        int c = i + j * Nx;
        T r = 0, x0 = 0;
        if (G.BCu[c] == -1) {
            int c2 = i - 1 + (j - 1) * ncx;
            r = ru[c] - gc<T>(G, GC_DZ) * (zp[c2 + 1] - zp[c2]);
            if (xu) x0 = T(0) + omega * idu[c] * (r - T(0));
        }
        fu[c] = r;
        if (xu) xu[c] = x0;
    }
    if (i <= Nx && j < Nz) {
        int c = i + j * (Nx + 1);
        T r = 0, x0 = 0;
        if (G.BCv[c] == -1) {
            int c2 = i - 1 + (j - 1) * ncx;
            r = rv[c] - gc<T>(G, GC_DX) * (zp[c2 + ncx] - zp[c2]);
            if (xv) x0 = T(0) + omega * idv[c] * (r - T(0));
        }
        fv[c] = r;
        if (xv) xv[c] = x0;
    }
}

// z pressure <- zero mean over the pressure equations (the mean cancels in
// the gradient of the right-hand side, so it is removed only here)
template <typename T>
__global__ void k_pmean_out(int np, const signed char *__restrict__ tp, const double *__restrict__ psum,
                            T *__restrict__ zp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < np && tp[i] == -1 && psum[1] > 0) zp[i] -= (T)psum[0] / (T)psum[1];
}

// z velocity <- the V-cycle's result; z pressure <- zero mean over the
// pressure equations (the mean cancels in the gradient of the right-hand side,
// so it is removed only here)
template <typename T>
__global__ void k_copy_out(size_t nu, size_t nv, int np, const T *__restrict__ xu, const T *__restrict__ xv,
                           const signed char *__restrict__ tp, const double *__restrict__ psum, T *__restrict__ zu,
                           T *__restrict__ zv, T *__restrict__ zp) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nu) zu[i] = xu[i];
    if (i < nv) zv[i] = xv[i];
    if (i < (size_t)np && tp[i] == -1 && psum[1] > 0) zp[i] -= (T)psum[0] / (T)psum[1];
}

template <typename T>
static mdz_status precondition(mdz_ctx *ctx, mg_hier<T> &H, const double *eta_n, const T *Dt, const T *r, T *z,
                               size_t nu, size_t nv, cudaStream_t st) {
    mg_level<T> &F = H.L[0];
    stokes_geom G = F.geom();
    const int np = F.ncx * F.ncz;
    // zero-mean pressure block: constants are the operator's null space; left
    // in, they grow in the iterates and cost the FP32 gradients their accuracy
    {
        int blocks = mdz_blocks(np, 256);
        if (blocks > 152 * 4) blocks = 152 * 4;
        k_precond_p<T><<<blocks, 256, 0, st>>>(G, F.D11, Dt, r + nu + nv, z + nu + nv, ctx->red_part + MDZ_RP_PRECP,
                                               ctx->red_cnt + MDZ_RC_PRECP, H.pmean);
        MDZ_LAUNCHED(ctx);
    }
    mdz_solver *S = ctx->solver;
    // a level-0 V-cycle of its own sweeps takes its first sweep from the
    // right-hand side kernel and writes its last sweep into z
    const bool fused = vcycle_smoothed<T>(ctx, H, 0) && S->nu2 > 0;
    k_precond_rhs<T><<<box_grid(F.Nx, F.Nz), dim3(32, 8), 0, st>>>(G, r, r + nu, z + nu + nv, F.fu, F.fv, F.idu,
                                                                  F.idv, (T)S->omega, fused ? F.xu : nullptr,
                                                                  fused ? F.xv : nullptr);
    MDZ_LAUNCHED(ctx);
    mdz_status s = vcycle<T>(ctx, H, 0, S->nu1, S->nu2, (T)S->omega, st, fused, fused ? z : nullptr,
                             fused ? z + nu : nullptr);
    if (s != MDZ_OK) return s;
    if (fused) {
        k_pmean_out<T><<<mdz_blocks(np), MDZ_THREADS, 0, st>>>(np, G.BCp, H.pmean, z + nu + nv);
    } else {
        size_t n = nu > nv ? nu : nv;
        if ((size_t)np > n) n = np;
        k_copy_out<T><<<mdz_blocks(n), MDZ_THREADS, 0, st>>>(nu, nv, np, F.xu, F.xv, G.BCp, H.pmean, z, z + nu,
                                                             z + nu + nv);
    }
    MDZ_LAUNCHED(ctx);
    return MDZ_OK;
}

// ---------------------------------------------------------------------------
// GCR kernels (vectors are u|v|p contiguous of length n).
// Orthogonalisation: classical Gram-Schmidt, with a second pass only where
// the first removed all but 1e-3 (FP64 basis) or 1e-1 (FP32 basis) of w's
// squared norm (a DGKS-type test; with the usual 1/2 the second pass ran in
// almost every FP32 iteration and made the plain FP64 solve 7 % slower for
// the same iteration counts; 1e-3 on FP32 bases cost 15-25 % more iterations
// on a 401^2 visco-elasto-plastic box),
// decided on the device: the first pass's k_gcr_dots sets sc[5] = 1 for a
// second pass, and the second-pass kernels return at once when it is 0.
// dots[0..k-1] = (w, W_q), dots[k] = (w, w), dots[k+1] = (w, r) of the pass
// whose coefficients the finish applies; sc[0] = 1/||w||, sc[1] = alpha,
// sc[2] = ||w||^2, sc[3] = running ||r||^2 (so the host reads it only every
// few iterations).
__device__ void gcr_scalars(int k, const double *d, double *sc, double *tri, bool second) {
    // column k of U: the pass's Gram-Schmidt coefficients (added to the first
    // pass's after a second pass) and the new direction's norm
    double *U = tri + (size_t)k * GCR_MAX_M;
    double nrm2 = d[k], wr = d[k + 1];
    for (int q = 0; q < k; q++) {
        nrm2 -= d[q] * d[q];
        wr -= d[q] * sc[8 + q];   // (w - sum beta_q W_q, r0) = (w, r0) - sum beta_q alpha_q
        U[q] = second ? U[q] + d[q] : d[q];
    }
    double nrm = sqrt(nrm2 > 0 ? nrm2 : 0.0);
    double alpha = nrm > 0 ? wr / nrm : 0.0;   // alpha_k = (W_k, r0) = (W_k, r_k): W orthonormal
    U[k] = nrm;
    sc[0] = nrm > 0 ? 1.0 / nrm : 0.0;
    sc[1] = alpha;
    sc[2] = nrm2;
    sc[3] -= alpha * alpha;   // ||r_k||^2 = ||r_k-1||^2 - alpha_k^2
    sc[8 + k] = alpha;
}

// gamma = U^-1 alpha (back substitution, one thread): x = x0 + Z gamma with
// the raw preconditioned vectors Z, whose orthogonalised combinations
// Z U^-1 are the directions whose images are the orthonormal W
__global__ void k_gcr_gamma(int k, const double *__restrict__ sc, double *__restrict__ tri) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double *g = tri + (size_t)GCR_MAX_M * GCR_MAX_M;
    for (int i = k - 1; i >= 0; i--) {
        double v = sc[8 + i];
        for (int j = i + 1; j < k; j++) v -= tri[(size_t)j * GCR_MAX_M + i] * g[j];
        const double dgl = tri[(size_t)i * GCR_MAX_M + i];
        g[i] = dgl != 0.0 ? v / dgl : 0.0;
    }
}

// first-pass correction w -= sum beta_q W_q, only when sc[5] asks for a
// second pass (grid-stride, so a skipped launch is short)
template <typename P>
__global__ void k_gcr_orth_if(size_t n, int k, const P *__restrict__ W, const double *__restrict__ beta,
                              const double *__restrict__ sc, P *__restrict__ w) {
    if (sc[5] == 0.0) return;
    __shared__ P bsh[GCR_MAX_M];
    for (int q = threadIdx.x; q < k; q += blockDim.x) bsh[q] = (P)beta[q];
    __syncthreads();
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        P ws = w[i];
        for (int q = 0; q < k; q++) ws -= bsh[q] * W[q * n + i];
        w[i] = ws;
    }
}

__global__ void k_set_scalar(double *dst, const double *src) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *dst = *src;
}

// W_k = (w - sum beta_q W_q) / ||.||, Z_k = z (the raw preconditioned
// vector) and the preconditioner's next input W_k, in precision P.  The
// residual is not touched per iteration: alpha_k = (W_k, r0) and the
// running norm are scalars (gcr_scalars), and r = r0 - sum alpha_q W_q is
// formed once per basis (k_gcr_rupdate), as is x (k_gcr_xupdate).  Per
// iteration this reads the basis W twice (the sums and here) and nothing of
// Z: about 2k + 7 vectors against 3k + 11 for the form that orthogonalised
// z and updated r every iteration.
template <typename P>
__global__ void k_gcr_finish(size_t n, int k, P *__restrict__ W, P *__restrict__ Z, const double *__restrict__ dots1,
                             const double *__restrict__ dots2, const double *__restrict__ sc,
                             const P *__restrict__ z, const P *__restrict__ w, P *__restrict__ pin,
                             double *__restrict__ next1, double *__restrict__ next2) {
    // the next iteration accumulates into the other parity's buffers, which
    // no kernel of this iteration reads: clear them here instead of by memsets
    if (blockIdx.x == 0 && next1)
        for (int q = threadIdx.x; q < k + 3; q += blockDim.x) { next1[q] = 0.0; next2[q] = 0.0; }
    __shared__ P bsh[GCR_MAX_M];
    const double *__restrict__ beta = sc[5] != 0.0 ? dots2 : dots1;
    for (int q = threadIdx.x; q < k; q += blockDim.x) bsh[q] = (P)beta[q];
    __syncthreads();
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    P ws = w[i];
    for (int q = 0; q < k; q++) ws -= bsh[q] * W[q * n + i];
    ws *= (P)sc[0];
    W[(size_t)k * n + i] = ws;
    pin[i] = ws;
    Z[(size_t)k * n + i] = z[i];
}

// r = r - sum alpha_q W_q over the basis (end of a basis); the P copy of the
// new r0 for the sums (rp, the FP32 form) and the preconditioner's input
template <typename P, typename T>
__global__ void k_gcr_rupdate(size_t n, int k, const P *__restrict__ W, const double *__restrict__ sc,
                              T *__restrict__ r, P *__restrict__ rp, P *__restrict__ pin) {
    __shared__ P ash[GCR_MAX_M];
    for (int q = threadIdx.x; q < k; q += blockDim.x) ash[q] = (P)sc[8 + q];
    __syncthreads();
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    P a = 0;
    for (int q = 0; q < k; q++) a += ash[q] * W[q * n + i];
    const T rn = (T)((double)r[i] - (double)a);
    r[i] = rn;
    if (rp) rp[i] = (P)rn;
    pin[i] = (P)rn;
}

// start of the solve: the P copy of r0 (FP32 form) and the first input
template <typename P, typename T>
__global__ void k_gcr_start(size_t n, const T *__restrict__ r, P *__restrict__ rp, P *__restrict__ pin) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const P v = (P)r[i];
    if (rp) rp[i] = v;
    pin[i] = v;
}

// x += sum_{q < k} gamma_q Z_q (gamma = U^-1 alpha, k_gcr_gamma): the basis
// part of the iterate, once per basis (at a restart and at the end)
template <typename P, typename T>
__global__ void k_gcr_xupdate(size_t n, int k, const P *__restrict__ Z, const double *__restrict__ gamma,
                              T *__restrict__ x) {
    __shared__ P ash[GCR_MAX_M];
    for (int q = threadIdx.x; q < k; q += blockDim.x) ash[q] = (P)gamma[q];
    __syncthreads();
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    P a = 0;
    for (int q = 0; q < k; q++) a += ash[q] * Z[q * n + i];
    x[i] = (T)((double)x[i] + (double)a);
}

// out[0] += (w, w), out[1] += (w, r): products, sums and the block reduction
// in the vectors' precision, block totals added in FP64 (as k_dots); a
// non-null flag holding 0 makes the launch a no-op

template <typename T>
__global__ void k_axpby(size_t n, double a, const T *__restrict__ x, double b, T *__restrict__ y) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = (T)(a * (double)x[i] + b * (double)y[i]);
}

template <typename Tin, typename Tout>
__global__ void k_convert(size_t n, const Tin *__restrict__ a, Tout *__restrict__ b) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (Tout)a[i];
}

// Pressure gauge: the decoupled operator annihilates a constant pressure, but
// the rheology does not (pressure-dependent yield), so every correction is
// returned with zero mean over the pressure equations.

static mdz_status remove_pressure_mean(mdz_ctx *ctx, double *p, cudaStream_t st) {
    const mdz_dgrid &g = ctx->g;
    int np = g.ncx * g.ncz;
    double *d = (double *)(ctx->d_counters + 24);
    int blocks = mdz_blocks(np, 256);
    if (blocks > 152 * 4) blocks = 152 * 4;
    k_psum<double><<<blocks, 256, 0, st>>>(np, g.BCp, p, ctx->red_part + MDZ_RP_PSUM, ctx->red_cnt + MDZ_RC_PSUM, d);
    MDZ_LAUNCHED(ctx);
    k_psub<double><<<mdz_blocks(np), MDZ_THREADS, 0, st>>>(np, g.BCp, d, p);
    MDZ_LAUNCHED(ctx);
    return MDZ_OK;
}

// out[q] = (a_q, b) for the nq vectors of the pointer table (each of length
// n, contiguous u|v|p like b).  FP32 vectors: one thread keeps Q = 8 running
// sums, so b is read once per 8 vectors and the loads of 8 independent chains
// overlap, and products, sums and the warp reductions stay FP32 with only the
// warp sums entering FP64 (FP64 instructions issue at a small fraction of
// the FP32 rate on this part, so even a per-thread FP64 reduction tree
// dominated the kernel).  FP64 vectors: Q = 1, one vector per block row (the
// per-element FP64 multiply-add is the bound there).  Block row y handles
// vectors y Q .. y Q + Q - 1; its blocks write their partials to
// part[q * gridDim.x + blockIdx.x] and the last block of the row to finish
// adds them up in block order (reduce.cuh): deterministic.  cnt: one arrival
// counter per block row.  A non-null flag holding 0 makes the launch a no-op.
template <typename T, int MDOT_Q>
__device__ __forceinline__ void dots_block(int nq, size_t n, const T *const *ap, const T *__restrict__ b,
                                           double *part, double (&bs)[MDOT_Q], double *sh) {
    T p[MDOT_Q];
#pragma unroll
    for (int j = 0; j < MDOT_Q; j++) p[j] = T(0);
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const T bi = b[i];
#pragma unroll
        for (int j = 0; j < MDOT_Q; j++)
            if (ap[j]) p[j] += ap[j][i] * bi;
    }
    mdz_block_sum<MDOT_Q, T>(p, bs, sh);
    const int q0 = blockIdx.y * MDOT_Q;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int j = 0; j < MDOT_Q; j++)
            if (q0 + j < nq) part[(size_t)(q0 + j) * gridDim.x + blockIdx.x] = bs[j];
    }
}

template <typename T, int MDOT_Q>
__global__ void __launch_bounds__(256) k_dots(int nq, size_t n, const T *const *__restrict__ a,
                                              const T *__restrict__ b, double *part, unsigned int *cnt,
                                              double *out, const double *flag) {
    if (flag && *flag == 0.0) return;
    __shared__ double sh[32 * MDOT_Q];
    const int q0 = blockIdx.y * MDOT_Q;
    const T *ap[MDOT_Q];
#pragma unroll
    for (int j = 0; j < MDOT_Q; j++) ap[j] = q0 + j < nq ? a[q0 + j] : nullptr;
    double bs[MDOT_Q];
    dots_block<T, MDOT_Q>(nq, n, ap, b, part, bs, sh);
    if (!mdz_arrive_last(cnt + blockIdx.y, gridDim.x)) return;
    const int nrow = nq - q0 < MDOT_Q ? nq - q0 : MDOT_Q;
    mdz_sum_partials(part + (size_t)q0 * gridDim.x, gridDim.x, nrow, out + q0);
}

// One Gram-Schmidt pass's sums in one launch: (w, W_q) for q < k, then
// (w, w) and (w, r) as vectors k and k + 1 (b = w), summed as k_dots does
// (the last block of each block row adds its row's partials in block order);
// the last row to finish (a second arrival counter) then runs the pass's
// scalar step: mode 1 the check of the first pass (sc[5] = 1 asks for a
// second pass, else the scalars), mode 2 the scalars of the second pass.
// With flag (mode 2) every block returns at once when *flag is 0.
// cnt[0]: rows finished, cnt[1 + y]: blocks of row y finished.
template <typename T, int MDOT_Q>
__global__ void __launch_bounds__(256) k_gcr_dots(int k, size_t n, const T *const *__restrict__ a,
                                                  const T *__restrict__ w, const T *__restrict__ r, double *part,
                                                  double *out, const double *flag, int mode, double *sc,
                                                  double *tri, unsigned int *cnt) {
    if (flag && *flag == 0.0) return;
    __shared__ double sh[32 * MDOT_Q];
    const int nq = k + 2, q0 = blockIdx.y * MDOT_Q;
    const T *ap[MDOT_Q];
#pragma unroll
    for (int j = 0; j < MDOT_Q; j++) {
        const int q = q0 + j;
        ap[j] = q < k ? a[q] : (q == k ? w : (q == k + 1 ? r : nullptr));
    }
    double bs[MDOT_Q];
    dots_block<T, MDOT_Q>(nq, n, ap, w, part, bs, sh);
    if (!mdz_arrive_last(cnt + 1 + blockIdx.y, gridDim.x)) return;
    const int nrow = nq - q0 < MDOT_Q ? nq - q0 : MDOT_Q;
    mdz_sum_partials(part + (size_t)q0 * gridDim.x, gridDim.x, nrow, out + q0);
    if (!mdz_arrive_last(cnt, gridDim.y)) return;
    if (threadIdx.x != 0) return;
    double d[GCR_MAX_M + 2];
    for (int q = 0; q < nq; q++) d[q] = __ldcg(out + q);
    if (mode == 1) {
        double nrm2 = d[k];
        for (int q = 0; q < k; q++) nrm2 -= d[q] * d[q];
        // second pass when the first removed all but 1e-3 (FP64 basis) or 1e-1
        // (FP32 basis: its orthogonality decays faster, and alpha is taken
        // from r0 through the triangle) of w's squared norm
        if (k > 0 && !(nrm2 > (sizeof(T) == 4 ? 1e-1 : 1e-3) * d[k])) {   // keep this pass's coefficients in U
            for (int q = 0; q < k; q++) tri[(size_t)k * GCR_MAX_M + q] = d[q];
            sc[5] = 1.0;
            return;
        }
        sc[5] = 0.0;
    }
    gcr_scalars(k, d, sc, tri, mode == 2);
}

template <typename T>
static mdz_status gcr_dots_launch(mdz_ctx *ctx, gcr_space<T> &S, int k, const T *w, const T *r, double *out,
                                  const double *flag, int mode, double *sc, cudaStream_t st) {
    constexpr int Q = sizeof(T) == 4 ? 8 : 1;
    const int tiles = (k + 2 + Q - 1) / Q;
    int bx = mdz_blocks((long long)S.n, 256 * (sizeof(T) == 4 ? 8 : 4));
    const int cap = (sizeof(T) == 4 ? 152 * 8 : 152 * 4 + tiles - 1) / tiles;
    if (bx > cap) bx = cap;
    if (bx < 8) bx = 8;
    k_gcr_dots<T, Q><<<dim3(bx, tiles), 256, 0, st>>>(k, S.n, S.dA0, w, r, ctx->red_part + MDZ_RP_DOTS, out, flag,
                                                       mode, sc, S.tri, ctx->red_cnt + MDZ_RC_GCR);
    MDZ_LAUNCHED(ctx);
    return MDZ_OK;
}

template <typename T>
static mdz_status dots_launch(mdz_ctx *ctx, gcr_space<T> &S, int q0, int nq, const T *b, double *out,
                              cudaStream_t st, const double *flag = nullptr) {
    if (nq <= 0) return MDZ_OK;
    // FP32: 8 vectors per block row, ~8 elements per thread; FP64: one vector
    // per block row, about 600 blocks in all
    constexpr int Q = sizeof(T) == 4 ? 8 : 1;
    const int tiles = (nq + Q - 1) / Q;
    int bx = mdz_blocks((long long)S.n, 256 * (sizeof(T) == 4 ? 8 : 4));
    const int cap = (sizeof(T) == 4 ? 152 * 8 : 152 * 4 + tiles - 1) / tiles;
    if (bx > cap) bx = cap;
    if (bx < 8) bx = 8;
    k_dots<T, Q><<<dim3(bx, tiles), 256, 0, st>>>(nq, S.n, S.dA0 + q0, b, ctx->red_part + MDZ_RP_DOTS,
                                                   ctx->red_cnt + MDZ_RC_DOTS, out, flag);
    MDZ_LAUNCHED(ctx);
    return MDZ_OK;
}

// The preconditioner's ~10 launches per level, captured once per precision
// (its buffers, coefficients and the Krylov vectors r, z never move; the
// coefficients' values are refreshed by mg_setup outside the graph).
template <typename T>
static mdz_status precond_graph(mdz_ctx *ctx, gcr_space<T> &S, mg_hier<T> &H, const double *eta_n, const T *Dt,
                                cudaStream_t st, cudaGraphExec_t *out, long long *launches, int *slot_out) {
    mdz_solver *SV = ctx->solver;
    const int slot = (sizeof(T) == 8 ? 0 : 2) + (H.newton ? 1 : 0) + (Dt ? 4 : 0);
    *slot_out = slot;
    if (SV->pre[slot] && SV->pre_eta[slot] == eta_n) {
        *out = SV->pre[slot];
        *launches = SV->pre_launches[slot];
        return MDZ_OK;
    }
    if (SV->pre[slot]) { cudaGraphExecDestroy(SV->pre[slot]); SV->pre[slot] = nullptr; }
    const long long l0 = ctx->launches;
    MDZ_CUDA(ctx, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    mdz_status s = precondition<T>(ctx, H, eta_n, Dt, S.pin, S.z, S.nu, S.nv, st);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(st, &g);
    if (s != MDZ_OK) { if (g) cudaGraphDestroy(g); return s; }
    if (e != cudaSuccess) return mdz_cuda_check(ctx, e, "preconditioner capture");
    e = cudaGraphInstantiate(&SV->pre[slot], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { SV->pre[slot] = nullptr; return mdz_cuda_check(ctx, e, "preconditioner graph"); }
    SV->pre_launches[slot] = ctx->launches - l0;
    SV->pre_eta[slot] = eta_n;
    {   // per level: nu1 + nu2 sweeps and one residual, each reading x, f, the
        // inverse diagonal and both viscosities and writing one vector, plus
        // the tags; restriction and prolongation one read + one write each;
        // the fine-level pressure block and right-hand side 3 vectors
        double b = 0.0;
        for (int l = 0; l < H.nlev; l++) {
            const mg_level<T> &L = H.L[l];
            double nuv = (double)(L.nu() + L.nv()), nc = (double)L.ncx * L.ncz, ng = (double)L.Nx * L.Nz;
            b += (SV->nu1 + SV->nu2 + 1) * (sizeof(T) * (4.0 * nuv + nc + ng) + (nuv + nc + ng));
            b += 4.0 * sizeof(T) * nuv;
        }
        b += 3.0 * sizeof(T) * (double)S.n;
        if (Dt) b += sizeof(T) * (double)S.np;
        SV->pre_bytes[slot] = b;
    }
    ctx->launches = l0;
    *out = SV->pre[slot];
    *launches = SV->pre_launches[slot];
    return MDZ_OK;
}

// ---------------------------------------------------------------------------
// GCR on K x = b (x0 = 0), right-preconditioned.  The preconditioner
// (V-cycle), the operator apply and the stored basis Z, W run in precision
// P; the iterate x, the residual r and every inner product are FP64 (T).
// P = T = double: the plain FP64 solve.  T = double, P = float: the inner
// solve of the FP32 form (r narrowed to FP32 before the preconditioner), whose
// recursive residual differs from b - K x only by FP32 rounding of the
// applies and basis vectors, which the FP64 defect correction outside absorbs.
template <typename T, typename P>
static mdz_status gcr_solve(mdz_ctx *ctx, gcr_space<T> &S, gcr_space<P> &SP, mg_hier<P> &H,
                            const stokes_coefs<P> &K, bool newton, const double *eta_n, double rtol, int maxit,
                            int *its_out, double *rel_out, cudaStream_t st) {
    constexpr bool mixed = sizeof(T) != sizeof(P);
    mdz_solver *SV = ctx->solver;
    stokes_geom G = mdz_stokes_geom(ctx);
    const size_t n = S.n, nu = S.nu, nv = S.nv;
    int nb = mdz_blocks(n);
    MDZ_CUDA(ctx, cudaMemsetAsync(S.x, 0, sizeof(T) * n, st));
    // ||r0||
    // S.dots layout (doubles, B = GCR_MAX_M + 8): first-pass sums of even / odd
    // iterations at 0 / 4B, the scalars sc at GCR_MAX_M + 4, second-pass sums
    // at 2B / 5B, a scratch sum at 3B
    const int B = GCR_MAX_M + 8;
    double *sc = S.dots + (GCR_MAX_M + 4), *dots = S.dots + 3 * B;
    double *dots1p[2] = {S.dots, S.dots + 4 * B}, *dots2p[2] = {S.dots + 2 * B, S.dots + 5 * B};
    for (int q = 0; q < 2; q++) {
        MDZ_CUDA(ctx, cudaMemsetAsync(dots1p[q], 0, sizeof(double) * (GCR_MAX_M + 3), st));
        MDZ_CUDA(ctx, cudaMemsetAsync(dots2p[q], 0, sizeof(double) * (GCR_MAX_M + 3), st));
    }
    mdz_status s;
    cudaGraphExec_t pre = nullptr;
    long long pre_launches = 0;
    int pslot = 0;
    const P *Dt = newton && SV->schur == 1 ? K.D11 : nullptr;   // tangent Schur scaling (Newton solves)
    if ((s = precond_graph<P>(ctx, SP, H, eta_n, Dt, st, &pre, &pre_launches, &pslot)) != MDZ_OK) return s;
    // (r, r) via the pointer-table slot m+1 against r itself
    if ((s = dots_launch<T>(ctx, S, S.m + 1, 1, S.r, dots, st)) != MDZ_OK) return s;
    k_set_scalar<<<1, 32, 0, st>>>(sc + 3, dots);
    MDZ_LAUNCHED(ctx);
    MDZ_CUDA(ctx, cudaMemcpyAsync(SV->sc, dots, sizeof(double), cudaMemcpyDeviceToHost, st));
    MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    {
        const volatile int *flags = (const volatile int *)(SV->sc + 20);
        if (flags[0]) return mdz_fail(ctx, MDZ_ERR_NOT_CONVERGED, "multigrid: coarsest-level block singular");
        if (flags[1]) return mdz_fail(ctx, MDZ_ERR_STATE, "multigrid: Galerkin entry outside the stencil footprint");
    }
    double rn2 = SV->sc[0], rn02 = rn2;
    int it = 0;
    if (rn02 == 0.0) { if (its_out) *its_out = 0; if (rel_out) *rel_out = 0.0; return MDZ_OK; }
    // the preconditioner's first input r0 and (FP32 form) the FP32 copy of r0
    k_gcr_start<P, T><<<nb, MDZ_THREADS, 0, st>>>(n, S.r, mixed ? SP.r : (P *)nullptr, SP.pin);
    MDZ_LAUNCHED(ctx);
    int k = 0;
    const double *gamma = SP.tri + (size_t)GCR_MAX_M * GCR_MAX_M;
    // end of a basis: x += Z U^-1 alpha, r = r0 - W alpha (and its copies)
    auto end_basis = [&](bool need_r) -> mdz_status {
        if (k == 0) return MDZ_OK;
        k_gcr_gamma<<<1, 32, 0, st>>>(k, sc, SP.tri);
        MDZ_LAUNCHED(ctx);
        k_gcr_xupdate<P, T><<<nb, MDZ_THREADS, 0, st>>>(n, k, SP.Z, gamma, S.x);
        MDZ_LAUNCHED(ctx);
        if (need_r) {
            k_gcr_rupdate<P, T><<<nb, MDZ_THREADS, 0, st>>>(n, k, SP.W, sc, S.r, mixed ? SP.r : (P *)nullptr, SP.pin);
            MDZ_LAUNCHED(ctx);
        }
        k = 0;
        return MDZ_OK;
    };
    const int check = SV->check > 0 ? SV->check : 1;
    for (it = 0; it < maxit; it++) {
        if (k == S.m && (s = end_basis(true)) != MDZ_OK) return s;   // restart: fold the basis into x and r
        cudaEvent_t ev;
        mdz_prof_begin(ctx, MDZ_PROF_MG_SMOOTH, st, &ev);
        MDZ_CUDA(ctx, cudaGraphLaunch(pre, st));
        ctx->launches += pre_launches;
        mdz_prof_end(ctx, MDZ_PROF_MG_SMOOTH, SV->pre_bytes[pslot], st, ev);
        mdz_prof_begin(ctx, MDZ_PROF_STOKES_APPLY, st, &ev);
        stokes_apply_launch<P>(G, K, stokes_cvec<P>{SP.z, SP.z + nu, SP.z + nu + nv},
                               stokes_vec<P>{SP.w, SP.w + nu, SP.w + nu + nv}, nullptr, newton, st);
        MDZ_LAUNCHED(ctx);
        {   // algorithmic bytes: input and output vectors, the D-tensor read once, tags
            size_t nc = S.np, ng = (size_t)G.Nx * G.Nz;
            double coef = newton ? (8.0 * nc + 4.0 * ng) : (2.0 * nc + ng);
            double bytes = sizeof(P) * (2.0 * n + coef) + (double)(nu + nv + nc + ng);
            mdz_prof_end(ctx, MDZ_PROF_STOKES_APPLY, bytes, st, ev);
        }
        mdz_prof_begin(ctx, MDZ_PROF_KRYLOV, st, &ev);
        // The basis W and the raw preconditioned vectors Z stay in the apply's
        // precision P (in the FP32 form: as the FP32 V-cycle and apply
        // produced them); x, r and every sum are FP64.  First pass:
        // (w, W_q) q < k, (w, w), (w, r0); the check decides on the device
        // whether a second pass runs.
        const int ng = nb < 152 * 8 ? nb : 152 * 8;
        double *d1 = dots1p[it & 1], *d2 = dots2p[it & 1];
        if ((s = gcr_dots_launch<P>(ctx, SP, k, SP.w, SP.r, d1, nullptr, 1, sc, st)) != MDZ_OK) return s;
        if (k > 0) {   // second pass (each launch returns at once unless sc[5] = 1)
            k_gcr_orth_if<P><<<ng, MDZ_THREADS, 0, st>>>(n, k, SP.W, d1, sc, SP.w);
            MDZ_LAUNCHED(ctx);
            if ((s = gcr_dots_launch<P>(ctx, SP, k, SP.w, SP.r, d2, sc + 5, 2, sc, st)) != MDZ_OK) return s;
        }
        k_gcr_finish<P><<<nb, MDZ_THREADS, 0, st>>>(n, k, SP.W, SP.Z, d1, d2, sc, SP.z, SP.w, SP.pin,
                                                     dots1p[(it + 1) & 1], dots2p[(it + 1) & 1]);
        MDZ_LAUNCHED(ctx);
        {   // algorithmic bytes (one Gram-Schmidt pass): the sums read W_q,
            // w and r0 (k + 2 P vectors); the finish reads W_q, w, z and
            // writes W_k, Z_k and the next input (k + 5)
            double pv = 2.0 * k + 7.0;
            mdz_prof_end(ctx, MDZ_PROF_KRYLOV, (double)n * sizeof(P) * pv, st, ev);
        }
        k++;
        // the running norm lives on the device; the host looks every `check`
        // iterations, at each restart and at the iteration limit
        if ((it + 1) % check != 0 && k != S.m && it + 1 < maxit) continue;
        MDZ_CUDA(ctx, cudaMemcpyAsync(SV->sc, sc, 4 * sizeof(double), cudaMemcpyDeviceToHost, st));
        MDZ_CUDA(ctx, cudaStreamSynchronize(st));
        rn2 = SV->sc[3];
        if (!std::isfinite(rn2)) return mdz_fail(ctx, MDZ_ERR_NAN, "GCR: NaN in the Krylov iteration");
        if (rn2 <= rtol * rtol * rn02 || (k == S.m)) {
            // fold the basis in and take the true norm of r at convergence
            // and at each restart
            if ((s = end_basis(true)) != MDZ_OK) return s;
            if ((s = dots_launch<T>(ctx, S, S.m + 1, 1, S.r, dots, st)) != MDZ_OK) return s;
            k_set_scalar<<<1, 32, 0, st>>>(sc + 3, dots);
            MDZ_LAUNCHED(ctx);
            MDZ_CUDA(ctx, cudaMemcpyAsync(SV->sc, dots, sizeof(double), cudaMemcpyDeviceToHost, st));
            MDZ_CUDA(ctx, cudaStreamSynchronize(st));
            rn2 = SV->sc[0];
            if (rn2 <= rtol * rtol * rn02) { it++; break; }
        }
    }
    if ((s = end_basis(false)) != MDZ_OK) return s;   // the current basis' part of the iterate
    if (its_out) *its_out = it;
    if (rel_out) *rel_out = sqrt(rn2 > 0 ? rn2 : 0.0) / sqrt(rn02);
    return MDZ_OK;
}

// ---------------------------------------------------------------------------
// Public device-level solve: K dx = F.  F and dx in grid layout (u | v | p
// contiguous, length n), FP64.  precision 64: plain FP64 GCR + FP64 V-cycle;
// precision 32: FP64 defect correction around FP32 GCR + FP32 V-cycle.
mdz_status mdz_dev_solve(mdz_ctx *ctx, const mdz_fields &f, bool newton, int precision, double rtol, int maxit,
                         const double *F, double *dx, mdz_solve_stats *stats, cudaStream_t st, bool reuse_mg) {
    mdz_status s = mdz_solver_ensure(ctx);
    if (s != MDZ_OK) return s;
    mdz_solver *SV = ctx->solver;
    gcr_space<double> &S64 = SV->g64;
    const size_t n = S64.n, nu = S64.nu, nv = S64.nv;
    stokes_geom G = mdz_stokes_geom(ctx);
    stokes_coefs<double> K64 = mdz_coefs64(f);
    int its = 0, total = 0, cycles = 0;
    double rel = 1.0;
    if (precision == 64) {
        const bool nh = newton && SV->mg_jacobian;
        if (!(reuse_mg && SV->mg64.built && SV->mg64.newton == nh))
            if ((s = mg_setup<double>(ctx, SV->mg64, f.eta_n, f.eta_s, K64, nh, st)) != MDZ_OK) return s;
        MDZ_CUDA(ctx, cudaMemcpyAsync(S64.r, F, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
        if ((s = gcr_solve<double, double>(ctx, S64, S64, SV->mg64, K64, newton, f.eta_n, rtol, maxit, &its, &rel,
                                           st)) != MDZ_OK)
            return s;
        MDZ_CUDA(ctx, cudaMemcpyAsync(dx, S64.x, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
        total = its;
        cycles = 1;
    } else {
        gcr_space<float> &S32 = SV->g32;
        // FP32 copy of the operator
        const double *Dsrc[12] = {f.D11_n, f.D12_n, f.D13_n, f.D14_n, f.D21_n, f.D22_n, f.D23_n, f.D24_n,
                                  f.D31_s, f.D32_s, f.D33_s, f.D34_s};
        for (int q = 0; q < 12; q++) {
            size_t m = q < 8 ? S32.np : (size_t)ctx->g.Nx * ctx->g.Nz;
            if (!newton && q != 0 && q != 5 && q != 10) continue;
            k_convert<double, float><<<mdz_blocks(m), MDZ_THREADS, 0, st>>>(m, Dsrc[q], S32.Dc[q]);
            MDZ_LAUNCHED(ctx);
        }
        stokes_coefs<float> K32{S32.Dc[0], S32.Dc[1], S32.Dc[2], S32.Dc[3], S32.Dc[4], S32.Dc[5], S32.Dc[6],
                                S32.Dc[7], S32.Dc[8], S32.Dc[9], S32.Dc[10], S32.Dc[11]};
        const bool nh = newton && SV->mg_jacobian;
        if (!(reuse_mg && SV->mg32.built && SV->mg32.newton == nh))
            if ((s = mg_setup<float>(ctx, SV->mg32, f.eta_n, f.eta_s, K32, nh, st)) != MDZ_OK) return s;
        // defect correction: r64 = F - K64 dx64 ; solve K32 e = r64 ; dx64 += e
        MDZ_CUDA(ctx, cudaMemsetAsync(dx, 0, sizeof(double) * n, st));
        MDZ_CUDA(ctx, cudaMemcpyAsync(S64.r, F, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
        double *dn = (double *)(ctx->d_counters + 8);
        double r0 = -1.0, prev = 1e300;
        auto defect = [&]() -> mdz_status {   // r64 = F - K64 dx
            stokes_apply_launch<double>(G, K64, stokes_cvec<double>{dx, dx + nu, dx + nu + nv},
                                        stokes_vec<double>{S64.t, S64.t + nu, S64.t + nu + nv}, nullptr, newton, st);
            MDZ_LAUNCHED(ctx);
            MDZ_CUDA(ctx, cudaMemcpyAsync(S64.r, F, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
            k_axpby<double><<<mdz_blocks(n), MDZ_THREADS, 0, st>>>(n, -1.0, S64.t, 1.0, S64.r);
            MDZ_LAUNCHED(ctx);
            return MDZ_OK;
        };
        // Each cycle solves for the current FP64 defect in FP32.  An FP32 solve
        // cannot resolve corrections whose K-image is below FP32 rounding of the
        // stresses, so the contraction per cycle degrades on stiff problems: the
        // loop runs while the defect still shrinks by 10 % and takes back a
        // cycle that made it grow.
        for (cycles = 0; cycles < 60; cycles++) {
            // norm of the FP64 defect
            if ((s = dots_launch<double>(ctx, S64, S64.m + 1, 1, S64.r, dn, st)) != MDZ_OK) return s;
            MDZ_CUDA(ctx, cudaMemcpyAsync(SV->sc + 8, dn, sizeof(double), cudaMemcpyDeviceToHost, st));
            MDZ_CUDA(ctx, cudaStreamSynchronize(st));
            double rn = sqrt(SV->sc[8]);
            if (r0 < 0) r0 = rn;
            rel = r0 > 0 ? rn / r0 : 0.0;
            if (rel <= rtol || r0 == 0.0) break;
            if (cycles > 0 && rel > prev) {   // the last correction made it worse: undo it
                k_axpby<double><<<mdz_blocks(n), MDZ_THREADS, 0, st>>>(n, -1.0, S64.x, 1.0, dx);
                MDZ_LAUNCHED(ctx);
                if ((s = defect()) != MDZ_OK) return s;
                rel = prev;
                break;
            }
            if (rel > 0.9 * prev || total >= maxit) break;   // refinement stalled or budget spent
            prev = rel;
            // Inner solve on the FP64 defect: FP64 Krylov space, FP32 stencils
            // and V-cycles.  The recursive residual differs from b - K64 x by
            // the FP32 rounding of the applies times the cancellation in the
            // Krylov sums, so each inner solve asks for at most three digits
            // and one basis length; the FP64 cycles carry the accuracy.
            double inner_rtol = rtol / rel;
            if (inner_rtol < 1e-3) inner_rtol = 1e-3;
            if (inner_rtol > 0.1) inner_rtol = 0.1;
            const int inner_max = maxit - total < S64.m ? maxit - total : S64.m;
            if ((s = gcr_solve<double, float>(ctx, S64, S32, SV->mg32, K32, newton, f.eta_n, inner_rtol, inner_max,
                                              &its, nullptr, st)) != MDZ_OK)
                return s;
            total += its;
            k_axpby<double><<<mdz_blocks(n), MDZ_THREADS, 0, st>>>(n, 1.0, S64.x, 1.0, dx);
            MDZ_LAUNCHED(ctx);
            if ((s = defect()) != MDZ_OK) return s;
        }
    }
    if ((s = remove_pressure_mean(ctx, dx + nu + nv, st)) != MDZ_OK) return s;
    if (stats) {
        stats->iterations = total;
        stats->refinements = cycles;
        stats->rel_residual = rel;
        stats->mg_levels = SV->mg64.nlev;
    }
    return MDZ_OK;
}

// ---------------------------------------------------------------------------
extern "C" mdz_status mdz_SolveStokesDefect(mdz_ctx *ctx, mdz_fields *f, int jacobian, int precision, double rtol,
                                            int maxit, const double *Fu, const double *Fv, const double *Fp,
                                            double *dxu, double *dxv, double *dxp, int *iterations,
                                            double *rel_residual) {
    if (!ctx || !f || !Fu || !Fv || !Fp || !dxu || !dxv || !dxp)
        return ctx ? mdz_fail(ctx, MDZ_ERR_ARG, "SolveStokesDefect: null argument") : MDZ_ERR_ARG;
    if (precision != 64 && precision != 32) return mdz_fail(ctx, MDZ_ERR_ARG, "SolveStokesDefect: precision 64 or 32");
    mdz_status s = mdz_ensure_fields(ctx);
    if (s != MDZ_OK) return s;
    if ((s = mdz_solver_ensure(ctx)) != MDZ_OK) return s;
    cudaStream_t st = ctx->stream;
    if ((s = mdz_upload_fields(ctx, f, st)) != MDZ_OK) return s;
    const mdz_dgrid &g = ctx->g;
    size_t nu = (size_t)g.Nx * (g.Nz + 1), nv = (size_t)(g.Nx + 1) * g.Nz, np = (size_t)g.ncx * g.ncz;
    double *buf = (double *)mdz_stage(ctx, 7, sizeof(double) * 2 * (nu + nv + np));
    if (!buf) return mdz_fail(ctx, MDZ_ERR_CUDA, "SolveStokesDefect: staging allocation failed");
    double *F = buf, *dx = buf + nu + nv + np;
    MDZ_CUDA(ctx, cudaMemcpyAsync(F, Fu, nu * 8, cudaMemcpyHostToDevice, st));
    MDZ_CUDA(ctx, cudaMemcpyAsync(F + nu, Fv, nv * 8, cudaMemcpyHostToDevice, st));
    MDZ_CUDA(ctx, cudaMemcpyAsync(F + nu + nv, Fp, np * 8, cudaMemcpyHostToDevice, st));
    mdz_solve_stats stt{};
    if ((s = mdz_dev_solve(ctx, ctx->d, jacobian != 0, precision, rtol, maxit, F, dx, &stt, st)) != MDZ_OK) return s;
    MDZ_CUDA(ctx, cudaMemcpyAsync(dxu, dx, nu * 8, cudaMemcpyDeviceToHost, st));
    MDZ_CUDA(ctx, cudaMemcpyAsync(dxv, dx + nu, nv * 8, cudaMemcpyDeviceToHost, st));
    MDZ_CUDA(ctx, cudaMemcpyAsync(dxp, dx + nu + nv, np * 8, cudaMemcpyDeviceToHost, st));
    MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    if (iterations) *iterations = stt.iterations;
    if (rel_residual) *rel_residual = stt.rel_residual;
    if (!(stt.rel_residual <= rtol))
        return mdz_fail(ctx, MDZ_ERR_NOT_CONVERGED, "SolveStokesDefect: relative residual %.3e > %.3e after %d its",
                        stt.rel_residual, rtol, stt.iterations);
    return MDZ_OK;
}
