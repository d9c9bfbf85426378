// Internal declarations shared by the CUDA translation units of the library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>
#include "mdoodz_gpu.h"
#include "reduce.cuh"

// kernel classes timed when profiling is on
enum { MDZ_PROF_VISCOSITY = 0, MDZ_PROF_STOKES_APPLY = 1, MDZ_PROF_MG_SMOOTH = 2, MDZ_PROF_P2G = 3, MDZ_PROF_MLP = 4,
       MDZ_PROF_KRYLOV = 5, MDZ_PROF_MG_SETUP = 6, MDZ_PROF_NCLS = 7 };
struct mdz_ctx;
void mdz_prof_begin(mdz_ctx *ctx, int cls, cudaStream_t st, cudaEvent_t *ev);
void mdz_prof_end(mdz_ctx *ctx, int cls, double bytes, cudaStream_t st, cudaEvent_t a);

#define MDZ_THREADS 256

// Device-side copy of the grid: coordinates and tags.  All arrays are owned by
// the context (cudaMalloc'd once at mdz_create).
struct mdz_dgrid {
    int Nx, Nz, ncx, ncz;
    double dx, dz, xmin, xmax, zmin, zmax;
    double idx, idz;   // 1/dx, 1/dz (marker kernels multiply; see ceil_quot)
    double *xg, *zg, *xc, *zc, *xvz, *zvx;
    signed char *BCu, *BCv, *BCp, *BCg;
    double *BCu_val, *BCv_val;
};

// ceil(d / h + add) exactly as the correctly rounded quotient d / h gives it,
// from the product with ih = 1/h: the two differ by a few units in the last
// place, so only a value that close to an integer pays for the division.  An
// FP64 division is a long instruction sequence on this part, and the marker
// kernels take several per marker where the reference divides by the grid
// spacing; the cell indices must still match the reference's bit for bit.
// The margin is fixed for |q| up to 2^16 (grids have fewer lines; a quotient
// beyond that lies outside the grid, where every caller clamps the index).
#define MDZ_CEIL_QUOT_TOL (16.0 * 2.220446049250313e-16 * 65538.0)
__device__ __forceinline__ double ceil_quot(double d, double h, double ih, double add) {
    const double q = d * ih + add;
    const double c = ceil(q), f = c - q;
    if (f > MDZ_CEIL_QUOT_TOL && f < 1.0 - MDZ_CEIL_QUOT_TOL) return c;
    return ceil(d / h + add);
}

// Marker store: structure of arrays, FP64 positions, int32 phases.
struct mdz_markers {
    int n = 0;
    long long cap = 0;
    double *x = nullptr, *z = nullptr, *vx = nullptr, *vz = nullptr;
    int *phase = nullptr;
    double *attr[MDZ_M_NATTR] = {nullptr};
};

// Cell binning of the resident markers: markers sorted by cell (stable).
struct mdz_bins {
    bool valid = false;
    int ncells = 0;
    int *cell = nullptr;        // per marker: cell index or -1 (inactive)
    int *count = nullptr;       // per cell
    int *start = nullptr;       // per cell + 1: exclusive scan of count
    int *cursor = nullptr;      // scratch for the scatter
    int *sorted = nullptr;      // marker indices grouped by cell, ascending inside a cell
    int *qvert = nullptr;       // per sorted position: the marker's nearest vertex, ip | jp << 16
    int *scan_partials = nullptr;
};

#define MDZ_XFER_STREAMS 4
struct mdz_ctx {
    // the grid description with the context's own copies of its coordinate
    // lines and tags (host_desc points at these; the Dirichlet values live on
    // the device only): PureShearALE rewrites the lines and bounds
    mdz_grid_desc host_desc{};
    std::vector<double> hline[6];        // xg, zg, xc, zc, xvz, zvx
    std::vector<signed char> htag[4];    // BCu, BCv, BCp, BCg
    double *ale_sums = nullptr;          // device: wall sums and counts of PureShearALE
    mdz_dgrid g{};
    int n_phases = 0;
    mdz_markers m;
    mdz_bins bins;
    cudaStream_t stream = nullptr;
    cudaStream_t xfer[MDZ_XFER_STREAMS] = {};   // copy streams of the batched marker transfers (lazy)
    long long launches = 0;
    mdz_fields d{};              // device mirrors of every grid field (allocated on first use)
    bool fields_ready = false;
    int *d_counters = nullptr;   // small device scratch: failure counters etc.
    // set by the time step around its projections: phase-fraction projections
    // count there the active nodes that received no marker weight
    int *p2g_empty = nullptr;
    // deterministic reductions (reduce.cuh): per-block partial slots and the
    // arrival counters of the last-block sums
    double *red_part = nullptr;
    unsigned int *red_cnt = nullptr;
    bool bcs_checked = false, bcs_ok = false, bcs_neumann = false;
    // optional per-launch event timing of the main kernel classes (bench roofline)
    bool profiling = false;
    struct prof_rec { int cls; cudaEvent_t a, b; double bytes; };
    std::vector<prof_rec> prof;
    double prof_ms[8] = {0}, prof_bytes[8] = {0};
    long long prof_n[8] = {0};
    struct mdz_solver *solver = nullptr;   // Krylov / multigrid workspace (solver.cu)
    struct mdz_mlp *mlp = nullptr;         // learned local-rheology guess (mlp.cu)
    struct mdz_reseed_ws *reseed = nullptr;   // quarter-cell workspace of the reseeding (reseed.cu)
    std::string err;
    // host-call staging buffers (grown on demand)
    void *stage[9] = {nullptr};
    size_t stage_bytes[9] = {0};
};

// ---- helpers -------------------------------------------------------------
mdz_status mdz_fail(mdz_ctx *ctx, mdz_status s, const char *fmt, ...);
mdz_status mdz_cuda_check(mdz_ctx *ctx, cudaError_t e, const char *what);
// Device staging buffer slot i with at least `bytes` bytes.
void *mdz_stage(mdz_ctx *ctx, int slot, size_t bytes);

#define MDZ_CUDA(ctx, call)                                                          \
    do {                                                                              \
        cudaError_t e__ = (call);                                                     \
        if (e__ != cudaSuccess) return mdz_cuda_check((ctx), e__, #call);             \
    } while (0)

#define MDZ_LAUNCHED(ctx)                                                            \
    do {                                                                              \
        (ctx)->launches++;                                                            \
        cudaError_t e__ = cudaGetLastError();                                         \
        if (e__ != cudaSuccess) return mdz_cuda_check((ctx), e__, "kernel launch");   \
    } while (0)

static inline int mdz_blocks(long long n, int threads = MDZ_THREADS) {
    long long b = (n + threads - 1) / threads;
    return (int)(b < 1 ? 1 : b);
}

// Node-set geometry: sizes and coordinate lines of a node set.
struct mdz_nodeset {
    int nx, nz;               // nodes per direction
    const double *X, *Z;      // coordinate lines (device)
    const signed char *tag;   // tags (device)
};
mdz_nodeset mdz_get_nodeset(const mdz_ctx *ctx, int centroid);

// Binning (markers.cu): the cell bins, and the scan / scatter / per-bin
// sort kernels the quarter-cell bins of the reseeding reuse.
mdz_status mdz_ensure_bins(mdz_ctx *ctx, cudaStream_t st);
__global__ void k_scan_blocks(int n, const int *__restrict__ in, int *__restrict__ out, int *__restrict__ partial);
__global__ void k_scan_partials(int nb, int *partial);
__global__ void k_scan_add(int n, int *__restrict__ out, const int *__restrict__ partial);
__global__ void k_bin_scatter(int n, const int *__restrict__ cell, const int *__restrict__ start,
                              int *__restrict__ cursor, int *__restrict__ sorted);
__global__ void k_bin_sort_segments(int ncells, const int *__restrict__ start, int *__restrict__ sorted);

// Marker reseeding (reseed.cu): the reseeding of CountPartCell on the resident
// markers; T_n, sxxd_n, szzd_n, p_n (centroids) and sxz_s (vertices) are
// device fields, read when direct = 0.
struct mdz_attr_ptrs { double *a[MDZ_M_NATTR]; };
// PureShearALE on device velocities u, v (stream st): moves the box, rewrites
// the grid lines (host copies and device), the spacings and the solver levels.
mdz_status mdz_dev_pure_shear_ale(mdz_ctx *ctx, const double *u, const double *v, double dt, cudaStream_t st);
mdz_status mdz_solver_regrid(mdz_ctx *ctx);
// Move the box to the given bounds and regenerate the grid lines over it.
mdz_status mdz_set_box(mdz_ctx *ctx, double xmin, double xmax, double zmin, double zmax, cudaStream_t st);
mdz_status mdz_dev_reseed(mdz_ctx *ctx, int min_part_cell, int direct, const double *T_n, const double *sxxd_n,
                          const double *szzd_n, const double *sxz_s, const double *p_n, cudaStream_t st,
                          int *n_added);
void mdz_reseed_free(mdz_ctx *ctx);

// Every mdz_fields member with its node set (X-macro): VX / VZ velocity nodes,
// CEN centroids, VER vertices, PPN / PPS phase fractions (n_phases rows).
#define MDZ_FIELD_LIST(X) \
    X(u, VX) \
    X(v, VZ) \
    X(p, CEN) \
    X(p_corr, CEN) \
    X(div_u, CEN) \
    X(div_u_s, VER) \
    X(exxd, CEN) \
    X(ezzd, CEN) \
    X(exz, VER) \
    X(exz_n, CEN) \
    X(exxd_s, VER) \
    X(ezzd_s, VER) \
    X(sxxd0, CEN) \
    X(szzd0, CEN) \
    X(sxz0, VER) \
    X(sxxd0_s, VER) \
    X(szzd0_s, VER) \
    X(sxz0_n, CEN) \
    X(mu_n, CEN) \
    X(mu_s, VER) \
    X(T, CEN) \
    X(T_s, VER) \
    X(P_s, VER) \
    X(d0_n, CEN) \
    X(d0_s, VER) \
    X(phi0_n, CEN) \
    X(phi0_s, VER) \
    X(X0_n, CEN) \
    X(X0_s, VER) \
    X(strain_n, CEN) \
    X(strain_s, VER) \
    X(dil_n, CEN) \
    X(dil_s, VER) \
    X(fric_n, CEN) \
    X(fric_s, VER) \
    X(C_n, CEN) \
    X(C_s, VER) \
    X(p0_n, CEN) \
    X(p0_s, VER) \
    X(bet_n, CEN) \
    X(bet_s, VER) \
    X(rho_n, CEN) \
    X(rho_s, VER) \
    X(phase_perc_n, PPN) \
    X(phase_perc_s, PPS) \
    X(eta_n, CEN) \
    X(eta_s, VER) \
    X(eta_phys_n, CEN) \
    X(eta_phys_s, VER) \
    X(VE_n, CEN) \
    X(VE_s, VER) \
    X(sxxd, CEN) \
    X(szzd, CEN) \
    X(sxz, VER) \
    X(sxz_n, CEN) \
    X(eII_el, CEN) \
    X(eII_pl, CEN) \
    X(eII_pwl, CEN) \
    X(eII_lin, CEN) \
    X(eII_cst, CEN) \
    X(d_n, CEN) \
    X(exx_el, CEN) \
    X(ezz_el, CEN) \
    X(exz_el, VER) \
    X(exx_diss, CEN) \
    X(ezz_diss, CEN) \
    X(exz_diss, VER) \
    X(detadexx_n, CEN) \
    X(detadezz_n, CEN) \
    X(detadgxz_n, CEN) \
    X(detadp_n, CEN) \
    X(ddivpdexx_n, CEN) \
    X(ddivpdezz_n, CEN) \
    X(ddivpdgxz_n, CEN) \
    X(ddivpdp_n, CEN) \
    X(detadexx_s, VER) \
    X(detadezz_s, VER) \
    X(detadgxz_s, VER) \
    X(detadp_s, VER) \
    X(div_u_el, CEN) \
    X(div_u_pl, CEN) \
    X(div_u_r, CEN) \
    X(Wtot, CEN) \
    X(Wel, CEN) \
    X(Wdiss, CEN) \
    X(X_n, CEN) \
    X(X_s, VER) \
    X(OverS_n, CEN) \
    X(OverS_s, VER) \
    X(D11_n, CEN) \
    X(D12_n, CEN) \
    X(D13_n, CEN) \
    X(D14_n, CEN) \
    X(D21_n, CEN) \
    X(D22_n, CEN) \
    X(D23_n, CEN) \
    X(D24_n, CEN) \
    X(D31_s, VER) \
    X(D32_s, VER) \
    X(D33_s, VER) \
    X(D34_s, VER) \
    X(roger_x, VX) \
    X(roger_z, VZ) \
    X(rhs_p, CEN) \
    X(gx, VX) \
    X(gz, VZ) \
    X(ru, VX) \
    X(rv, VZ) \
    X(rp, CEN) \
    X(eII_exp, CEN) \
    X(eII_gbs, CEN) \
    X(kx, VX) \
    X(kz, VZ) \
    X(Cv, CEN) \
    X(Qr, CEN) \
    X(dT, CEN) \
    X(alp, CEN)

enum mdz_field_kind { MDZ_K_VX, MDZ_K_VZ, MDZ_K_CEN, MDZ_K_VER, MDZ_K_PPN, MDZ_K_PPS };
size_t mdz_field_count(const mdz_ctx *ctx, int kind);
mdz_status mdz_ensure_fields(mdz_ctx *ctx);
mdz_status mdz_upload_fields(mdz_ctx *ctx, const mdz_fields *h, cudaStream_t st);
mdz_status mdz_download_fields(mdz_ctx *ctx, const mdz_fields *h, const char *const *names, int n, cudaStream_t st);

// device launchers (rheology.cu)
mdz_status mdz_dev_strain_rates(mdz_ctx *ctx, const mdz_fields &f, cudaStream_t st);
mdz_status mdz_dev_c2v(mdz_ctx *ctx, const double *cen, double *ver, cudaStream_t st);
mdz_status mdz_dev_v2c(mdz_ctx *ctx, double *cen, const double *ver, cudaStream_t st);
mdz_status mdz_check_materials(mdz_ctx *ctx, const mdz_materials *m);
// Local rheology on centroids and vertices.  d_counters: [0] local solves not
// converged, [1] learned starts that fell back to the plain solve, [2] learned
// starts.  learned: every local solve starts from a guess and the plain solve
// reruns where the polish fails; the guess is the MLP's (weights loaded in the
// context) unless warm = 2, which starts from the solutions the previous
// evaluation recorded (same phase fractions: within one time step).  warm >= 1
// records each converged solve in the guess buffer for the next evaluation.
mdz_status mdz_dev_viscosity(mdz_ctx *ctx, const mdz_materials *m, const mdz_rheo_params *prm, const mdz_fields &f,
                             int *d_counters, cudaStream_t st, bool learned = false, bool fp32 = false,
                             int warm = 0);
mdz_status mdz_dev_operators(mdz_ctx *ctx, const mdz_rheo_params *prm, const mdz_fields &f, int jacobian,
                             cudaStream_t st);
mdz_status mdz_dev_rhs(mdz_ctx *ctx, const mdz_rheo_params *prm, double gx, double gz, const mdz_fields &f,
                       cudaStream_t st);
mdz_status mdz_dev_rk4(mdz_ctx *ctx, const double *du, const double *dv, double dt, cudaStream_t st);
