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
// A 32 x 8 block covers a 32 x 8 tile of the index box; it first computes the
// strain rates of the input once per centroid and vertex the tile's rows read
// (34 x 10 of each, with a two-cell halo) into shared memory, then each
// thread evaluates its rows from them.  A Newton row reads six centroid and
// six vertex rates, each shared by about ten rows: computed per row they made
// the FP64 apply FP64-pipe bound (FP64 runs at a small fraction of the FP32
// rate on this part) and the FP32 apply load-bound.
template <typename T, bool NEWTON, bool RES>
__global__ void __launch_bounds__(256) k_stokes_apply(stokes_geom G, stokes_coefs<T> D, stokes_cvec<T> x,
                                                      stokes_vec<T> y, stokes_cvec<T> b, T celvol) {
    __shared__ T s_ex[RT_H][RT_W], s_ez[RT_H][RT_W], s_g[RT_H][RT_W];
    const int Nx = G.Nx, Nz = G.Nz, ncx = G.ncx, ncz = G.ncz;
    const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 8;
    const rates_tile<T> rt{s_ex, s_ez, s_g, i0 - 2, j0 - 2, i0 - 1, j0 - 1};
    {
        const rates_direct<T> rd = direct_rates<T>(G, x);
        for (int t = threadIdx.x + threadIdx.y * 32; t < RT_W * RT_H; t += 256) {
            const int a = t % RT_W, h = t / RT_W;
            const int kc = rt.c0x + a, lc = rt.c0z + h, kv = rt.v0x + a, lv = rt.v0z + h;
            pair2<T> e{T(0), T(0)};
            if (kc >= 0 && kc < ncx && lc >= 0 && lc < ncz) e = rd.exx(kc, lc);
            s_ex[h][a] = e.x;
            s_ez[h][a] = e.y;
            s_g[h][a] = (kv >= 0 && kv < Nx && lv >= 0 && lv < Nz) ? rd.gxz(kv, lv) : T(0);
        }
    }
    __syncthreads();
    const int i = i0 + threadIdx.x, j = j0 + threadIdx.y;
    if (i < Nx && j <= Nz) {            // Vx node (i, j)
        int c = i + j * Nx;
        T r = 0;
        if (G.BCu[c] == -1) {
            r = xrow<T, NEWTON>(G, D, x, i, j, rt);
            if (RES) r -= b.u[c];
            r *= celvol;
        }
        y.u[c] = r;
    }
    if (i <= Nx && j < Nz) {            // Vz node (i, j)
        int c = i + j * (Nx + 1);
        T r = 0;
        if (G.BCv[c] == -1) {
            r = zrow<T, NEWTON>(G, D, x, i, j, rt);
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
        // equations: inner (-1) and Neumann (2) velocity nodes
        if (i < nu && (tu[i] == -1 || tu[i] == 2)) { double f = fu[i]; acc[0] += f * f; acc[3] += 1; }
        if (i < nv && (tv[i] == -1 || tv[i] == 2)) { double f = fv[i]; acc[1] += f * f; acc[4] += 1; }
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
static bool supported_bcs(const mdz_ctx *ctx, bool *neumann) {
    // inner (-1), Dirichlet on the boundary (0), free-slip ghosts (13), and
    // Neumann (2) on the west / east Vx lines and the south / north Vz lines
    const mdz_grid_desc &d = ctx->host_desc;
    size_t nu = (size_t)d.Nx * (d.Nz + 1), nv = (size_t)(d.Nx + 1) * d.Nz, np = (size_t)(d.Nx - 1) * (d.Nz - 1);
    *neumann = false;
    for (size_t i = 0; i < nu; i++) {
        const int t = d.BCu_type[i], k = (int)(i % d.Nx), l = (int)(i / d.Nx);
        if (t == 2 && (k == 0 || k == d.Nx - 1) && l > 0 && l < d.Nz) { *neumann = true; continue; }
        if (t != -1 && t != 0 && t != 13) return false;
    }
    for (size_t i = 0; i < nv; i++) {
        const int t = d.BCv_type[i], k = (int)(i % (d.Nx + 1)), l = (int)(i / (d.Nx + 1));
        if (t == 2 && (l == 0 || l == d.Nz - 1) && k > 0 && k < d.Nx) { *neumann = true; continue; }
        if (t != -1 && t != 0 && t != 13) return false;
    }
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
        ctx->bcs_ok = supported_bcs(ctx, &ctx->bcs_neumann);
        ctx->bcs_checked = true;
    }
    if (!ctx->bcs_ok)
        return mdz_fail(ctx, MDZ_ERR_UNSUPPORTED,
                        "Stokes: only inner equations with Dirichlet (0), free-slip (13) and wall Neumann (2) "
                        "boundaries are implemented");
    return MDZ_OK;
}

stokes_coefs<double> mdz_coefs64(const mdz_fields &f) {
    return stokes_coefs<double>{f.D11_n, f.D12_n, f.D13_n, f.D14_n, f.D21_n, f.D22_n, f.D23_n, f.D24_n,
                                f.D31_s, f.D32_s, f.D33_s, f.D34_s};
}

// ---------------------------------------------------------------------------
// Neumann rows (tag 2): Xmomentum_WestNeumannDecoupled / _EastNeumannDecoupled
// and Zmomentum_SouthNeumannDecoupled / _NorthNeumannDecoupled
// (SOURCE/StokesAssemblyDecoupled.c:476-795, 1168-1428).  The reference calls
// the same functions from its Picard and its Jacobian builders, but the
// Jacobian builder sets comp = 1 (:3851), which adds the 2/3 compressible
// terms to these rows; the Picard operator and the residual use comp = 0
// (the incompressible model).  Viscosities eta_n, eta_s are taken directly,
// the prescribed traction BC*.val / h moves to the right-hand side.  Each row is a list of (unknown, coefficient) entries with
// the reference's two selections: the assembled entries (AddCoeff2), whose
// Dirichlet-like neighbours (tags 0, 31, 11, 13) go to the right-hand side as
// coefficient x value (twice the value for tag 11), and the entries its
// residual sums directly.  Residual: F = (-b + sum over Dirichlet-like assembled
// entries of c val + sum over residual entries of c x) x cell volume, with
// b = roger (west / south: minus, east / north: plus the traction over h);
// the reference takes the Dirichlet part from its last assembly, identical to
// this where that assembly saw the same state.  Operator: the assembled entries
// that are unknowns.  The north row's residual reads the pressure one cell
// below the one its assembled row uses (c2 - ncx, :1418), kept as it is.
namespace {
struct nrow_entry {
    double c;
    int kind, idx;        // 0 u, 1 v, 2 p
    bool assembled, residual;
    double mult;          // Dirichlet value multiplier of the assembled entry
};

__device__ __forceinline__ bool dirlike(int t) { return t == 0 || t == 31 || t == 11 || t == 13; }

struct nrow {
    nrow_entry e[11];
    int n = 0;
    __device__ void add(int kind, int idx, double c, bool assembled, bool residual, double mult = 1.0) {
        e[n++] = nrow_entry{c, kind, idx, assembled, residual, mult};
    }
};

__device__ void neumann_x(const stokes_geom &G, const double *eta_n, const double *eta_s, int k, int l, bool west,
                          double comp, nrow &R) {
    const int nx = G.Nx, ncx = G.ncx, nxvz = nx + 1;
    const int c1 = k + l * nx, c2 = k - 1 + (l - 1) * ncx, c3 = k + l * nxvz;
    const double ixx = G.cd[GC_IXX], izz = G.cd[GC_IZZ], ixz = G.cd[GC_IXZ], idx = G.cd[GC_IDX];
    const double etaC = west ? eta_n[c2 + 1] : eta_n[c2], etaN = eta_s[c1], etaS = eta_s[c1 - nx];
    const int tS = G.BCu[c1 - nx], tN = G.BCu[c1 + nx], tO = west ? G.BCu[c1 + 1] : G.BCu[c1 - 1];
    double uC = 0, uO = 0, uS = 0, uN = 0, vSW = 0, vSE = 0, vNW = 0, vNE = 0, pO = 0;
    const double c23 = comp * 2.0 / 3.0;
    if (tO != 30) { uC = -2.0 * ixx * etaC + c23 * ixx * etaC; uO = 2.0 * ixx * etaC - c23 * ixx * etaC; }
    if (tS != 30 && tN != 30) {
        if (tS != 13) { uS = izz * etaS; uC += -izz * etaS; }
        if (tN != 13) { uN = izz * etaN; uC += -izz * etaN; }
    }
    if (tS == 30 && tN != 30 && tN != 13) { uC += -izz * etaN; uN = izz * etaN; }
    if (tS != 30 && tN == 30 && tS != 13) { uC += -izz * etaS; uS = izz * etaS; }
    if (tS == 11) uC += -izz * etaS;
    if (tN == 11) uC += -izz * etaN;
    const bool sp = G.BCv[c3 - nxvz] != 30 && G.BCv[c3 - nxvz + 1] != 30;
    const bool np_ = G.BCv[c3 + 1] != 30 && G.BCv[c3] != 30;
    if (sp) { vSE = -ixz * etaS + c23 * ixz * etaC; vSW = ixz * etaS - c23 * ixz * etaC; }
    if (np_) { vNE = ixz * etaN - c23 * ixz * etaC; vNW = -ixz * etaN + c23 * ixz * etaC; }
    const int ip = west ? c2 + 1 : c2;
    const bool pin = G.BCp[ip] != 30;
    if (pin) pO = west ? -idx : idx;
    R.add(0, c1, -uC, true, true);
    R.add(0, c1 - nx, -uS, tS != 30, tS != 30 && tS != 11, tS == 11 ? 2.0 : 1.0);
    R.add(0, west ? c1 + 1 : c1 - 1, -uO, tO != 30, tO != 30);
    R.add(0, c1 + nx, -uN, tN != 30, tN != 30 && tN != 11, tN == 11 ? 2.0 : 1.0);
    const int vi[4] = {c3 - nxvz, c3 - nxvz + 1, c3, c3 + 1};
    const double vc[4] = {-vSW, -vSE, -vNW, -vNE};
    for (int q = 0; q < 4; q++) {
        const bool pair = q < 2 ? sp : np_;
        const int t = G.BCv[vi[q]];
        R.add(1, vi[q], vc[q], pair, pair && t != 11 && t != 0);
    }
    R.add(2, ip, -pO, pin, pin);
}

__device__ void neumann_z(const stokes_geom &G, const double *eta_n, const double *eta_s, int k, int l, bool south,
                          double comp, nrow &R) {
    const int nx = G.Nx, ncx = G.ncx, nxvz = nx + 1;
    const int c1 = k + l * nx, c2 = k - 1 + (l - 1) * ncx, c3 = k + l * nxvz;
    const double ixx = G.cd[GC_IXX], izz = G.cd[GC_IZZ], ixz = G.cd[GC_IXZ], idz = G.cd[GC_IDZ];
    const double etaC = south ? eta_n[c2 + ncx] : eta_n[c2], etaE = eta_s[c1], etaW = eta_s[c1 - 1];
    const int tW = G.BCv[c3 - 1], tE = G.BCv[c3 + 1], tO = south ? G.BCv[c3 + nxvz] : G.BCv[c3 - nxvz];
    double uSW = 0, uSE = 0, uNW = 0, uNE = 0, vC = 0, vO = 0, vW = 0, vE = 0, pO = 0;
    const bool sp = G.BCu[c1 - 1] != 30 && G.BCu[c1] != 30;
    const bool np_ = G.BCu[c1 + nx - 1] != 30 && G.BCu[c1 + nx] != 30;
    const double c23 = comp * 2.0 / 3.0;   // etaS = etaN = etaC in these rows
    if (sp) { uSW = ixz * etaW - c23 * etaC * ixz; uSE = -ixz * etaE + c23 * etaC * ixz; }
    if (np_) { uNW = -ixz * etaW + c23 * etaC * ixz; uNE = ixz * etaE - c23 * etaC * ixz; }
    if (tO != 30) { vC = -2.0 * izz * etaC + c23 * etaC * izz; vO = 2.0 * izz * etaC - c23 * etaC * izz; }
    if (tW != 30 && tE != 30) {
        if (tW != 13) { vW = ixx * etaW; vC += -ixx * etaW; }
        if (tE != 13) { vE = ixx * etaE; vC += -ixx * etaE; }
    }
    if (tW == 30 && tE != 30 && tE != 13) { vE = ixx * etaE; vC += -ixx * etaE; }
    if (tW != 30 && tE == 30 && tW != 13) { vW = ixx * etaW; vC += -ixx * etaW; }
    if (tW == 11) vC += -ixx * etaW;
    if (tE == 11) vC += -ixx * etaE;
    const int ip = south ? c2 + ncx : c2;
    const bool pin = G.BCp[ip] != 30;
    if (pin) pO = south ? -idz : idz;
    const int ui[4] = {c1 - 1, c1, c1 + nx - 1, c1 + nx};
    const double uc[4] = {-uSW, -uSE, -uNW, -uNE};
    for (int q = 0; q < 4; q++) {
        const bool pair = q < 2 ? sp : np_;
        const int t = G.BCu[ui[q]];
        R.add(0, ui[q], uc[q], pair, pair && t != 11 && t != 0);
    }
    R.add(1, c3 - 1, -vW, tW != 30, tW != 30 && tW != 11, tW == 11 ? 2.0 : 1.0);
    R.add(1, c3, -vC, true, true);
    R.add(1, c3 + 1, -vE, tE != 30, tE != 30 && tE != 11, tE == 11 ? 2.0 : 1.0);
    R.add(1, south ? c3 + nxvz : c3 - nxvz, -vO, tO != 30, tO != 30);
    if (south) {
        R.add(2, ip, -pO, pin, pin);
    } else {   // assembled on c2, summed by the residual on c2 - ncx
        R.add(2, ip, -pO, pin, false);
        const bool pin2 = G.BCp[c2 - ncx] != 30;
        R.add(2, c2 - ncx, -pO, false, pin2);
    }
}

// One thread per wall node: west / east Vx lines (l = 1..Nz-1), south /
// north Vz lines (k = 1..Nx-1).  RES: y = residual rows (b = roger_x /
// roger_z, bu / bv = the Dirichlet values); else y = operator rows.
template <bool RES>
__global__ void k_neumann_rows(stokes_geom G, const double *__restrict__ eta_n, const double *__restrict__ eta_s,
                               stokes_cvec<double> x, const double *__restrict__ bx, const double *__restrict__ bz,
                               const double *__restrict__ bu, const double *__restrict__ bv, double *__restrict__ yu,
                               double *__restrict__ yv, double comp) {
    const int Nx = G.Nx, Nz = G.Nz, nxvz = Nx + 1;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int nX = 2 * (Nz - 1), nZ = 2 * (Nx - 1);
    if (t >= nX + nZ) return;
    nrow R;
    int row, kind;
    double b;
    if (t < nX) {
        const bool west = t < Nz - 1;
        const int l = 1 + (west ? t : t - (Nz - 1)), k = west ? 0 : Nx - 1;
        row = k + l * Nx;
        if (G.BCu[row] != 2) return;
        kind = 0;
        neumann_x(G, eta_n, eta_s, k, l, west, comp, R);
        b = RES ? bx[row] + (west ? -bu[row] : bu[row]) * G.cd[GC_IDX] : 0.0;
    } else {
        const int q = t - nX;
        const bool south = q < Nx - 1;
        const int k = 1 + (south ? q : q - (Nx - 1)), l = south ? 0 : Nz - 1;
        row = k + l * nxvz;
        if (G.BCv[row] != 2) return;
        kind = 1;
        neumann_z(G, eta_n, eta_s, k, l, south, comp, R);
        b = RES ? bz[row] + (south ? -bv[row] : bv[row]) * G.cd[GC_IDZ] : 0.0;
    }
    double r = RES ? -b : 0.0;
    for (int q = 0; q < R.n; q++) {
        const nrow_entry &e = R.e[q];
        const int tag = e.kind == 0 ? G.BCu[e.idx] : (e.kind == 1 ? G.BCv[e.idx] : G.BCp[e.idx]);
        const double xv = e.kind == 0 ? x.u[e.idx] : (e.kind == 1 ? x.v[e.idx] : x.p[e.idx]);
        if (RES) {
            if (e.assembled && e.kind != 2 && dirlike(tag))
                r += e.c * e.mult * (e.kind == 0 ? bu[e.idx] : bv[e.idx]);
            if (e.residual) r += e.c * xv;
        } else if (e.assembled && !dirlike(tag)) {
            r += e.c * xv;
        }
    }
    r *= G.cd[GC_CELVOL];
    if (kind == 0) yu[row] = r;
    else yv[row] = r;
}
}  // namespace

static mdz_status neumann_launch(mdz_ctx *ctx, bool res, bool jacobian, const mdz_fields &f, stokes_cvec<double> x,
                                 double *yu, double *yv, cudaStream_t st) {
    if (!ctx->bcs_neumann) return MDZ_OK;
    const mdz_dgrid &g = ctx->g;
    const int n = 2 * (g.Nz - 1) + 2 * (g.Nx - 1);
    stokes_geom G = mdz_stokes_geom(ctx);
    if (res)
        k_neumann_rows<true><<<mdz_blocks(n, 128), 128, 0, st>>>(G, f.eta_n, f.eta_s, x, f.roger_x, f.roger_z,
                                                                  g.BCu_val, g.BCv_val, yu, yv, 0.0);
    else
        k_neumann_rows<false><<<mdz_blocks(n, 128), 128, 0, st>>>(G, f.eta_n, f.eta_s, x, nullptr, nullptr, nullptr,
                                                                   nullptr, yu, yv, jacobian ? 1.0 : 0.0);
    MDZ_LAUNCHED(ctx);
    return MDZ_OK;
}

mdz_status mdz_dev_residual(mdz_ctx *ctx, const mdz_fields &f, double *d_norms6, cudaStream_t st) {
    stokes_geom G = mdz_stokes_geom(ctx);
    stokes_cvec<double> x{f.u, f.v, f.p_corr}, b{f.roger_x, f.roger_z, f.rhs_p};
    stokes_vec<double> y{f.ru, f.rv, f.rp};
    stokes_apply_launch<double>(G, mdz_coefs64(f), x, y, &b, false, st);
    MDZ_LAUNCHED(ctx);
    mdz_status s = neumann_launch(ctx, true, false, f, x, f.ru, f.rv, st);
    if (s != MDZ_OK) return s;
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
    if ((s = neumann_launch(ctx, false, jacobian != 0, ctx->d, stokes_cvec<double>{dxu, dxv, dxp}, dyu, dyv, st)) !=
        MDZ_OK)
        return s;
    MDZ_CUDA(ctx, cudaMemcpyAsync(yu, dyu, nu * 8, cudaMemcpyDeviceToHost, st));
    MDZ_CUDA(ctx, cudaMemcpyAsync(yv, dyv, nv * 8, cudaMemcpyDeviceToHost, st));
    MDZ_CUDA(ctx, cudaMemcpyAsync(yp, dyp, np * 8, cudaMemcpyDeviceToHost, st));
    MDZ_CUDA(ctx, cudaStreamSynchronize(st));
    return MDZ_OK;
}
