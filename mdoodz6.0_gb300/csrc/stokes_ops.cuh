// Matrix-free decoupled Stokes operator on the staggered grid.
//
// One thread per (i, j) of the (Nx+1) x (Nz+1) index box evaluates whichever
// of the three equations exist there: x-momentum at Vx node (i, j), z-momentum
// at Vz node (i, j), continuity at centroid (i, j).  The momentum rows are the
// composition the reference's stencils encode:
//   strain rates of the input -> tangent stresses (D-tensor) -> divergence,
// with the reference's per-row flags (in*) and averaging weights (w*) so that
// the result equals its assembled matrices row by row:
//   Picard rows:  Xmomentum_InnerNodesDecoupled / Zmomentum_InnerNodesDecoupled
//                 (SOURCE/StokesAssemblyDecoupled.c:109-234, 796-1167)
//   Newton rows:  Xjacobian_InnerNodesDecoupled3 / Zjacobian_InnerNodesDecoupled3
//                 (SOURCE/StokesAssemblyDecoupled.c:3034-3426, 3427-3833)
//   continuity:   Continuity_InnerNodesDecoupled (SOURCE/StokesAssemblyDecoupled.c:62-103)
// Inner equations only (tag -1); Neumann (2), periodic, air and free-surface
// rows are rejected by the host before launch.  All rows are multiplied by the
// cell volume as in the reference.
#pragma once
#include "mdz_internal.cuh"

template <typename T>
struct pair2 {
    T x, y;
};

template <typename T>
struct stokes_coefs {
    // centroids: D11..D14, D21..D24 ; vertices: D31..D34 (Picard uses D11, D22, D33 only)
    const T *D11, *D12, *D13, *D14, *D21, *D22, *D23, *D24;
    const T *D31, *D32, *D33, *D34;
};

template <typename T>
struct stokes_vec {
    T *u, *v, *p;
};

template <typename T>
struct stokes_cvec {
    const T *u, *v, *p;
};

// geometry constants in both precisions (gc<T>): a kernel in FP32 must not
// convert an FP64 constant per thread, FP64 conversions issue at a small
// fraction of the FP32 rate on this part
enum { GC_DX = 0, GC_DZ, GC_IDX, GC_IDZ, GC_CELVOL, GC_IXX, GC_IZZ, GC_IXZ, GC_N };

struct stokes_geom {
    int Nx, Nz, ncx, ncz;
    double dx, dz;
    const signed char *BCu, *BCv, *BCp, *BCg;
    double idx, idz;   // 1/dx, 1/dz: the stencils multiply (a division costs a
                       // long FP64 instruction sequence on this part)
    double cd[GC_N];
    float cf[GC_N];
};

template <typename T>
__host__ __device__ __forceinline__ T gc(const stokes_geom &G, int k) {
    if constexpr (sizeof(T) == 8) return G.cd[k];
    else return G.cf[k];
}

inline stokes_geom make_geom(int Nx, int Nz, double dx, double dz, const signed char *BCu, const signed char *BCv,
                             const signed char *BCp, const signed char *BCg) {
    stokes_geom G{Nx, Nz, Nx - 1, Nz - 1, dx, dz, BCu, BCv, BCp, BCg, 1.0 / dx, 1.0 / dz, {0}, {0}};
    const double c[GC_N] = {dx, dz, 1.0 / dx, 1.0 / dz, dx * dz, 1.0 / (dx * dx), 1.0 / (dz * dz), 1.0 / (dx * dz)};
    for (int k = 0; k < GC_N; k++) { G.cd[k] = c[k]; G.cf[k] = (float)c[k]; }
    return G;
}

// 1/w for the averaging weights w in {2, 3, 4}; w in {0, 1} stays (exact
// constants, identical to the division)
template <typename T>
__device__ __forceinline__ T wrecip(T w) {
    return w > T(3.5) ? T(0.25) : (w > T(2.5) ? T(1.0 / 3.0) : (w > T(1.5) ? T(0.5) : w));
}

// Strain rates of the input the rows are built from: deviatoric normal
// rates at centroid (kc, lc) and the engineering shear rate at vertex
// (kv, lv).  rates_direct computes them from the velocities where a row asks;
// rates_tile (k_stokes_apply) reads them from a shared-memory tile where the
// block computed each one once (a Newton row reads six of each, and every
// centroid / vertex is shared by about ten rows).
template <typename T>
struct rates_direct {
    const T *u, *v;
    int nx, nxvz;
    T idx, idz;
    __device__ __forceinline__ pair2<T> exx(int kc, int lc) const {
        const int cu = kc + (lc + 1) * nx, cv = kc + 1 + lc * nxvz;
        const T dudx = (u[cu + 1] - u[cu]) * idx, dvdz = (v[cv + nxvz] - v[cv]) * idz;
        const T div = dudx + dvdz;
        return pair2<T>{dudx - div * T(1.0 / 3.0), dvdz - div * T(1.0 / 3.0)};
    }
    __device__ __forceinline__ T gxz(int kv, int lv) const {
        const int cu = kv + lv * nx, cv = kv + lv * nxvz;
        return (u[cu + nx] - u[cu]) * idz + (v[cv + 1] - v[cv]) * idx;
    }
};

// centroids kc in [c0x, c0x + RT_W), lc in [c0z, c0z + RT_H); vertices
// kv in [v0x, v0x + RT_W), lv in [v0z, v0z + RT_H)
constexpr int RT_W = 34, RT_H = 10;
template <typename T>
struct rates_tile {
    const T (*ex)[RT_W], (*ez)[RT_W], (*g)[RT_W];
    int c0x, c0z, v0x, v0z;
    __device__ __forceinline__ pair2<T> exx(int kc, int lc) const {
        return pair2<T>{ex[lc - c0z][kc - c0x], ez[lc - c0z][kc - c0x]};
    }
    __device__ __forceinline__ T gxz(int kv, int lv) const { return g[lv - v0z][kv - v0x]; }
};

template <typename T>
__device__ __forceinline__ rates_direct<T> direct_rates(const stokes_geom &G, const stokes_cvec<T> &x) {
    return rates_direct<T>{x.u, x.v, G.Nx, G.Nx + 1, gc<T>(G, GC_IDX), gc<T>(G, GC_IDZ)};
}

// x-momentum row at Vx node (k, l), k in 1..Nx-2, l in 1..Nz-1.
template <typename T, bool NEWTON, typename RS>
__device__ __forceinline__ T xrow(const stokes_geom &G, const stokes_coefs<T> &D, const stokes_cvec<T> &x, int k,
                                  int l, const RS &rs) {
    const int nx = G.Nx, ncx = G.ncx, nxvz = nx + 1;
    const int c1 = k + l * nx, c2 = k - 1 + (l - 1) * ncx;
    const T idx = gc<T>(G, GC_IDX), idz = gc<T>(G, GC_IDZ);
    const int iPrW = c2, iPrE = c2 + 1, ixyN = c1, ixyS = c1 - nx;
    const T inW = G.BCp[iPrW] == -1 ? T(1) : T(0), inE = G.BCp[iPrE] == -1 ? T(1) : T(0);
    const T inS = (G.BCg[ixyS] != 30 && G.BCu[c1 - nx] != 13) ? T(1) : T(0);
    const T inN = (G.BCg[ixyN] != 30 && G.BCu[c1 + nx] != 13) ? T(1) : T(0);
    // velocity gradients on the row's control volume
    const T *p = x.p;
    (void)nxvz;
    auto exx_c = [&](int kc, int lc) { return rs.exx(kc, lc); };
    auto gxz_v = [&](int kv, int lv) { return rs.gxz(kv, lv); };
    pair2<T> eW = exx_c(k - 1, l - 1), eE = exx_c(k, l - 1);
    T gN = gxz_v(k, l), gS = gxz_v(k, l - 1);
    T TxxE, TxxW, TxzN, TxzS;
    if (!NEWTON) {
        TxxE = D.D11[iPrE] * eE.x;
        TxxW = D.D11[iPrW] * eW.x;
        TxzN = D.D33[ixyN] * gN;
        TxzS = D.D33[ixyS] * gS;
    } else {
        const int nzvx = G.Nz + 1;
        const int iPrSW = iPrW - ncx, iPrSE = iPrE - ncx, iPrNW = iPrW + ncx, iPrNE = iPrE + ncx;
        const int ixySW = ixyS - 1, ixySE = ixyS + 1, ixyNW = ixyN - 1, ixyNE = ixyN + 1;
        T inSWc = 0, inSEc = 0, inNWc = 0, inNEc = 0, inSWv = 0, inSEv = 0, inNWv = 0, inNEv = 0;
        if (l > 1 || (l == 1 && G.BCu[c1 - nx] == 11)) {
            if (G.BCp[iPrSW] == -1) inSWc = 1;
            if (G.BCp[iPrSE] == -1) inSEc = 1;
        }
        if (l < nzvx - 2 || (l == nzvx - 2 && G.BCu[c1 + nx] == 11)) {
            if (G.BCp[iPrNW] == -1) inNWc = 1;
            if (G.BCp[iPrNE] == -1) inNEc = 1;
        }
        {   // k > 0 always holds for inner rows
            if (G.BCg[ixySW] != 30) inSWv = 1;
            if (G.BCg[ixyNW] != 30) inNWv = 1;
        }
        {
            if (G.BCg[ixySE] != 30) inSEv = 1;
            if (G.BCg[ixyNE] != 30) inNEv = 1;
        }
        T wE = inN + inS + inNEv + inSEv, wW = inN + inS + inNWv + inSWv;
        T wS = inW + inE + inSWc + inSEc, wN = inW + inE + inNWc + inNEc;
        wW = wrecip(wW);
        wE = wrecip(wE);
        wS = wrecip(wS);
        wN = wrecip(wN);
        // shear rate averaged onto the two centroids, with this row's weights
        T gNW = inNWv != T(0) ? gxz_v(k - 1, l) : T(0), gSW = inSWv != T(0) ? gxz_v(k - 1, l - 1) : T(0);
        T gNE = inNEv != T(0) ? gxz_v(k + 1, l) : T(0), gSE = inSEv != T(0) ? gxz_v(k + 1, l - 1) : T(0);
        T gE = wE * (inN * gN + inS * gS + inNEv * gNE + inSEv * gSE);
        T gW = wW * (inN * gN + inS * gS + inNWv * gNW + inSWv * gSW);
        TxxE = D.D11[iPrE] * eE.x + D.D12[iPrE] * eE.y + D.D13[iPrE] * gE + D.D14[iPrE] * p[iPrE];
        TxxW = D.D11[iPrW] * eW.x + D.D12[iPrW] * eW.y + D.D13[iPrW] * gW + D.D14[iPrW] * p[iPrW];
        // normal rates and pressure averaged onto the two vertices
        pair2<T> eSW = inSWc != T(0) ? exx_c(k - 1, l - 2) : pair2<T>{T(0), T(0)};
        pair2<T> eSE = inSEc != T(0) ? exx_c(k, l - 2) : pair2<T>{T(0), T(0)};
        pair2<T> eNW = inNWc != T(0) ? exx_c(k - 1, l) : pair2<T>{T(0), T(0)};
        pair2<T> eNE = inNEc != T(0) ? exx_c(k, l) : pair2<T>{T(0), T(0)};
        T pSW = inSWc != T(0) ? p[iPrSW] : T(0), pSE = inSEc != T(0) ? p[iPrSE] : T(0);
        T pNW = inNWc != T(0) ? p[iPrNW] : T(0), pNE = inNEc != T(0) ? p[iPrNE] : T(0);
        T exxS = wS * (inW * eW.x + inE * eE.x + inSWc * eSW.x + inSEc * eSE.x);
        T ezzS = wS * (inW * eW.y + inE * eE.y + inSWc * eSW.y + inSEc * eSE.y);
        T pS_ = wS * (inW * p[iPrW] + inE * p[iPrE] + inSWc * pSW + inSEc * pSE);
        T exxN = wN * (inW * eW.x + inE * eE.x + inNWc * eNW.x + inNEc * eNE.x);
        T ezzN = wN * (inW * eW.y + inE * eE.y + inNWc * eNW.y + inNEc * eNE.y);
        T pN_ = wN * (inW * p[iPrW] + inE * p[iPrE] + inNWc * pNW + inNEc * pNE);
        TxzS = D.D31[ixyS] * exxS + D.D32[ixyS] * ezzS + D.D33[ixyS] * gS + D.D34[ixyS] * pS_;
        TxzN = D.D31[ixyN] * exxN + D.D32[ixyN] * ezzN + D.D33[ixyN] * gN + D.D34[ixyN] * pN_;
    }
    T grad = (p && G.BCp[iPrE] != 30 && G.BCp[iPrW] != 30) ? (p[iPrE] - p[iPrW]) * idx : T(0);
    if (NEWTON) grad = (inE * p[iPrE] - inW * p[iPrW]) * idx;
    return -(inE * TxxE - inW * TxxW) * idx - (inN * TxzN - inS * TxzS) * idz + grad;
}

// z-momentum row at Vz node (k, l), k in 1..Nx-1, l in 1..Nz-2.
template <typename T, bool NEWTON, typename RS>
__device__ __forceinline__ T zrow(const stokes_geom &G, const stokes_coefs<T> &D, const stokes_cvec<T> &x, int k,
                                  int l, const RS &rs) {
    const int nx = G.Nx, ncx = G.ncx, nxvz = nx + 1;
    const int c3 = k + l * nxvz, c1 = k + l * nx, c2 = k - 1 + (l - 1) * ncx;
    const T idx = gc<T>(G, GC_IDX), idz = gc<T>(G, GC_IDZ);
    const int iPrS = c2, iPrN = c2 + ncx, ixyW = c1 - 1, ixyE = c1;
    T inS = 0, inN = 0;
    if (G.BCv[c3 - nxvz] != 30 && G.BCv[c3 + nxvz] != 30) { inS = 1; inN = 1; }
    if (G.BCv[c3 - nxvz] == 30 && G.BCv[c3 + nxvz] != 30) inN = 1;
    if (G.BCv[c3 - nxvz] != 30 && G.BCv[c3 + nxvz] == 30) inS = 1;
    if (G.BCp[iPrS] == -1) inS = 1;
    if (G.BCp[iPrN] == -1) inN = 1;
    const T inW = (G.BCg[ixyW] != 30 && G.BCv[c3 - 1] != 13) ? T(1) : T(0);
    const T inE = (G.BCg[ixyE] != 30 && G.BCv[c3 + 1] != 13) ? T(1) : T(0);
    const T *v = x.v, *p = x.p;
    auto exx_c = [&](int kc, int lc) { return rs.exx(kc, lc); };
    auto gxz_v = [&](int kv, int lv) { return rs.gxz(kv, lv); };
    pair2<T> eS = exx_c(k - 1, l - 1), eN = exx_c(k - 1, l);
    T gW = gxz_v(k - 1, l), gE = gxz_v(k, l);
    T TzzN, TzzS, TxzE, TxzW, ndrop = 0;
    if (!NEWTON) {
        TzzN = D.D22[iPrN] * eN.y;
        TzzS = D.D22[iPrS] * eS.y;
        TxzE = D.D33[ixyE] * gE;
        TxzW = D.D33[ixyW] * gW;
    } else {
        const int nz = G.Nz;
        const int iPrSW = iPrS - 1, iPrSE = iPrS + 1, iPrNW = iPrN - 1, iPrNE = iPrN + 1;
        const int ixySW = ixyW - nx, ixyNW = ixyW + nx, ixySE = ixyE - nx, ixyNE = ixyE + nx;
        T inSWc = 0, inSEc = 0, inNWc = 0, inNEc = 0, inSWv = 0, inSEv = 0, inNWv = 0, inNEv = 0;
        if (k > 1 || (k == 1 && G.BCv[c3 - 1] == -1)) {
            if (G.BCp[iPrSW] == -1) inSWc = 1;
            if (G.BCp[iPrNW] == -1) inNWc = 1;
        }
        if (k < nxvz - 2 || (k == nxvz - 2 && G.BCv[c3 + 1] == -1)) {
            if (G.BCp[iPrSE] == -1) inSEc = 1;
            if (G.BCp[iPrNE] == -1) inNEc = 1;
        }
        if (l > 0) {
            if (G.BCg[ixySW] != 30) inSWv = 1;
            if (G.BCg[ixySE] != 30) inSEv = 1;
        }
        if (l < nz - 1) {
            if (G.BCg[ixyNW] != 30) inNWv = 1;
            if (G.BCg[ixyNE] != 30) inNEv = 1;
        }
        T wE = inN + inS + inNEc + inSEc, wW = inN + inS + inNWc + inSWc;
        T wS = inW + inE + inSWv + inSEv, wN = inW + inE + inNWv + inNEv;
        wW = wrecip(wW);
        wE = wrecip(wE);
        wS = wrecip(wS);
        wN = wrecip(wN);
        // shear rate averaged onto centroids S and N
        T gSW = inSWv != T(0) ? gxz_v(k - 1, l - 1) : T(0), gSE = inSEv != T(0) ? gxz_v(k, l - 1) : T(0);
        T gNW = inNWv != T(0) ? gxz_v(k - 1, l + 1) : T(0), gNE = inNEv != T(0) ? gxz_v(k, l + 1) : T(0);
        T gS = wS * (inW * gW + inE * gE + inSWv * gSW + inSEv * gSE);
        T gN = wN * (inW * gW + inE * gE + inNWv * gNW + inNEv * gNE);
        TzzS = D.D21[iPrS] * eS.x + D.D22[iPrS] * eS.y + D.D23[iPrS] * gS + D.D24[iPrS] * p[iPrS];
        TzzN = D.D21[iPrN] * eN.x + D.D22[iPrN] * eN.y + D.D23[iPrN] * gN + D.D24[iPrN] * p[iPrN];
        // normal rates and pressure averaged onto vertices W and E
        pair2<T> eSW = inSWc != T(0) ? exx_c(k - 2, l - 1) : pair2<T>{T(0), T(0)};
        pair2<T> eNW = inNWc != T(0) ? exx_c(k - 2, l) : pair2<T>{T(0), T(0)};
        pair2<T> eSE = inSEc != T(0) ? exx_c(k, l - 1) : pair2<T>{T(0), T(0)};
        pair2<T> eNE = inNEc != T(0) ? exx_c(k, l) : pair2<T>{T(0), T(0)};
        T pSW = inSWc != T(0) ? p[iPrSW] : T(0), pNW = inNWc != T(0) ? p[iPrNW] : T(0);
        T pSE = inSEc != T(0) ? p[iPrSE] : T(0), pNE = inNEc != T(0) ? p[iPrNE] : T(0);
        T exxW = wW * (inN * eN.x + inS * eS.x + inNWc * eNW.x + inSWc * eSW.x);
        T ezzW = wW * (inN * eN.y + inS * eS.y + inNWc * eNW.y + inSWc * eSW.y);
        T pW_ = wW * (inN * p[iPrN] + inS * p[iPrS] + inNWc * pNW + inSWc * pSW);
        T exxE = wE * (inN * eN.x + inS * eS.x + inNEc * eNE.x + inSEc * eSE.x);
        T ezzE = wE * (inN * eN.y + inS * eS.y + inNEc * eNE.y + inSEc * eSE.y);
        T pE_ = wE * (inN * p[iPrN] + inS * p[iPrS] + inNEc * pNE + inSEc * pSE);
        TxzW = D.D31[ixyW] * exxW + D.D32[ixyW] * ezzW + D.D33[ixyW] * gW + D.D34[ixyW] * pW_;
        TxzE = D.D31[ixyE] * exxE + D.D32[ixyE] * ezzE + D.D33[ixyE] * gE + D.D34[ixyE] * pE_;
        // The reference's Jacobian assembles the diagonal Vz neighbours only
        // where they are plain unknowns (tag -1, StokesAssemblyDecoupled.c:
        // 3669-3711): a Neumann wall node (tag 2) diagonal to the first or the
        // last inner row has no entry there, so its coupling (the coefficients
        // of :3573-3576 with comp = 1) is taken out of this row.
        if (l == 1 || l == nz - 2) {
            const T ixz = idx * idz, third = T(1.0 / 3.0);
            T drop = 0;
            if (l == 1 && G.BCv[c3 - nxvz - 1] == 2)
                drop += (T(-3) * D.D23[iPrS] * inS * inSWv * wS + D.D31[ixyW] * inSWc * inW * wW -
                         T(2) * D.D32[ixyW] * inSWc * inW * wW) * third * ixz * v[c3 - nxvz - 1];
            if (l == 1 && G.BCv[c3 - nxvz + 1] == 2)
                drop += (T(3) * D.D23[iPrS] * inS * inSEv * wS - D.D31[ixyE] * inE * inSEc * wE +
                         T(2) * D.D32[ixyE] * inE * inSEc * wE) * third * ixz * v[c3 - nxvz + 1];
            if (l == nz - 2 && G.BCv[c3 + nxvz - 1] == 2)
                drop += (T(3) * D.D23[iPrN] * inN * inNWv * wN - D.D31[ixyW] * inNWc * inW * wW +
                         T(2) * D.D32[ixyW] * inNWc * inW * wW) * third * ixz * v[c3 + nxvz - 1];
            if (l == nz - 2 && G.BCv[c3 + nxvz + 1] == 2)
                drop += (T(-3) * D.D23[iPrN] * inN * inNEv * wN + D.D31[ixyE] * inE * inNEc * wE -
                         T(2) * D.D32[ixyE] * inE * inNEc * wE) * third * ixz * v[c3 + nxvz + 1];
            ndrop = drop;
        }
    }
    T grad = (p && G.BCp[iPrS] != 30 && G.BCp[iPrN] != 30) ? (p[iPrN] - p[iPrS]) * idz : T(0);
    return -(inN * TzzN - inS * TzzS) * idz - (inE * TxzE - inW * TxzW) * idx + grad - ndrop;
}

template <typename T, bool NEWTON>
__device__ __forceinline__ T xrow(const stokes_geom &G, const stokes_coefs<T> &D, const stokes_cvec<T> &x, int k,
                                  int l) {
    return xrow<T, NEWTON>(G, D, x, k, l, direct_rates<T>(G, x));
}
template <typename T, bool NEWTON>
__device__ __forceinline__ T zrow(const stokes_geom &G, const stokes_coefs<T> &D, const stokes_cvec<T> &x, int k,
                                  int l) {
    return zrow<T, NEWTON>(G, D, x, k, l, direct_rates<T>(G, x));
}

// continuity row at centroid (k, l)
template <typename T>
__device__ __forceinline__ T crow(const stokes_geom &G, const stokes_cvec<T> &x, int k, int l) {
    const int nx = G.Nx, nxvz = nx + 1;
    const int c1 = k + (l + 1) * nx, c3 = k + l * nxvz + 1;
    const T idx = gc<T>(G, GC_IDX), idz = gc<T>(G, GC_IDZ);
    T r = 0;
    if (G.BCu[c1] != 13) r += -x.u[c1] * idx;
    if (G.BCu[c1 + 1] != 13) r += x.u[c1 + 1] * idx;
    if (G.BCv[c3] != 13) r += -x.v[c3] * idz;
    if (G.BCv[c3 + nxvz] != 13) r += x.v[c3 + nxvz] * idz;
    return r;
}
