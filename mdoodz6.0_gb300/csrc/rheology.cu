// Grid-side rheology kernels: strain rates, centroid<->vertex averaging, the
// local visco-elasto-plastic solve per node and phase with its consistent
// tangent, the rheological operators D11..D34 and the momentum RHS.
//
// Reference behaviour followed (paths inside the MDOODZ 6.0 repository):
//   StrainRateComponents            SOURCE/RheologyDensity.c:1902-1984
//   InterpCentroidsToVerticesDouble SOURCE/GridRoutines.c:106-198
//   InterpVerticesToCentroidsDouble SOURCE/GridRoutines.c:204-228
//   Viscosity                       SOURCE/RheologyDensity.c:44-707
//   NonNewtonianViscosityGrid       SOURCE/RheologyDensity.c:961-1415
//   RheologicalOperators            SOURCE/RheologyDensity.c:713-954
//   EvaluateRHS                     SOURCE/StokesRoutines.c:922-1133
// Isotropic, incompressible, non-reactive subset; the host rejects the rest.
#include <cmath>
#include "mdz_internal.cuh"
#include "mlp.cuh"


#define ZEROC 273.15

// ---------------------------------------------------------------------------
// Strain rates.  One thread per vertex computes exz; one per centroid div, exx, ezz.
__global__ void k_strain_centroids(mdz_dgrid g, const double *__restrict__ u, const double *__restrict__ v,
                                   double *__restrict__ div, double *__restrict__ exx, double *__restrict__ ezz) {
    int c0 = blockIdx.x * blockDim.x + threadIdx.x;
    int ncx = g.ncx, Nx = g.Nx;
    if (c0 >= ncx * g.ncz) return;
    int k = c0 % ncx, l = c0 / ncx, c1 = k + l * Nx, c2 = k + l * (Nx + 1);
    signed char t = g.BCp[c0];
    if (t != 30 && t != 31) {
        double dudx = (u[c1 + 1 + Nx] - u[c1 + Nx]) * g.idx, dvdz = (v[c2 + 1 + (Nx + 1)] - v[c2 + 1]) * g.idz;
        double d = dudx + dvdz;
        div[c0] = d;
        exx[c0] = dudx - 1.0 / 3.0 * d;
        ezz[c0] = dvdz - 1.0 / 3.0 * d;
    } else {
        div[c0] = 0.0; exx[c0] = 0.0; ezz[c0] = 0.0;
    }
}

__global__ void k_strain_vertices(mdz_dgrid g, const double *__restrict__ u, const double *__restrict__ v,
                                  double *__restrict__ exz) {
    int c1 = blockIdx.x * blockDim.x + threadIdx.x;
    int Nx = g.Nx;
    if (c1 >= Nx * g.Nz) return;
    int k = c1 % Nx, l = c1 / Nx, c2 = k + l * (Nx + 1);
    double e = 0.0;
    if (g.BCg[c1] != 30) {
        if (g.BCu[c1] != 30 && g.BCu[c1 + Nx] != 30) e += 0.5 * (u[c1 + Nx] - u[c1]) * g.idz;
        if (g.BCv[c2] != 30 && g.BCv[c2 + 1] != 30) e += 0.5 * (v[c2 + 1] - v[c2]) * g.idx;
    }
    exz[c1] = e;
}

__global__ void k_exz_to_centroids(mdz_dgrid g, const double *__restrict__ exz, double *__restrict__ exz_n) {
    int c0 = blockIdx.x * blockDim.x + threadIdx.x;
    int ncx = g.ncx, Nx = g.Nx;
    if (c0 >= ncx * g.ncz) return;
    int k = c0 % ncx, l = c0 / ncx, c1 = k + l * Nx;
    double e = 0.0, s = 0.0;
    if (g.BCp[c0] != 30 && g.BCp[c0] != 31) {
        if (g.BCg[c1] != 30) { e += exz[c1]; s++; }
        if (g.BCg[c1 + 1] != 30) { e += exz[c1 + 1]; s++; }
        if (g.BCg[c1 + Nx] != 30) { e += exz[c1 + Nx]; s++; }
        if (g.BCg[c1 + Nx + 1] != 30) { e += exz[c1 + Nx + 1]; s++; }
        if (s > 0) e /= s;
    }
    exz_n[c0] = e;
}

// Centroid -> vertex average with the zero-flux padding of the reference:
// the padded ring repeats the nearest interior centroid (corners: diagonal).
__global__ void k_c2v(mdz_dgrid g, const double *__restrict__ cen, double *__restrict__ ver) {
    int c1 = blockIdx.x * blockDim.x + threadIdx.x;
    int Nx = g.Nx, ncx = g.ncx, ncz = g.ncz;
    if (c1 >= Nx * g.Nz) return;
    int k = c1 % Nx, l = c1 / Nx;
    double r = 0.0;
    if (g.BCg[c1] != 30) {
        // padded indices of the four centroids around vertex (k, l): columns k-1, k; rows l-1, l
        int kw = k - 1 < 0 ? 0 : k - 1, ke = k > ncx - 1 ? ncx - 1 : k;
        int ls = l - 1 < 0 ? 0 : l - 1, ln = l > ncz - 1 ? ncz - 1 : l;
        r = 0.25 * (cen[kw + ls * ncx] + cen[ke + ls * ncx] + cen[kw + ln * ncx] + cen[ke + ln * ncx]);
    }
    ver[c1] = r;
}

__global__ void k_v2c(mdz_dgrid g, double *__restrict__ cen, const double *__restrict__ ver) {
    int c0 = blockIdx.x * blockDim.x + threadIdx.x;
    int ncx = g.ncx, Nx = g.Nx;
    if (c0 >= ncx * g.ncz) return;
    int k = c0 % ncx, l = c0 / ncx, c1 = k + l * Nx;
    if (g.BCp[c0] != 30 && g.BCp[c0] != 31) cen[c0] = 0.25 * (ver[c1] + ver[c1 + 1] + ver[c1 + Nx] + ver[c1 + 1 + Nx]);
}

// ---------------------------------------------------------------------------
// Local solve.  Outputs of one (node, phase) solve.
struct visc_res {
    double eta, txx, tzz, txz, etaVE, VEcoeff, Eii_el, Eii_pl, Eii_pwl, Eii_lin, Eii_cst, Eii_exp, Eii_gbs;
    double Exx_el, Ezz_el, Exz_el, Exx_diss, Ezz_diss, Exz_diss, d1;
    double detadexx, detadezz, detadexz, detadp, X1, OverS;
    double ddivpdexx, ddivpdezz, ddivpdexz, ddivpdp, Pcorr, div_el, div_pl;
    double eta_ve, gdot;    // converged local unknowns (training labels of the learned guess)
    double eta_up;          // the reference's start of the visco-elastic iteration
    int ve_fail, vp_fail, ve_its, vp_its;
    int learned, fallback;  // started from a learned guess; polish failed and the plain solve reran
    float lab_x, lab_y;     // the converged solve as a start: ln(eta_ve / eta_up), gdot / (2 Eii)
};

// Polish budget of a learned start: Newton-type updates allowed before the
// plain solve takes over.
#define MDZ_POLISH_STEPS 3

// Precision-generic helpers of the local solve (FP64 or FP32 instances).
__device__ __forceinline__ double msqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float msqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double mexp(double x) { return exp(x); }
__device__ __forceinline__ float mexp(float x) { return expf(x); }
__device__ __forceinline__ double mlog(double x) { return log(x); }
__device__ __forceinline__ float mlog(float x) { return logf(x); }
__device__ __forceinline__ double mfabs(double x) { return fabs(x); }
__device__ __forceinline__ float mfabs(float x) { return fabsf(x); }
__device__ __forceinline__ double msin(double x) { return sin(x); }
__device__ __forceinline__ float msin(float x) { return sinf(x); }
__device__ __forceinline__ void msincos(double x, double *s, double *c) { sincos(x, s, c); }
__device__ __forceinline__ void msincos(float x, float *s, float *c) { sincosf(x, s, c); }
__device__ __forceinline__ double mpow(double x, double y) { return pow(x, y); }
__device__ __forceinline__ float mpow(float x, float y) { return powf(x, y); }

template <typename Real>
__device__ __forceinline__ Real dmin(Real a, Real b) { return a <= b ? a : b; }

// Materials as the local solves read them: the public parameters plus
// lnK_pwl = ln(pref F A^(-1/n) f^(-r/n)), the part of the logarithm of the
// dislocation prefactor B_pwl (Viscosity, SOURCE/RheologyDensity.c:153-154)
// that depends on neither the node nor the iteration.  Taken once per
// launch on the host; NaN where the product is not positive and finite, and the
// solve then multiplies the reference's factors out as they stand.
struct mdz_mat_k : mdz_materials {
    double lnK_pwl[MDZ_MAX_PHASES];
};

static mdz_mat_k mat_k(const mdz_materials &m) {
    mdz_mat_k k;
    static_cast<mdz_materials &>(k) = m;
    for (int p = 0; p < MDZ_MAX_PHASES; p++) {
        double v = NAN;
        const double n = m.npwl[p], pf = m.pref_pwl[p] * m.Fpwl[p], A = m.Apwl[p], f = m.fpwl[p], r = m.rpwl[p];
        if (p < m.n_phases && m.pwlv[p] != 0 && n != 0 && pf > 0 && A > 0 && (r == 0 || f > 0)) {
            v = std::log(pf) - std::log(A) / n;
            if (r != 0) v -= r / n * std::log(f);
            if (!std::isfinite(v)) v = NAN;
        }
        k.lnK_pwl[p] = v;
    }
    return k;
}

// ln(1 + x) by its Mercator series through x^7, for |x| < 1/32 (truncation
// below x^8 / 8 < 2^-43): the Halley update of the learned start needs only
// its root at x = 0 to be exact, and the FP64 logarithm costs several times
// these seven multiply-adds on this part.
__device__ __forceinline__ double ln1p_series(double x) {
    return x * (1.0 + x * (-0.5 + x * (1.0 / 3.0 + x * (-0.25 + x * (0.2 + x * (-1.0 / 6.0 + x * (1.0 / 7.0)))))));
}

// pow with the exponents the creep laws make trivial (0, 1, 2, -1, -2:
// grain-size and melt exponents switched off, linear diffusion creep and its
// tangent, squares) taken exactly; each costs a full FP64 log/exp pair
// otherwise, and FP64 throughput is what bounds the local solves on this part.
template <typename Real, typename Y>
__device__ __forceinline__ Real fpow(Real x, Y y0) {
    const Real y = Real(y0);
    if (y == Real(0)) return Real(1);
    if (y == Real(1)) return x;
    if (y == Real(2)) return x * x;
    if (y == Real(-1)) return Real(1) / x;
    if (y == Real(-2)) return Real(1) / (x * x);
    return mpow(x, y);
}

// exp with the zero argument of switched-off melt weakening taken exactly
template <typename Real>
__device__ __forceinline__ Real fexp(Real x) { return x == Real(0) ? Real(1) : mexp(x); }

template <typename Real>
__device__ void visc_local_t(int p, Real G, Real T, Real P, Real d, Real phi, Real X0, Real Exx,
                           Real Ezz, Real Exz, Real Gxx, Real Gzz, Real Gxz, Real Txx0, Real Tzz0,
                           Real Txz0, const mdz_mat_k &m, const mdz_rheo_params &prm, Real dil, Real fric,
                           Real C, Real P0, Real beta, visc_res &o, const float *guess) {
    const Real R = Real(m.R), dt = Real(prm.dt), tol = sizeof(Real) == 8 ? Real(1.0e-11) : Real(1.0e-4);
    const int nitmax = 20;
    int elastic = prm.iselastic, it;
    const bool constant = Real(m.cstv[p]) != 0, dislocation = Real(m.pwlv[p]) != 0, diffusion = Real(m.linv[p]) != 0;
    // Peierls creep only below 1200 C (tested before the 0 C clamp, :137),
    // grain-boundary sliding, tension cut-off; the learned start models none
    // of them, so their solves take the reference's start
    const bool peierls = m.expv[p] != 0 && T < Real((1200.0 + ZEROC) / prm.scale_T);
    const bool gbs = m.gbsv[p] != 0, tensile = m.is_tensile[p] != 0;
    if (peierls || gbs || tensile) guess = nullptr;
    Real K = Real(1.0) / beta, res = Real(0.0);
    const Real Tii0 = msqrt(Txx0 * Txx0 + Txz0 * Txz0);
    const Real n_pwl = Real(m.npwl[p]), Va_pwl = Real(m.Vpwl[p]), n_lin = Real(m.nlin[p]), m_lin = Real(m.mlin[p]);
    Real B_lin = 0, C_pwl = 0, C_lin = 0, dCpwldP = 0, dClindP = 0;
    Real eta_pwl = Real(0.0), eta_lin = Real(0.0), eta_cst = Real(0.0), eta_vep = Real(0.0), eta_vp = Real(0.0);
    const Real eta_vp0 = Real(m.eta_vp[p]), n_vp = Real(m.n_vp[p]);
    Real Eii_pwl = 0, Eii_lin = 0, Eii_cst = 0, Eii_exp = 0, Eii_gbs = 0;
    o.Eii_pl = Real(0.0); o.OverS = Real(0.0); o.ve_fail = 0; o.vp_fail = 0; o.vp_its = 0;

    Real Eyy = -(Exx + Ezz), Gyy = -(Gxx + Gzz);
    Real Eii = msqrt(Real(1.0) / Real(2.0) * (Exx * Exx + Ezz * Ezz + Eyy * Eyy) + Exz * Exz);
    Real Gii = msqrt(Real(1.0) / Real(2.0) * (Gxx * Gxx + Gzz * Gzz + Gyy * Gyy) + Gxz * Gxz);
    if (Eii * Real(prm.scale_E) < Real(1e-30)) Eii = Real(1e-30) / Real(prm.scale_E);
    if (Gii * Real(prm.scale_E) < Real(1e-30)) Gii = Real(1e-30) / Real(prm.scale_E);
    const Real f_ani = Gii / Eii;
    // reciprocals taken once per solve: an FP64 division is a long instruction
    // sequence on this part, and the reference's formulas divide some fifty
    // times per local solve
    const Real iEii = Real(1.0) / Eii, iGii = Real(1.0) / Gii;
    o.Pcorr = P;
    if (prm.step == 0) elastic = 0;
    o.d1 = Real(m.gs_ref[p]);
    if (elastic == 0) { G = Real(1e1); K = Real(1e1); dil = Real(0.0); }
    if (T < Real(ZEROC) / Real(prm.scale_T)) T = Real(ZEROC) / Real(prm.scale_T);
    const Real iRT = Real(1.0) / (R * T);
    // FP64 dislocation creep in log form: ln B_pwl from the per-phase constant,
    // then C_pwl = (2 f_ani B_pwl)^-n and eta_pwl = B_pwl Eii^(1/n - 1) as two
    // exponentials after one logarithm (the product form takes three pow and an
    // exp), and in the learned polish Eii_pwl = exp(ln C_pwl + n ln Tii) with
    // ln Tii = lnTE + ln eta_ve known.  FP32 keeps the product form: rounding of
    // the logarithms' sums there is at the size of its convergence test.
    const bool logform = sizeof(Real) == 8 && dislocation && isfinite(m.lnK_pwl[p]);
    Real lnC_pwl = Real(0.0), lnTE = Real(0.0), ln_eta_pwl = Real(0.0);
    if (dislocation) {
        const Real in = Real(1.0) / n_pwl;
        if (logform) {
            Real lnB = Real(m.lnK_pwl[p]) + (Real(m.Qpwl[p]) + P * Va_pwl) * iRT * in;
            if (Real(m.mpwl[p]) != Real(0.0)) lnB += Real(m.mpwl[p]) * in * mlog(d);
            if (Real(m.apwl[p]) != Real(0.0)) lnB -= Real(m.apwl[p]) * phi * in;
            // ln(2 f_ani): f_ani = Gii / Eii is 1 up to rounding for isotropic rates,
            // where ln 2 + x - x^2/2 + x^3/3 (x = f_ani - 1, |x| < 2^-20) is exact
            // to rounding and spares an FP64 logarithm
            const Real xf = f_ani - Real(1.0);
            const Real LE = mlog(Eii),
                       LF = mfabs(xf) < Real(9.5367431640625e-07)
                                ? Real(0.69314718055994530942) + xf * (Real(1.0) + xf * (Real(-0.5) + xf * Real(1.0 / 3.0)))
                                : mlog(Real(2.0) * f_ani);   // ln 2; 2^-20
            lnTE = LF + LE;   // ln(2 f_ani Eii) = ln Tii - ln eta_ve
            lnC_pwl = -n_pwl * (LF + lnB);
            C_pwl = mexp(lnC_pwl);
            ln_eta_pwl = lnB + (in - Real(1.0)) * LE;
            eta_pwl = mexp(ln_eta_pwl);
        } else {
            Real B_pwl = Real(m.pref_pwl[p]) * Real(m.Fpwl[p]) * fpow(Real(m.Apwl[p]), -in) * mexp((Real(m.Qpwl[p]) + P * Va_pwl) * iRT * in) *
                           fpow(d, Real(m.mpwl[p]) * in) * fpow(Real(m.fpwl[p]), -Real(m.rpwl[p]) * in) * fexp(-Real(m.apwl[p]) * phi * in);
            C_pwl = fpow(Real(2.0) * f_ani * B_pwl, -n_pwl);
            eta_pwl = B_pwl * fpow(Eii, in - Real(1.0));
        }
        dCpwldP = -C_pwl * Va_pwl * iRT;
    }
    if (diffusion) {
        const Real in = Real(1.0) / n_lin;
        B_lin = Real(m.Flin[p]) * fpow(Real(m.Alin[p]), -in) * mexp((Real(m.Qlin[p]) + P * Real(m.Vlin[p])) * iRT * in) *
                fpow(Real(m.flin[p]), -Real(m.rlin[p]) * in) * fexp(-Real(m.alin[p]) * phi * in);
        C_lin = fpow(Real(2.0) * f_ani * B_lin, -n_lin);
        dClindP = -C_lin * Real(m.Vlin[p]) * iRT;
        eta_lin = B_lin * fpow(Eii, in - Real(1.0)) * fpow(d, m_lin * in);
    }
    // grain-boundary sliding: a creep law of the dislocation form (:176-180)
    const Real n_gbs = Real(m.ngbs[p]);
    Real C_gbs = Real(0.0), eta_gbs = Real(0.0);
    if (gbs) {
        const Real in = Real(1.0) / n_gbs;
        const Real B_gbs = Real(m.Fgbs[p]) * fpow(Real(m.Agbs[p]), -in) *
                           mexp((Real(m.Qgbs[p]) + P * Real(m.Vgbs[p])) * iRT * in) * fpow(d, Real(m.mgbs[p]) * in) *
                           fpow(Real(m.fgbs[p]), -Real(m.rgbs[p]) * in) * fexp(-Real(m.agbs[p]) * phi * in);
        C_gbs = fpow(Real(2.0) * f_ani * B_gbs, -n_gbs);
        eta_gbs = B_gbs * fpow(Eii, in - Real(1.0));
    }
    // Peierls creep, exponential law as a power law of exponent ST + n
    // (:181-199): ST = Q / RT 2 gamma (1 - gamma)
    const Real n_exp = Real(m.nexp[p]);
    Real ST = Real(0.0), B_exp = Real(0.0), C_exp = Real(0.0), eta_exp = Real(0.0);
    if (peierls) {
        const Real gam = Real(m.Gexp[p]), Ea = Real(m.Qexp[p]);
        ST = Ea * iRT * Real(2.0) * gam * (Real(1.0) - gam);
        const Real sn = ST + n_exp, isn = Real(1.0) / sn;
        const Real Arr = mexp(-Ea * iRT * (Real(1.0) - gam) * (Real(1.0) - gam));
        const Real F_exp = mpow(mpow(Real(2.0), Real(1.0) - ST - n_exp) / mpow(msqrt(Real(3.0)), sn + Real(1.0)), isn);
        B_exp = F_exp * (mpow(gam * Real(m.Sexp[p]), ST * isn) / mpow(Real(m.Eexp[p]) * Arr, isn));
        C_exp = mpow(Real(2.0) * f_ani * B_exp, -sn);
        eta_exp = B_exp * mpow(Eii, isn - Real(1.0));
    }
    Real cos_fric, sin_fric;
    msincos(fric, &sin_fric, &cos_fric);
    Real sin_dil = dil == Real(0.0) ? Real(0.0) : msin(dil);
    Real Tyield = C * cos_fric + P * sin_fric;
    if (Real(m.Slim[p]) < Tyield) { sin_fric = Real(0.0); cos_fric = Real(1.0); sin_dil = Real(0.0); C = Real(m.Slim[p]); Tyield = Real(m.Slim[p]); }
    // tension cut-off (:204-213): below the tension pressure -25 MPa the yield
    // line turns to pass through (P_tens, 0)
    bool tens = false;
    if (tensile) {
        const Real P_tens = Real(-25e6) / Real(prm.scale_S);
        const Real sin_fric_tens = -C * cos_fric / P_tens;
        if (C * cos_fric + P * sin_fric_tens < Tyield) {
            sin_fric = sin_fric_tens;
            Tyield = C * cos_fric + P * sin_fric_tens;
            tens = true;
        }
    }
    o.X1 = X0;
    const Real eta_el = G * dt;
    if (constant) eta_cst = Real(m.eta0[p]);
    Real eta_up = Real(1.0e100) / Real(prm.scale_eta);
    if (constant) eta_up = dmin(eta_up, eta_cst);
    if (dislocation) eta_up = dmin(eta_up, eta_pwl);
    if (elastic) eta_up = dmin(eta_up, eta_el);
    if (peierls) eta_up = dmin(eta_up, eta_exp);
    if (diffusion) eta_up = dmin(eta_up, eta_lin);
    if (gbs) eta_up = dmin(eta_up, eta_gbs);
    // local Newton on the visco-elastic viscosity
    Real eta_ve = eta_up, Tii;
    const Real dm_lin = fpow(o.d1, -m_lin);
    bool ve_done = false;
    o.eta_up = eta_up;
    o.learned = guess != nullptr;
    o.fallback = 0;
    const Real i2eta_el = Real(0.5) / eta_el, ifcst = constant ? Real(0.5) / (f_ani * eta_cst) : Real(0.0);
    if (guess) {
        // Learned start s = mlog(eta_ve), polished by Halley steps on
        // g(s) = mlog(sum of the strain rates) - mlog(Eii): every mechanism's
        // rate is c_k mexp(n_k s), so g' and g'' are rate-weighted means of n_k
        // and n_k^2 (in s the residual is nearly linear; Halley in eta itself
        // left 39 % of the solves unconverged after two steps).  Converged
        // means the reference's own test below holds.  The network predicts
        // ln(eta_ve / eta_up), eta_up being the reference's start (the
        // smallest viscosity of the active mechanisms).
        Real s = (logform && eta_up == eta_pwl ? ln_eta_pwl : mlog(eta_up)) + (Real)guess[0];
        for (it = 0; it <= MDZ_POLISH_STEPS; it++) {
            eta_ve = mexp(s);
            Tii = Real(2.0) * f_ani * eta_ve * Eii;
            const Real Eel = elastic ? Tii * i2eta_el : Real(0.0);
            if (constant) Eii_cst = Tii * ifcst;
            if (dislocation) Eii_pwl = logform ? mexp(lnC_pwl + n_pwl * (lnTE + s)) : C_pwl * fpow(Tii, n_pwl);
            if (diffusion) Eii_lin = C_lin * fpow(Tii, n_lin) * dm_lin;
            const Real S0 = Eel + Eii_pwl + Eii_lin + Eii_cst;
            res = mfabs((Eii - S0) * iEii);
            // a start is accepted only after one update: a warm start can
            // pass the test as it stands, with an error the size of the change
            // in strain rate since it was recorded (the reference's iteration
            // always ends one quadratic step past the test)
            if (it > 0 && res < tol / 100) { ve_done = true; break; }
            if (it == MDZ_POLISH_STEPS) break;
            if (!(S0 > Real(0.0))) break;
            const Real S1 = Eel + n_pwl * Eii_pwl + n_lin * Eii_lin + Eii_cst;
            const Real S2 = Eel + n_pwl * n_pwl * Eii_pwl + n_lin * n_lin * Eii_lin + Eii_cst;
            const Real iS0 = Real(1.0) / S0;
            const Real q = S0 * iEii;
            const Real g = (sizeof(Real) == 8 && mfabs(q - Real(1.0)) < Real(0.03125)) ? Real(ln1p_series(double(q - Real(1.0)))) : mlog(q);
            const Real g1 = S1 * iS0, g2 = S2 * iS0 - g1 * g1;
            const Real den = Real(2.0) * g1 * g1 - g * g2;
            s -= den > Real(0.0) ? Real(2.0) * g * g1 / den : g / g1;
        }
        o.ve_its = it;
        if (!ve_done) {
            o.fallback = 1;
            eta_ve = eta_up;
            Eii_pwl = 0; Eii_lin = 0; Eii_cst = 0;
        }
    }
    const Real dfel = elastic ? -Eii / eta_el : Real(0.0), dfcst = constant ? -Eii / eta_cst : Real(0.0);
    for (it = 0; !ve_done && it < nitmax; it++) {
        Tii = Real(2.0) * f_ani * eta_ve * Eii;
        if (constant) Eii_cst = Tii * ifcst;
        if (dislocation) Eii_pwl = C_pwl * fpow(Tii, n_pwl);
        if (gbs) Eii_gbs = C_gbs * fpow(Tii, n_gbs);
        if (peierls) Eii_exp = C_exp * mpow(Tii, ST + n_exp);
        if (diffusion) Eii_lin = C_lin * fpow(Tii, n_lin) * dm_lin;
        Real r = Eii - elastic * Tii * i2eta_el - (Eii_pwl + Eii_exp + Eii_lin + Eii_gbs + Eii_cst);
        res = mfabs(r * iEii);
        if (res < tol / 100) break;
        const Real ieta = Real(1.0) / eta_ve;
        Real dfdeta = dfel + dfcst;
        // (grain-boundary sliding has no term here in the reference)
        if (peierls) dfdeta += -Eii_exp * (ST + n_exp) * ieta;
        if (diffusion) dfdeta += -Eii_lin * n_lin * ieta;
        if (dislocation) dfdeta += -Eii_pwl * n_pwl * ieta;
        eta_ve -= r / dfdeta;
    }
    if (!ve_done) {   // iterations of a failed polish count too
        o.ve_its = it + (guess ? MDZ_POLISH_STEPS : 0);
        if (it == nitmax - 1 && res > tol) o.ve_fail = 1;
    }
    o.eta_ve = eta_ve;
    // Eii_pwl = C_pwl Tii^n_pwl was evaluated at the final eta_ve when the
    // iteration stopped on its convergence test (not when it ran out): then
    // Tii^n_pwl is Eii_pwl / C_pwl, and the powers of Tii below follow from it
    // without another FP64 pow each
    const bool pwl_fresh = dislocation && (ve_done || res < tol / 100) && C_pwl > Real(0.0) && Eii_pwl > Real(0.0);
    Tii = Real(2.0) * eta_ve * f_ani * Eii;
    const Real Tn = !dislocation ? Real(0.0) : (pwl_fresh ? Eii_pwl / C_pwl : fpow(Tii, n_pwl));   // Tii^n_pwl
    const Real iTii = Real(1.0) / Tii, TG = Tii * iGii;   // Tii / (f_ani Eii) = Tii / Gii
    Real Txx = Gxx * TG, Tzz = Gzz * TG, Txz = Gxz * TG;
    Real Exx_lin = 0, Ezz_lin = 0, Exz_lin = 0, Exx_cst = 0, Ezz_cst = 0, Exz_cst = 0;
    Real Exx_exp = 0, Ezz_exp = 0, Exz_exp = 0;
    if (peierls) {
        eta_exp = B_exp * mpow(Eii_exp, Real(1.0) / (ST + n_exp) - Real(1.0));
        const Real h = Real(0.5) / eta_exp;
        Exx_exp = Txx * h; Ezz_exp = Tzz * h; Exz_exp = Txz * h;
    }
    if (dislocation) eta_pwl = Tii / (Real(2.0) * C_pwl * Tn);   // (2 C)^-1 Tii^(1-n)
    if (diffusion) {
        const Real in = Real(1.0) / n_lin;
        eta_lin = B_lin * fpow(Eii_lin, in - Real(1.0)) * fpow(o.d1, m_lin * in);
        const Real h = Real(0.5) / eta_lin;
        Exx_lin = Txx * h; Ezz_lin = Tzz * h; Exz_lin = Txz * h;
    }
    if (constant) {
        const Real h = Real(0.5) / eta_cst;
        Exx_cst = Txx * h; Ezz_cst = Tzz * h; Exz_cst = Txz * h;
    }
    // visco-elastic tangent
    Real deta = Real(0.0);
    if (dislocation) deta += -C_pwl * (Tn * iTii * iTii * iTii) * (n_pwl - Real(1.0));   // Tii^(n-3)
    if (peierls) deta += -C_exp * mpow(Tii, n_exp + ST - Real(3.0)) * (n_exp + ST - Real(1.0));
    if (diffusion) deta += -C_lin * fpow(Tii, n_lin - Real(3.0)) * (n_lin - Real(1.0)) * dm_lin;
    const Real e2 = fpow(eta_ve, Real(2.0));
    Real dTxx = deta * (Real(2.0) * Txx + Tzz) * e2, dTzz = deta * (Real(2.0) * Tzz + Txx) * e2, dTxz = Real(2.0) * deta * Txz * e2;
    Real den = Real(1.0) - Real(2.0) * (dTxx * Exx + dTzz * Ezz + dTxz * Exz);
    const Real e2den = Real(2.0) * eta_ve / den;
    Real dve_dExx = dTxx * e2den, dve_dEzz = dTzz * e2den;
    Real dve_dExz = dTxz * e2den;
    Real dummy = Real(0.0), Jii = Tii * Tii;
    if (dislocation) dummy += -Real(2.0) * (Tn * iTii) * dCpwldP;   // Jii^((n-1)/2) = Tii^(n-1)
    if (diffusion) dummy += -Real(2.0) * fpow(Jii, (Real(1.0) / Real(2.0)) * n_lin - Real(1.0) / Real(2.0)) * fpow(d, -m_lin) * dClindP;
    Real dve_dP = fpow(eta_ve, 2) * dummy;
    // plastic return mapping on gdot
    Real gdot = Real(0.0), dQdtxx = 0, dQdtzz = 0, dQdtxz = 0, dQdP = 0, divp = Real(0.0), Pc = P;
    Real dlamdExx = 0, dlamdEzz = 0, dlamdExz = 0, dlamdP = 0;
    Real dvep_dExx = 0, dvep_dEzz = 0, dvep_dExz = 0, dvep_dP = 0;
    Real F_trial = Tii - Tyield;
    // tensile domain: the dilation angle that returns the stress to the
    // tension corner (:456-465, SimpleYields.m of the reference)
    if (tens) {
        eta_vp = eta_vp0 * fpow(Eii, Real(1.0) / n_vp - Real(1.0));
        const Real Pc_chk = -(C * cos_fric) / (-Tii / P + sin_fric);
        sin_dil = (P * eta_ve + P * eta_vp - Pc_chk * eta_ve - Pc_chk * eta_vp) /
                  (K * dt * (C * cos_fric + Pc_chk * sin_fric - Tii));
    }
    const bool is_pl = F_trial > Real(1e-17);
    Real dsdExx = Real(0.0), dsdEzz = Real(0.0), dsdExz = Real(0.0), dsdP = Real(0.0);   // d sin_dil / d .
    if (is_pl) {
        const Real in_vp = Real(1.0) / n_vp;
        eta_vp = eta_vp0 * fpow(Eii, in_vp - 1);
        gdot = F_trial / (eta_ve + eta_vp + K * dt * sin_fric * sin_dil);
        dQdtxx = Txx * Real(0.5) * iTii; dQdtzz = Tzz * Real(0.5) * iTii; dQdtxz = Txz * iTii;
        const Real F_trial0 = F_trial, iF0 = Real(1.0) / F_trial0;
        bool vp_done = false;
        if (guess) {
            // learned start: gdot = fraction * 2 Eii, at most MDZ_POLISH_STEPS
            // Newton updates, the reference's own convergence test
            Real frac = (Real)guess[1];
            frac = frac > Real(1e-6) ? (frac < Real(1.0) ? frac : Real(1.0)) : Real(1e-6);
            const Real gdot_plain = gdot;
            gdot = frac * Real(2.0) * Eii;
            for (it = 0; it <= MDZ_POLISH_STEPS; it++) {
                dQdP = -sin_dil;
                divp = -gdot * dQdP;
                Pc = P + K * dt * divp;
                eta_vp = eta_vp0 * fpow(mfabs(gdot), in_vp - Real(1.0));
                Tyield = C * cos_fric + Pc * sin_fric + gdot * eta_vp;
                F_trial = Tii - eta_ve * gdot - Tyield;
                res = mfabs(F_trial);
                if (it > 0 && (res < tol || res * iF0 < tol)) { vp_done = true; break; }
                if (it == MDZ_POLISH_STEPS) break;
                Real dFdgdot = -eta_ve - eta_vp * in_vp - K * dt * sin_fric * sin_dil;
                gdot -= F_trial / dFdgdot;
            }
            o.vp_its = it;
            if (!vp_done) {
                o.fallback = 1;
                gdot = gdot_plain;
            }
        }
        for (it = 0; !vp_done && it < nitmax; it++) {
            dQdP = -sin_dil;
            divp = -gdot * dQdP;
            Pc = P + K * dt * divp;
            eta_vp = eta_vp0 * fpow(mfabs(gdot), in_vp - Real(1.0));
            Tyield = C * cos_fric + Pc * sin_fric + gdot * eta_vp;
            F_trial = Tii - eta_ve * gdot - Tyield;
            res = mfabs(F_trial);
            if (res < tol || res * iF0 < tol) break;
            Real dFdgdot = -eta_ve - eta_vp * in_vp - K * dt * sin_fric * sin_dil;
            gdot -= F_trial / dFdgdot;
        }
        if (!vp_done) {
            o.vp_its = it + (guess ? MDZ_POLISH_STEPS : 0);
            if (it == nitmax - 1 && (res > tol || res * iF0 > tol)) o.vp_fail = 1;
        }
        Txx = Real(2.0) * eta_ve * (Exx - gdot * dQdtxx);
        Tzz = Real(2.0) * eta_ve * (Ezz - gdot * dQdtzz);
        Real Tyy = -(Txx + Tzz);
        Txz = Real(2.0) * eta_ve * (Exz - gdot * dQdtxz / Real(2.0));
        Tii = msqrt(Real(0.5) * (fpow(Txx, Real(2.0)) + fpow(Tzz, Real(2.0)) + fpow(Tyy, Real(2.0))) + fpow(Txz, Real(2.0)));
        eta_vep = Tii * Real(0.5) * iEii;
        o.Eii_pl = gdot / Real(2.0);
        Tii = Real(2.0) * eta_vep * Eii;
        o.OverS = eta_vp * gdot;
        o.Pcorr = Pc;
        // visco-elasto-plastic tangent
        if (tens) {   // derivatives of the tensile dilation angle (:578-587)
            const Real dEii_dExx = (Real(2.0) * Exx + Ezz) * Real(0.5) * iEii, dEii_dEzz = (Real(2.0) * Ezz + Exx) * Real(0.5) * iEii;
            const Real dEii_dExz = Exz * iEii;
            const Real Ccf = C * cos_fric, A = Real(2.0) * Eii * eta_ve - P * sin_fric, A2 = A * A;
            const Real iden = Real(1.0) / (K * dt * A * (C * P * cos_fric * sin_fric + (Ccf - Real(2.0) * Eii * eta_ve) * A));
            const Real Q = C * P * cos_fric * sin_fric + A2;
            auto dsd = [&](Real dve, Real dE) {
                const Real dT = Eii * dve + dE * eta_ve;
                return (Real(2.0) * K * dt * sin_dil * dT * Q +
                        P * (-Ccf * dve * A + Real(2.0) * Ccf * (eta_ve + eta_vp) * dT + dve * A2)) * iden;
            };
            dsdExx = dsd(dve_dExx, dEii_dExx);
            dsdEzz = dsd(dve_dEzz, dEii_dEzz);
            dsdExz = dsd(dve_dExz, dEii_dExz);
            dsdP = (Real(2.0) * C * Eii * cos_fric * (eta_ve + eta_vp) * (P * dve_dP - eta_ve) - C * P * cos_fric * dve_dP * A +
                    Real(2.0) * Eii * K * dt * sin_dil * (C * cos_fric * sin_fric * (P * dve_dP - eta_ve) + dve_dP * A2) +
                    A2 * (P * dve_dP + eta_ve + eta_vp)) * iden;
        }
        const Real ev = eta_ve * iEii;
        Real dFdExx = (Real(2.0) * Exx + Ezz) * ev + Real(2.0) * Eii * dve_dExx;
        Real dFdEzz = (Real(2.0) * Ezz + Exx) * ev + Real(2.0) * Eii * dve_dEzz;
        Real dFdExz = Real(2.0) * Exz * ev + Real(2.0) * Eii * dve_dExz;
        Real dFdP = -sin_fric + Real(2.0) * Eii * dve_dP;
        Real gg = Real(1.0) / (eta_ve + eta_vp * in_vp + K * dt * sin_fric * sin_dil);
        dlamdExx = gg * (dFdExx - gdot * (dve_dExx + K * dt * sin_fric * dsdExx));
        dlamdEzz = gg * (dFdEzz - gdot * (dve_dEzz + K * dt * sin_fric * dsdEzz));
        dlamdExz = gg * (dFdExz - gdot * (dve_dExz + K * dt * sin_fric * dsdExz));
        dlamdP = gg * (dFdP - gdot * (dve_dP + K * dt * sin_fric * dsdP));
        Real q = in_vp - Real(1.0);
        const Real evg = eta_vp / gdot;
        Real dvp_dExx = evg * dlamdExx * q, dvp_dEzz = evg * dlamdEzz * q;
        Real dvp_dExz = evg * dlamdExz * q, dvp_dP = evg * dlamdP * q;
        Real a = eta_vp + K * dt * sin_fric * sin_dil;
        const Real TyE3 = Tyield * Real(0.5) * iEii * iEii * iEii, h2 = Real(0.5) * iEii;   // Tyield / (2 Eii^3), 1 / (2 Eii)
        dvep_dExx = -Real(0.5) * (Real(2.0) * Exx + Ezz) * TyE3 + (a * dlamdExx + gdot * dvp_dExx + gdot * K * dt * sin_fric * dsdExx) * h2;
        dvep_dEzz = -Real(0.5) * (Real(2.0) * Ezz + Exx) * TyE3 + (a * dlamdEzz + gdot * dvp_dEzz + gdot * K * dt * sin_fric * dsdEzz) * h2;
        dvep_dExz = -Exz * TyE3 + (a * dlamdExz + gdot * dvp_dExz + gdot * K * dt * sin_fric * dsdExz) * h2;
        dvep_dP = (sin_fric + a * dlamdP + gdot * dvp_dP + gdot * K * dt * sin_fric * dsdP) * h2;
    }
    o.gdot = gdot;
    Real inv_eta_diss = Real(0.0);
    if (peierls) inv_eta_diss += Real(1.0) / eta_exp;
    if (dislocation) inv_eta_diss += Real(1.0) / eta_pwl;
    if (diffusion) inv_eta_diss += Real(1.0) / eta_lin;
    if (constant) inv_eta_diss += Real(1.0) / eta_cst;
    if (!is_pl) {
        o.detadexx = dve_dExx; o.detadezz = dve_dEzz; o.detadexz = dve_dExz; o.detadp = dve_dP;
        o.etaVE = eta_ve;
        o.ddivpdexx = Real(0.0); o.ddivpdezz = Real(0.0); o.ddivpdexz = Real(0.0); o.ddivpdp = Real(0.0);
    } else {
        o.detadexx = dvep_dExx; o.detadezz = dvep_dEzz; o.detadexz = dvep_dExz; o.detadp = dvep_dP;
        o.etaVE = eta_vep;
        o.ddivpdexx = -dQdP * dlamdExx + gdot * dsdExx;
        o.ddivpdezz = -dQdP * dlamdEzz + gdot * dsdEzz;
        o.ddivpdexz = -dQdP * dlamdExz + gdot * dsdExz;
        o.ddivpdp = -dQdP * dlamdP + gdot * dsdP + Real(0.0);
        inv_eta_diss += Real(1.0) / eta_vep;
    }
    // eta_pwl is re-evaluated unconditionally in the reference (C_pwl = 0 when
    // dislocation creep is off, which makes the dislocation parts vanish); Tii
    // is still the visco-elastic one unless the plastic branch changed it
    // 1 / (2 eta_pwl) = C_pwl Tii^(n-1): no division of the reference's
    // fpow(2 C_pwl, -1) fpow(Tii, 1 - n) is needed where Tii^n is known
    const Real h_pwl = !(C_pwl > Real(0.0)) ? Real(0.0) : (dislocation && !is_pl ? C_pwl * Tn * iTii : C_pwl * fpow(Tii, n_pwl - Real(1.0)));
    eta_pwl = Real(0.5) / h_pwl;
    o.Exx_el = (Real)elastic * (Txx - Txx0) * i2eta_el;
    o.Ezz_el = (Real)elastic * (Tzz - Tzz0) * i2eta_el;
    o.Exz_el = (Real)elastic * (Txz - Txz0) * i2eta_el;
    o.Exx_diss = gdot * dQdtxx + Exx_lin + Txx * h_pwl + Exx_exp + Exx_cst;
    o.Ezz_diss = gdot * dQdtzz + Ezz_lin + Tzz * h_pwl + Ezz_exp + Ezz_cst;
    o.Exz_diss = gdot * dQdtxz / Real(2.0) + Exz_lin + Txz * h_pwl + Exz_exp + Exz_cst;
    o.Eii_el = (Real)elastic * mfabs(Tii - Tii0) * i2eta_el;
    o.Eii_pwl = Tii * h_pwl;
    o.Eii_lin = Eii_lin;
    o.Eii_cst = Eii_cst;
    o.Eii_exp = Eii_exp;
    o.Eii_gbs = Eii_gbs;
    o.div_pl = divp;
    o.div_el = -(Pc - P0) / (K * dt);
    Real eta = Real(1.0) / inv_eta_diss;
    o.VEcoeff = elastic == 0 ? Real(0.0) : Real(2.0) * eta_ve * i2eta_el;
    if (prm.step == 0) o.etaVE = eta;
    o.txx = Txx; o.tzz = Tzz; o.txz = Txz;
    if (eta > Real(prm.maxeta)) eta = Real(prm.maxeta);
    if (eta < Real(prm.mineta)) eta = Real(prm.mineta);
    const bool clamped = o.etaVE > Real(prm.maxeta) || o.etaVE < Real(prm.mineta);
    if (o.etaVE > Real(prm.maxeta)) o.etaVE = Real(prm.maxeta);
    if (o.etaVE < Real(prm.mineta)) o.etaVE = Real(prm.mineta);
    if (clamped && prm.clamp_tangent) {   // the limiter is flat: its tangent is zero
        o.detadexx = Real(0.0); o.detadezz = Real(0.0); o.detadexz = Real(0.0); o.detadp = Real(0.0);
    }
    o.eta = eta;
    // the start the next evaluation of this (node, phase) can polish from, in
    // the learned guess's encoding; FP32 logarithms suffice for a start
    o.lab_x = logf((float)eta_ve) - logf((float)o.eta_up);
    o.lab_y = (float)(gdot * Real(0.5) * iEii);
}


// The reference's local solve in FP64 (all call sites but the inexact FP32
// evaluations of k_viscosity_* use this one).
__device__ __forceinline__ void visc_local(int p, double G, double T, double P, double d, double phi, double X0,
                                           double Exx, double Ezz, double Exz, double Gxx, double Gzz, double Gxz,
                                           double Txx0, double Tzz0, double Txz0, const mdz_mat_k &m,
                                           const mdz_rheo_params &prm, double dil, double fric, double C, double P0,
                                           double beta, visc_res &o, const float *guess = nullptr) {
    visc_local_t<double>(p, G, T, P, d, phi, X0, Exx, Ezz, Exz, Gxx, Gzz, Gxz, Txx0, Tzz0, Txz0, m, prm, dil, fric,
                         C, P0, beta, o, guess);
}

// One (node, phase) local solve: in FP32 when asked (an inexact evaluation
// for a non-linear iteration far from convergence; FP64 transcendental
// functions issue at a small fraction of the FP32 rate on this part), with
// the FP64 solve taking over wherever the FP32 one failed or overflowed;
// otherwise the FP64 solve, from the learned start when one is given.
__device__ __forceinline__ void visc_node_phase(bool fp32, int p, double G, double T, double P, double d, double phi,
                                                double X0, const double *E, double Txx0, double Tzz0, double Txz0,
                                                const mdz_mat_k &m, const mdz_rheo_params &prm, double dil,
                                                double fric, double C, double P0, double beta, visc_res &o,
                                                const float *guess) {
    if (fp32) {
        visc_local_t<float>(p, (float)G, (float)T, (float)P, (float)d, (float)phi, (float)X0, (float)E[0],
                            (float)E[1], (float)E[2], (float)E[3], (float)E[4], (float)E[5], (float)Txx0,
                            (float)Tzz0, (float)Txz0, m, prm, (float)dil, (float)fric, (float)C, (float)P0,
                            (float)beta, o, nullptr);
        const bool ok = !o.ve_fail && !o.vp_fail && isfinite(o.eta) && isfinite(o.etaVE) && isfinite(o.txx) &&
                        isfinite(o.tzz) && isfinite(o.txz) && isfinite(o.detadexx) && isfinite(o.detadezz) &&
                        isfinite(o.detadexz) && isfinite(o.detadp) && isfinite(o.Pcorr);
        if (ok) return;
    }
    visc_local(p, G, T, P, d, phi, X0, E[0], E[1], E[2], E[3], E[4], E[5], Txx0, Tzz0, Txz0, m, prm, dil, fric, C,
               P0, beta, o, guess);
}

// Effective rates entering the local solve (isotropic form of the elastic
// stress correction, NonNewtonianViscosityGrid :1060-1094): E[0..2] Exx, Ezz,
// Exz and E[3..5] Gxx, Gzz, Gxz, with the reference's inverse of Da evaluated
// for ani = 0 (iDa11 = iDa22 = 1/2, iDa33 = 1, off-diagonals 0).
__device__ __forceinline__ void eff_rates(double exx, double ezz, double exz, double sxx0, double szz0, double sxz0,
                                          double etae, double *E) {
    const double i11 = 0.5, i22 = 0.5, i33 = 1.0, z = 0.0, ie = 1.0 / etae;   // one division, not four
    double Exx = exx + (i11 * sxx0 + z * szz0 + z * sxz0) * ie;
    double Ezz = ezz + (z * sxx0 + i22 * szz0 + z * sxz0) * ie;
    double Exz = exz + (z * sxx0 + z * szz0 + i33 * sxz0) * 0.5 * ie;
    double gxz = 2.0 * exz + (z * sxx0 + z * szz0 + i33 * sxz0) * ie;
    E[0] = Exx; E[1] = Ezz; E[2] = Exz;
    E[3] = Exx * 1.0 + Ezz * z + gxz * z;
    E[4] = Ezz * 1.0 + Exx * z - gxz * z;
    E[5] = Exx * z - Exx * z + gxz * 0.5;
}

__device__ __forceinline__ void put(double *p, int i, double v) {
    if (p) p[i] = v;
}

// Counters of the local solves: [0] not converged, [1] learned starts whose
// polish failed (plain solve rerun), [2] learned starts (int32), and at int
// offset 48 the 64-bit total of local Newton iterations (visco-elastic plus
// plastic); warp-aggregated atomics.
__device__ __forceinline__ void count_local(int *counters, int fails, int fallbacks, int learned, int iters) {
    if (!counters) return;
    const unsigned mask = __activemask();
    const int lane = threadIdx.x & 31, leader = __ffs(mask) - 1;
    const int a = __reduce_add_sync(mask, fails), b = __reduce_add_sync(mask, fallbacks),
              c = __reduce_add_sync(mask, learned), d = __reduce_add_sync(mask, iters);
    if (lane == leader) {
        if (a) atomicAdd(&counters[0], a);
        if (b) atomicAdd(&counters[1], b);
        if (c) atomicAdd(&counters[2], c);
        if (d) atomicAdd(reinterpret_cast<unsigned long long *>(counters + 48), (unsigned long long)d);
    }
}

// One thread per centroid: loop over phases with a fraction above 1e-13.
__global__ void __launch_bounds__(128) k_viscosity_centroids(mdz_dgrid g, mdz_mat_k m, mdz_rheo_params prm,
                                                             mdz_fields f, int *__restrict__ counters,
                                                             const float2 *guess, float2 *labels, int fp32) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    int nc = g.ncx * g.ncz;
    if (c >= nc) return;
    const int avg = prm.eta_avg, nph = m.n_phases;
    double eta = 0, eta_phys = 0, VE = 0, sxx = 0, szz = 0, sxz = 0, eel = 0, epl = 0, epwl = 0, elin = 0, ecst = 0,
           eexp = 0, egbs = 0,
           dn = 0, xel = 0, xdi = 0, zel = 0, zdi = 0, dexx = 0, dezz = 0, dgxz = 0, dp = 0, vxx = 0, vzz = 0,
           vxz = 0, vp = 0, pc = 0, del = 0, dpl = 0, Wt = 0, We = 0, Wd = 0, X = 0, OS = 0;
    int fails = 0, fallbacks = 0, learned = 0, iters = 0;
    signed char t = g.BCp[c];
    if (t != 30 && t != 31) {
        const double etae = prm.iselastic == 1 ? prm.dt * f.mu_n[c] : 1.0;
        const double exx = f.exxd[c], ezz = f.ezzd[c], exz = f.exz_n[c];
        const double sxx0 = f.sxxd0[c], szz0 = f.szzd0[c], sxz0 = f.sxz0_n[c];
        double E[6];
        eff_rates(exx, ezz, exz, sxx0, szz0, sxz0, etae, E);
        const double mu = f.mu_n[c], T = f.T[c], P = f.p[c], d0 = f.d0_n[c], phi0 = f.phi0_n[c];
        const double X0 = f.X0_n ? f.X0_n[c] : 0.0, P0 = f.p0_n ? f.p0_n[c] : 0.0;
        const double dil = f.dil_n[c], fric = f.fric_n[c], Coh = f.C_n[c], bet = f.bet_n[c];
        for (int p = 0; p < nph; p++) {
            double w = f.phase_perc_n[(size_t)p * nc + c];
            if (!(fabs(w) > 1.0e-13)) continue;
            visc_res o;
            float gs[2];
            if (guess) {
                const float2 q = guess[(size_t)p * nc + c];
                gs[0] = q.x; gs[1] = q.y;
            }
            visc_node_phase(fp32 != 0, p, mu, T, P, d0, phi0, X0, E, sxx0, szz0, sxz0, m, prm, dil, fric, Coh, P0, bet, o,
                            guess ? gs : nullptr);
            // labels may be the guess buffer itself: this thread read its entry above
            if (labels) labels[(size_t)p * nc + c] = make_float2(o.lab_x, o.lab_y);
            fails += o.ve_fail + o.vp_fail;
            fallbacks += o.fallback;
            iters += o.ve_its + o.vp_its;
            learned += o.learned;
            if (avg == 0) {
                eta += w * o.etaVE; eta_phys += w * o.eta; dexx += w * o.detadexx; dezz += w * o.detadezz;
                dgxz += w * o.detadexz / 2.0; dp += w * o.detadp;
            }
            if (avg == 0 || avg == 2) { sxx += w * o.txx; szz += w * o.tzz; sxz += w * o.txz; }
            VE += w * o.VEcoeff; eel += w * o.Eii_el; epl += w * o.Eii_pl; epwl += w * o.Eii_pwl;
            elin += w * o.Eii_lin; ecst += w * o.Eii_cst; dn += w * 1.0 / o.d1;
            eexp += w * o.Eii_exp; egbs += w * o.Eii_gbs;
            xel += w * o.Exx_el; xdi += w * o.Exx_diss; zel += w * o.Ezz_el; zdi += w * o.Ezz_diss;
            Wt += w * (o.txx * exx + o.tzz * ezz + (o.txx + o.tzz) * (exx + ezz) + 2.0 * o.txz * exz);
            Wd += w * (o.txx * o.Exx_diss + o.tzz * o.Ezz_diss + (o.txx + o.tzz) * (o.Exx_diss + o.Ezz_diss) +
                       2.0 * o.txz * o.Exz_diss);
            We += w * (o.txx * o.Exx_el + o.tzz * o.Ezz_el + (o.txx + o.tzz) * (o.Exx_el + o.Ezz_el) +
                       2.0 * o.txz * o.Exz_el);
            vxx += w * o.ddivpdexx; vzz += w * o.ddivpdezz; vxz += w * o.ddivpdexz / 2.0; vp += w * o.ddivpdp;
            pc += w * o.Pcorr; del += w * o.div_el; dpl += w * o.div_pl;
            X += w * o.X1; OS += w * o.OverS;
            if (avg == 1) {
                sxx += w * 1.0 / o.txx; szz += w * 1.0 / o.tzz; sxz += w * 1.0 / o.txz;
                eta += w * 1.0 / o.etaVE; eta_phys += w * 1.0 / o.eta;
                double ie2 = pow(o.etaVE, 2.0);
                dexx += w * o.detadexx / ie2; dezz += w * o.detadezz / ie2;
                dgxz += w * o.detadexz / 2.0 / ie2; dp += w * o.detadp / ie2;
            }
            if (avg == 2) {
                eta += w * log(o.etaVE); eta_phys += w * log(o.eta);
                dexx += w * o.detadexx / o.etaVE; dezz += w * o.detadezz / o.etaVE;
                dgxz += w * o.detadexz / 2.0 / o.etaVE; dp += w * o.detadp / o.etaVE;
            }
        }
        dn = 1.0 / dn;
        if (avg == 1) {
            sxx = 1.0 / sxx; szz = 1.0 / szz; sxz = 1.0 / sxz; eta = 1.0 / eta; eta_phys = 1.0 / eta_phys;
            double e2 = pow(eta, 2.0);
            dexx *= e2; dezz *= e2; dgxz *= e2; dp *= e2;
        }
        if (avg == 2) {
            eta = exp(eta); eta_phys = exp(eta_phys);
            dexx *= eta; dezz *= eta; dgxz *= eta; dp *= eta;
        }
    }
    put(f.eta_n, c, eta); put(f.eta_phys_n, c, eta_phys); put(f.VE_n, c, VE);
    put(f.sxxd, c, sxx); put(f.szzd, c, szz); put(f.sxz_n, c, sxz);
    put(f.eII_el, c, eel); put(f.eII_pl, c, epl); put(f.eII_pwl, c, epwl); put(f.eII_lin, c, elin);
    put(f.eII_cst, c, ecst); put(f.d_n, c, dn); put(f.eII_exp, c, eexp); put(f.eII_gbs, c, egbs);
    put(f.exx_el, c, xel); put(f.exx_diss, c, xdi); put(f.ezz_el, c, zel); put(f.ezz_diss, c, zdi);
    put(f.detadexx_n, c, dexx); put(f.detadezz_n, c, dezz); put(f.detadgxz_n, c, dgxz); put(f.detadp_n, c, dp);
    put(f.ddivpdexx_n, c, vxx); put(f.ddivpdezz_n, c, vzz); put(f.ddivpdgxz_n, c, vxz); put(f.ddivpdp_n, c, vp);
    put(f.p_corr, c, pc); put(f.div_u_el, c, del); put(f.div_u_pl, c, dpl); put(f.div_u_r, c, 0.0);
    put(f.Wtot, c, Wt); put(f.Wel, c, We); put(f.Wdiss, c, Wd); put(f.X_n, c, X); put(f.OverS_n, c, OS);
    count_local(counters, fails, fallbacks, learned, iters);
}

__global__ void __launch_bounds__(128) k_viscosity_vertices(mdz_dgrid g, mdz_mat_k m, mdz_rheo_params prm,
                                                            mdz_fields f, int *__restrict__ counters,
                                                            const float2 *guess, float2 *labels, int fp32) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    int nv = g.Nx * g.Nz;
    if (c >= nv) return;
    const int avg = prm.eta_avg, nph = m.n_phases;
    double VE = 0, sxz = 0, eta_phys = 0, eta = 0, zel = 0, zdi = 0, dexx = 0, dezz = 0, dgxz = 0, dp = 0, X = 0,
           OS = 0;
    int fails = 0, fallbacks = 0, learned = 0, iters = 0;
    if (g.BCg[c] != 30) {
        const double etae = prm.iselastic == 1 ? prm.dt * f.mu_s[c] : 1.0;
        const double sxx0 = f.sxxd0_s[c], szz0 = f.szzd0_s[c], sxz0 = f.sxz0[c];
        double E[6];
        eff_rates(f.exxd_s[c], f.ezzd_s[c], f.exz[c], sxx0, szz0, sxz0, etae, E);
        const double mu = f.mu_s[c], T = f.T_s[c], P = f.P_s[c], d0 = f.d0_s[c], phi0 = f.phi0_s[c];
        const double X0 = f.X0_s ? f.X0_s[c] : 0.0, P0 = f.p0_s ? f.p0_s[c] : 0.0;
        const double dil = f.dil_s[c], fric = f.fric_s[c], Coh = f.C_s[c], bet = f.bet_s[c];
        for (int p = 0; p < nph; p++) {
            double w = f.phase_perc_s[(size_t)p * nv + c];
            if (!(fabs(w) > 1.0e-13)) continue;
            visc_res o;
            float gs[2];
            if (guess) {
                const float2 q = guess[(size_t)p * nv + c];
                gs[0] = q.x; gs[1] = q.y;
            }
            visc_node_phase(fp32 != 0, p, mu, T, P, d0, phi0, X0, E, sxx0, szz0, sxz0, m, prm, dil, fric, Coh, P0, bet, o,
                            guess ? gs : nullptr);
            // labels may be the guess buffer itself: this thread read its entry above
            if (labels) labels[(size_t)p * nv + c] = make_float2(o.lab_x, o.lab_y);
            fails += o.ve_fail + o.vp_fail;
            fallbacks += o.fallback;
            iters += o.ve_its + o.vp_its;
            learned += o.learned;
            if (avg == 0) {
                eta += w * o.etaVE; eta_phys += w * o.eta; dexx += w * o.detadexx; dezz += w * o.detadezz;
                dgxz += w * o.detadexz / 2.0; dp += w * o.detadp;
            }
            if (avg == 0 || avg == 2) sxz += w * o.txz;
            VE += w * o.VEcoeff; zel += w * o.Exz_el; zdi += w * o.Exz_diss; OS += w * o.OverS; X += w * o.X1;
            if (avg == 1) {
                sxz += w * 1.0 / o.txz; eta += w * 1.0 / o.etaVE; eta_phys += w * 1.0 / o.eta;
                double ie2 = pow(o.etaVE, 2.0);
                dexx += w * o.detadexx / ie2; dezz += w * o.detadezz / ie2;
                dgxz += w * o.detadexz / 2.0 / ie2; dp += w * o.detadp / ie2;
            }
            if (avg == 2) {
                eta += w * log(o.etaVE); eta_phys += w * log(o.eta);
                dexx += w * o.detadexx / o.etaVE; dezz += w * o.detadezz / o.etaVE;
                dgxz += w * o.detadexz / 2.0 / o.etaVE; dp += w * o.detadp / o.etaVE;
            }
        }
        if (avg == 1) {
            sxz = 1.0 / sxz; eta = 1.0 / eta; eta_phys = 1.0 / eta_phys;
            double e2 = pow(eta, 2.0);
            dexx *= e2; dezz *= e2; dgxz *= e2; dp *= e2;
        }
        if (avg == 2) {
            eta = exp(eta); eta_phys = exp(eta_phys);
            dexx *= eta; dezz *= eta; dgxz *= eta; dp *= eta;
        }
    }
    put(f.VE_s, c, VE); put(f.sxz, c, sxz); put(f.eta_phys_s, c, eta_phys); put(f.eta_s, c, eta);
    put(f.exz_el, c, zel); put(f.exz_diss, c, zdi);
    put(f.detadexx_s, c, dexx); put(f.detadezz_s, c, dezz); put(f.detadgxz_s, c, dgxz); put(f.detadp_s, c, dp);
    put(f.X_s, c, X); put(f.OverS_s, c, OS);
    count_local(counters, fails, fallbacks, learned, iters);
}

// ---------------------------------------------------------------------------
// Rheological operators (isotropic): Picard D = 2 eta I / eta; Newton adds the
// tangent terms 2 deta/dE * G.
__global__ void k_operators(mdz_dgrid g, mdz_rheo_params prm, mdz_fields f, int jacobian) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int nc = g.ncx * g.ncz, nv = g.Nx * g.Nz;
    if (i < nc) {
        int k = i;
        double d11 = 0, d12 = 0, d13 = 0, d14 = 0, d21 = 0, d22 = 0, d23 = 0, d24 = 0;
        if (g.BCp[k] != 30 && g.BCp[k] != 31) {
            double eta = f.eta_n[k];
            d11 = 2.0 * eta; d22 = 2.0 * eta;
            if (jacobian) {
                double etae = prm.iselastic == 1 ? prm.dt * f.mu_n[k] : 1.0, E[6];
                eff_rates(f.exxd[k], f.ezzd[k], f.exz_n[k], f.sxxd0[k], f.szzd0[k], f.sxz0_n[k], etae, E);
                // K = 0 (incompressible): the K*dt*ddivp terms vanish
                d11 += 2.0 * f.detadexx_n[k] * E[3];
                d12 = 2.0 * f.detadezz_n[k] * E[3];
                d13 = 2.0 * f.detadgxz_n[k] * E[3];
                d14 = 2.0 * f.detadp_n[k] * E[0];
                d21 = 2.0 * f.detadexx_n[k] * E[4];
                d22 += 2.0 * f.detadezz_n[k] * E[4];
                d23 = 2.0 * f.detadgxz_n[k] * E[4];
                d24 = 2.0 * f.detadp_n[k] * E[1];
            }
        }
        f.D11_n[k] = d11; f.D12_n[k] = d12; f.D13_n[k] = d13; f.D14_n[k] = d14;
        f.D21_n[k] = d21; f.D22_n[k] = d22; f.D23_n[k] = d23; f.D24_n[k] = d24;
    }
    if (i < nv) {
        int k = i;
        double d31 = 0, d32 = 0, d33 = 0, d34 = 0;
        if (g.BCg[k] != 30) {
            double eta = f.eta_s[k];
            d33 = eta;
            if (jacobian) {
                double etae = prm.iselastic == 1 ? prm.dt * f.mu_s[k] : 1.0, E[6];
                eff_rates(f.exxd_s[k], f.ezzd_s[k], f.exz[k], f.sxxd0_s[k], f.szzd0_s[k], f.sxz0[k], etae, E);
                d31 = 2.0 * f.detadexx_s[k] * E[5];
                d32 = 2.0 * f.detadezz_s[k] * E[5];
                d33 += 2.0 * f.detadgxz_s[k] * E[5];
                d34 = 2.0 * f.detadp_s[k] * E[2];
            }
        }
        f.D31_s[k] = d31; f.D32_s[k] = d32; f.D33_s[k] = d33; f.D34_s[k] = d34;
    }
}

// ---------------------------------------------------------------------------
// Momentum RHS (body force + elastic stress history), continuity RHS = 0.
__global__ void k_rhs(mdz_dgrid g, mdz_rheo_params prm, double gx, double gz, mdz_fields f) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int Nx = g.Nx, Nz = g.Nz, ncx = g.ncx, nu = Nx * (Nz + 1), nvz = (Nx + 1) * Nz;
    double dx = g.dx, dz = g.dz, dt = prm.dt;
    if (i < nu) {
        int c = i, k = c % Nx, l = c / Nx, c2 = k + (l - 1) * ncx;
        double r = 0.0;
        if (f.gx) f.gx[c] = gx;
        signed char t = g.BCu[c];
        if (l > 0 && l < Nz && (t == -1 || t == 2 || t == -2)) {
            int iPrW = c2 - 1, iPrE = c2, ixyN = c, ixyS = c - Nx;
            double inW = (k > 0 && g.BCp[iPrW] == -1) ? 1.0 : 0.0, inE = (k < Nx - 1 && g.BCp[iPrE] == -1) ? 1.0 : 0.0;
            double inS = (g.BCg[ixyS] != 30 && g.BCu[c - Nx] != 13) ? 1.0 : 0.0;
            double inN = (g.BCg[ixyN] != 30 && g.BCu[c + Nx] != 13) ? 1.0 : 0.0;
            r = -gx * (0.5 * (f.rho_s[ixyS] + f.rho_s[ixyN]));
            if (prm.iselastic == 1 && k > 0 && k < Nx - 1) {
                if (inE) r -= g.idx * (f.eta_n[iPrE] / (f.mu_n[iPrE] * dt) * f.sxxd0[iPrE]);
                if (inW) r -= g.idx * (-f.eta_n[iPrW] / (f.mu_n[iPrW] * dt) * f.sxxd0[iPrW]);
                if (inN) r -= g.idz * (f.eta_s[ixyN] / (f.mu_s[ixyN] * dt) * f.sxz0[ixyN]);
                if (inS) r -= g.idz * (-f.eta_s[ixyS] / (f.mu_s[ixyS] * dt) * f.sxz0[ixyS]);
            }
        }
        f.roger_x[c] = -r;
    }
    if (i < nvz) {
        int c = i, NxVz = Nx + 1, k = c % NxVz, l = c / NxVz, c1 = k + l * Nx - 1, c2 = k - 1 + (l - 1) * ncx;
        double r = 0.0;
        if (f.gz) f.gz[c] = gz;
        if (k > 0 && k < NxVz - 1 && g.BCv[c] == -1) {
            int iPrS = c2, iPrN = c2 + ncx, ixyE = c1 + 1, ixyW = c1;
            double inS = (l > 0 && g.BCp[iPrS] == -1) ? 1.0 : 0.0, inN = (l < Nz - 1 && g.BCp[iPrN] == -1) ? 1.0 : 0.0;
            double inW = (g.BCg[ixyW] != 30 && g.BCv[c - 1] != 13) ? 1.0 : 0.0;
            double inE = (g.BCg[ixyE] != 30 && g.BCv[c + 1] != 13) ? 1.0 : 0.0;
            r = -gz * (0.5 * ((l > 0 ? f.rho_n[iPrS] : 0.0) + (l < Nz - 1 ? f.rho_n[iPrN] : 0.0)));
            if (prm.iselastic == 1 && l > 0 && l < Nz - 1) {
                if (inN) r -= g.idz * (f.eta_n[iPrN] / (f.mu_n[iPrN] * dt) * (f.szzd0[iPrN]));
                if (inS) r -= g.idz * (-f.eta_n[iPrS] / (f.mu_n[iPrS] * dt) * (f.szzd0[iPrS]));
                if (inE) r -= g.idx * (f.eta_s[ixyE] / (f.mu_s[ixyE] * dt) * f.sxz0[ixyE]);
                if (inW) r -= g.idx * (-f.eta_s[ixyW] / (f.mu_s[ixyW] * dt) * f.sxz0[ixyW]);
            }
        }
        f.roger_z[c] = -r;
    }
    if (i < ncx * g.ncz && g.BCp[i] != 30 && g.BCp[i] != 31) f.rhs_p[i] = 0.0;
}

// ---------------------------------------------------------------------------
// Device-level launchers (used by the host drop-ins and by the time step).
mdz_status mdz_dev_strain_rates(mdz_ctx *ctx, const mdz_fields &f, cudaStream_t st) {
    const mdz_dgrid &g = ctx->g;
    int nc = g.ncx * g.ncz, nv = g.Nx * g.Nz;
    k_strain_centroids<<<mdz_blocks(nc), MDZ_THREADS, 0, st>>>(g, f.u, f.v, f.div_u, f.exxd, f.ezzd);
    MDZ_LAUNCHED(ctx);
    k_strain_vertices<<<mdz_blocks(nv), MDZ_THREADS, 0, st>>>(g, f.u, f.v, f.exz);
    MDZ_LAUNCHED(ctx);
    k_exz_to_centroids<<<mdz_blocks(nc), MDZ_THREADS, 0, st>>>(g, f.exz, f.exz_n);
    MDZ_LAUNCHED(ctx);
    k_c2v<<<mdz_blocks(nv), MDZ_THREADS, 0, st>>>(g, f.exxd, f.exxd_s);
    MDZ_LAUNCHED(ctx);
    k_c2v<<<mdz_blocks(nv), MDZ_THREADS, 0, st>>>(g, f.ezzd, f.ezzd_s);
    MDZ_LAUNCHED(ctx);
    return MDZ_OK;
}

mdz_status mdz_dev_c2v(mdz_ctx *ctx, const double *cen, double *ver, cudaStream_t st) {
    k_c2v<<<mdz_blocks(ctx->g.Nx * ctx->g.Nz), MDZ_THREADS, 0, st>>>(ctx->g, cen, ver);
    MDZ_LAUNCHED(ctx);
    return MDZ_OK;
}

mdz_status mdz_dev_v2c(mdz_ctx *ctx, double *cen, const double *ver, cudaStream_t st) {
    k_v2c<<<mdz_blocks(ctx->g.ncx * ctx->g.ncz), MDZ_THREADS, 0, st>>>(ctx->g, cen, ver);
    MDZ_LAUNCHED(ctx);
    return MDZ_OK;
}

mdz_status mdz_check_materials(mdz_ctx *ctx, const mdz_materials *m) {
    if (m->n_phases < 1 || m->n_phases > MDZ_MAX_PHASES || m->n_phases > ctx->n_phases)
        return mdz_fail(ctx, MDZ_ERR_ARG, "materials: %d phases (context has %d)", m->n_phases, ctx->n_phases);
    for (int p = 0; p < m->n_phases; p++) {
        if (m->gs[p] || m->reac_soft[p] || m->phase_mix[p])
            return mdz_fail(ctx, MDZ_ERR_UNSUPPORTED,
                            "phase %d: grain-size evolution and reaction mixing are not implemented", p);
        if (m->gbsv[p] && m->ngbs[p] <= 0) return mdz_fail(ctx, MDZ_ERR_ARG, "phase %d: ngbs must be > 0", p);
        if (m->expv[p] && !(m->Gexp[p] > 0 && m->Gexp[p] < 1 && m->Eexp[p] > 0 && m->Sexp[p] > 0))
            return mdz_fail(ctx, MDZ_ERR_ARG, "phase %d: Peierls creep needs 0 < Gexp < 1, Eexp > 0, Sexp > 0", p);
        if (m->pwlv[p] && m->npwl[p] <= 0) return mdz_fail(ctx, MDZ_ERR_ARG, "phase %d: npwl must be > 0", p);
        if (m->linv[p] && m->nlin[p] <= 0) return mdz_fail(ctx, MDZ_ERR_ARG, "phase %d: nlin must be > 0", p);
        if (m->n_vp[p] <= 0) return mdz_fail(ctx, MDZ_ERR_ARG, "phase %d: n_vp must be > 0", p);
    }
    return MDZ_OK;
}

// ---------------------------------------------------------------------------
// Learned guess: per (node, phase) MLP inference, one warp per 32 nodes and a
// warp-synchronous tensor-core pass per phase present in the warp.
__device__ __forceinline__ double eii_of(const double *E, const mdz_rheo_params &prm) {
    const double Eyy = -(E[0] + E[1]);
    double Eii = sqrt(0.5 * (E[0] * E[0] + E[1] * E[1] + Eyy * Eyy) + E[2] * E[2]);
    if (Eii * prm.scale_E < 1e-30) Eii = 1e-30 / prm.scale_E;
    return Eii;
}

template <bool CENT>
__global__ void __launch_bounds__(256) k_mlp_guess(mdz_dgrid g, int nph, mdz_rheo_params prm, mdz_fields f,
                                                   mdz_mlp_norm nm, const unsigned char *__restrict__ packed,
                                                   float2 *__restrict__ guess) {
    extern __shared__ __align__(16) unsigned char sm[];
    __nv_bfloat16 *XS = reinterpret_cast<__nv_bfloat16 *>(sm + MLP_PACK_BYTES);
    float *YS = reinterpret_cast<float *>(XS + 8 * 32 * MLP_S1);
    mlp_load_weights(sm, packed);
    for (int i = threadIdx.x; i < 8 * 32 * MLP_S1; i += blockDim.x) XS[i] = __float2bfloat16_rn(0.f);
    __syncthreads();
    const mlp_w W = mlp_views(sm);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __nv_bfloat16 *xs = XS + warp * 32 * MLP_S1;
    float *ys = YS + warp * 64;
    const int nn = CENT ? g.ncx * g.ncz : g.Nx * g.Nz;
    for (int base = (blockIdx.x * 8 + warp) * 32; base < nn; base += gridDim.x * 8 * 32) {
        const int c = base + lane;
        bool act = c < nn;
        if (act) act = CENT ? (g.BCp[c] != 30 && g.BCp[c] != 31) : (g.BCg[c] != 30);
        double Eii = 1.0 / prm.scale_E, T = ZEROC / prm.scale_T, P = 0.0;
        if (act) {
            double E[6];
            if (CENT) {
                const double etae = prm.iselastic == 1 ? prm.dt * f.mu_n[c] : 1.0;
                eff_rates(f.exxd[c], f.ezzd[c], f.exz_n[c], f.sxxd0[c], f.szzd0[c], f.sxz0_n[c], etae, E);
                T = f.T[c];
                P = f.p[c];
            } else {
                const double etae = prm.iselastic == 1 ? prm.dt * f.mu_s[c] : 1.0;
                eff_rates(f.exxd_s[c], f.ezzd_s[c], f.exz[c], f.sxxd0_s[c], f.szzd0_s[c], f.sxz0[c], etae, E);
                T = f.T_s[c];
                P = f.P_s[c];
            }
            Eii = eii_of(E, prm);
            if (T < ZEROC / prm.scale_T) T = ZEROC / prm.scale_T;
        }
        for (int p = 0; p < nph; p++) {
            const double w = act ? (CENT ? f.phase_perc_n[(size_t)p * nn + c] : f.phase_perc_s[(size_t)p * nn + c]) : 0.0;
            const bool need = act && fabs(w) > 1.0e-13;
            if (!__any_sync(0xffffffffu, need)) continue;
            float x[8];
            mlp_inputs(nm, prm, Eii, T, P, prm.dt, p, x);
            *reinterpret_cast<uint4 *>(xs + lane * MLP_S1) =
                make_uint4(mlp_pack2(x[0], x[1]), mlp_pack2(x[2], x[3]), mlp_pack2(x[4], x[5]), mlp_pack2(x[6], x[7]));
            __syncwarp();
            mlp_warp_infer(W, xs, ys);
            __syncwarp();
            if (need) guess[(size_t)p * nn + c] = make_float2(ys[2 * lane], ys[2 * lane + 1]);
            __syncwarp();
        }
    }
}

mdz_status mdz_dev_mlp_guess(mdz_ctx *ctx, const mdz_materials *m, const mdz_rheo_params *prm, const mdz_fields &f,
                             float2 *guess_n, float2 *guess_s, cudaStream_t st) {
    const mdz_dgrid &g = ctx->g;
    const int nc = g.ncx * g.ncz, nv = g.Nx * g.Nz;
    const size_t smem = MLP_PACK_BYTES + 8 * 32 * MLP_S1 * 2 + 8 * 64 * 4;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    auto grid = [&](int n) { int b = (n + 255) / 256; return b < 4 * sms ? (b < 1 ? 1 : b) : 4 * sms; };
    cudaEvent_t ev;
    mdz_prof_begin(ctx, MDZ_PROF_MLP, st, &ev);
    k_mlp_guess<true><<<grid(nc), 256, smem, st>>>(g, m->n_phases, *prm, f, ctx->mlp->norm, ctx->mlp->packed, guess_n);
    MDZ_LAUNCHED(ctx);
    k_mlp_guess<false><<<grid(nv), 256, smem, st>>>(g, m->n_phases, *prm, f, ctx->mlp->norm, ctx->mlp->packed, guess_s);
    MDZ_LAUNCHED(ctx);
    // per node: 6 FP64 rate/stress inputs, mu, T, P, the phase fractions, the tag; one float2 per phase out
    const double bytes = (double)(nc + nv) * (8.0 * (9 + m->n_phases) + 1 + 8.0 * m->n_phases);
    mdz_prof_end(ctx, MDZ_PROF_MLP, bytes, st, ev);
    return MDZ_OK;
}

// Training tuples: (strain rate, T, P, dt, phase) drawn from the ranges with a
// counter-based generator, labelled by the plain local solve.
__device__ __forceinline__ double mlp_u01(unsigned long long seed, long long i, int k) {
    unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(5 * i + k + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

__global__ void __launch_bounds__(128) k_mlp_samples(long long n, unsigned long long seed, mdz_mat_k m,
                                                     mdz_rheo_params prm, double lo0, double hi0, double lo1,
                                                     double hi1, double lo2, double hi2, double lo3, double hi3,
                                                     mdz_mlp_norm nm, uint4 *__restrict__ X, float2 *__restrict__ Y) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double Eii = pow(10.0, lo0 + (hi0 - lo0) * mlp_u01(seed, i, 0)) / prm.scale_E;
    double T = (lo1 + (hi1 - lo1) * mlp_u01(seed, i, 1)) / prm.scale_T;
    const double P = (lo2 + (hi2 - lo2) * mlp_u01(seed, i, 2)) / prm.scale_S;
    const double dt = pow(10.0, lo3 + (hi3 - lo3) * mlp_u01(seed, i, 3)) * prm.scale_E;
    int ph = (int)(mlp_u01(seed, i, 4) * m.n_phases);
    if (ph > m.n_phases - 1) ph = m.n_phases - 1;
    mdz_rheo_params q = prm;
    q.dt = dt;
    if (T < ZEROC / q.scale_T) T = ZEROC / q.scale_T;
    visc_res o;
    visc_local(ph, m.mu[ph], T, P, m.gs_ref[ph], 0.0, 0.0, Eii, -Eii, 0.0, Eii, -Eii, 0.0, 0.0, 0.0, 0.0, m, q,
               m.psi[ph], m.phi[ph], m.C[ph], P, m.bet[ph], o);
    float2 lab = mlp_labels(o.eta_ve, o.eta_up, o.gdot, Eii);
    lab.x = fminf(fmaxf(lab.x, -8.f), 1.f);
    lab.y = fminf(fmaxf(lab.y, 0.f), 1.f);
    float x[8];
    mlp_inputs(nm, q, Eii, T, P, dt, ph, x);
    X[i] = make_uint4(mlp_pack2(x[0], x[1]), mlp_pack2(x[2], x[3]), mlp_pack2(x[4], x[5]), mlp_pack2(x[6], x[7]));
    Y[i] = lab;
}

mdz_status mdz_dev_mlp_samples(mdz_ctx *ctx, const mdz_materials *m, const mdz_rheo_params *prm, long long n,
                               unsigned long long seed, const double lo[4], const double hi[4],
                               const mdz_mlp_norm &norm, uint4 *X, float2 *Y, cudaStream_t st) {
    k_mlp_samples<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(n, seed, mat_k(*m), *prm, lo[0], hi[0], lo[1], hi[1], lo[2],
                                                                hi[2], lo[3], hi[3], norm, X, Y);
    MDZ_LAUNCHED(ctx);
    return MDZ_OK;
}

mdz_status mdz_dev_viscosity(mdz_ctx *ctx, const mdz_materials *m, const mdz_rheo_params *prm, const mdz_fields &f,
                             int *d_counters, cudaStream_t st, bool learned, bool fp32, int warm) {
    const mdz_dgrid &g = ctx->g;
    int nc = g.ncx * g.ncz, nv = g.Nx * g.Nz;
    // vertex copies of centroid fields (NonNewtonianViscosityGrid :979-983)
    mdz_status s;
    if ((s = mdz_dev_c2v(ctx, f.div_u, f.div_u_s, st)) != MDZ_OK) return s;
    if ((s = mdz_dev_c2v(ctx, f.T, f.T_s, st)) != MDZ_OK) return s;
    if ((s = mdz_dev_c2v(ctx, f.p, f.P_s, st)) != MDZ_OK) return s;
    if ((s = mdz_dev_c2v(ctx, f.d0_n, f.d0_s, st)) != MDZ_OK) return s;
    if ((s = mdz_dev_c2v(ctx, f.phi0_n, f.phi0_s, st)) != MDZ_OK) return s;
    const float2 *guess_n = nullptr, *guess_s = nullptr;
    float2 *lab_n = nullptr, *lab_s = nullptr;
    if (learned && !fp32) {
        float2 *buf = mdz_mlp_guess_buffer(ctx, (size_t)m->n_phases * (nc + nv));
        if (!buf) return mdz_fail(ctx, MDZ_ERR_CUDA, "learned guess: buffer allocation failed");
        if (warm != 2)
            if ((s = mdz_dev_mlp_guess(ctx, m, prm, f, buf, buf + (size_t)m->n_phases * nc, st)) != MDZ_OK) return s;
        guess_n = buf;
        guess_s = buf + (size_t)m->n_phases * nc;
        if (warm >= 1) { lab_n = buf; lab_s = buf + (size_t)m->n_phases * nc; }
    }
    cudaEvent_t ev;
    mdz_prof_begin(ctx, MDZ_PROF_VISCOSITY, st, &ev);
    const mdz_mat_k mk = mat_k(*m);
    k_viscosity_centroids<<<mdz_blocks(nc, 128), 128, 0, st>>>(g, mk, *prm, f, d_counters, guess_n, lab_n, fp32 ? 1 : 0);
    MDZ_LAUNCHED(ctx);
    k_viscosity_vertices<<<mdz_blocks(nv, 128), 128, 0, st>>>(g, mk, *prm, f, d_counters, guess_s, lab_s, fp32 ? 1 : 0);
    MDZ_LAUNCHED(ctx);
    // algorithmic bytes: per centroid 17 + n_phases FP64 inputs and 35 outputs,
    // per vertex 17 + n_phases inputs and 12 outputs, plus the tags
    double bytes = (double)nc * (8.0 * (17 + m->n_phases + 35) + 1) + (double)nv * (8.0 * (17 + m->n_phases + 12) + 1);
    mdz_prof_end(ctx, MDZ_PROF_VISCOSITY, bytes, st, ev);
    return MDZ_OK;
}

mdz_status mdz_dev_operators(mdz_ctx *ctx, const mdz_rheo_params *prm, const mdz_fields &f, int jacobian,
                             cudaStream_t st) {
    const mdz_dgrid &g = ctx->g;
    int n = g.Nx * g.Nz;
    k_operators<<<mdz_blocks(n), MDZ_THREADS, 0, st>>>(g, *prm, f, jacobian);
    MDZ_LAUNCHED(ctx);
    return MDZ_OK;
}

mdz_status mdz_dev_rhs(mdz_ctx *ctx, const mdz_rheo_params *prm, double gx, double gz, const mdz_fields &f,
                       cudaStream_t st) {
    const mdz_dgrid &g = ctx->g;
    int n = (g.Nx + 1) * (g.Nz + 1);
    k_rhs<<<mdz_blocks(n), MDZ_THREADS, 0, st>>>(g, *prm, gx, gz, f);
    MDZ_LAUNCHED(ctx);
    return MDZ_OK;
}
