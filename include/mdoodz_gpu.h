/*
 * mdoodz_gpu.h -- C ABI of the GB300 (sm_103a) implementation of MDOODZ 6.0's
 * per-time-step data-parallel path: marker->grid projection, local
 * visco-elasto-plastic rheology with its Newton tangent, the matrix-free
 * decoupled staggered-grid Stokes residual / Jacobian inside a Newton-GCR loop,
 * and grid->marker interpolation with RK4 advection.
 *
 * Conventions shared with the reference (MDOODZ 6.0, paths relative to its
 * repository):
 *   - grid layout, row-major with x fastest (SOURCE/GridRoutines.c:481-528):
 *       vertices   Nx   x Nz      c1 = k + l*Nx
 *       centroids (Nx-1)x(Nz-1)   c0 = k + l*(Nx-1)
 *       Vx nodes   Nx   x(Nz+1)   c1 = k + l*Nx
 *       Vz nodes  (Nx+1)x Nz      c3 = k + l*(Nx+1)
 *   - boundary tags are the reference's char codes (SOURCE/set_Shear_VEVP.c:165-175):
 *       -1 inner, 0 Dirichlet on the boundary, 11 Dirichlet off the boundary,
 *       13 free-slip (Neumann) ghost, 2 Neumann, -2/-12 periodic, 30 air, 31 free surface;
 *   - node-set selector = the reference's `centroid` argument of P2Mastah
 *       (1 centroids, 0 vertices, -1 Vx nodes, -2 Vz nodes);
 *   - FP64 everywhere in the plain form, int32 marker phases (-1 = inactive).
 *
 * Every function is plain C: pointers and sizes only.  Functions whose name
 * starts with mdz_dev_ take DEVICE pointers and a cudaStream_t passed as void*;
 * all others take HOST pointers and are synchronous.  Every call returns an
 * mdz_status; mdz_last_error() gives a one-line message for the last failure.
 * The library never falls back to a CPU path: without a usable CUDA device,
 * mdz_create() fails with MDZ_ERR_CUDA.
 *
 * The library is not re-entrant: one context is used from one host thread.
 */
#ifndef MDOODZ_GPU_H
#define MDOODZ_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define MDZ_MAX_PHASES 20           /* mat_prop arrays hold 20 phases (SOURCE/header_MDOODZ.h:49) */
#define MDZ_P2G_MAX_FIELDS 8        /* fields one batched projection pass can produce */

typedef enum {
    MDZ_OK = 0,
    MDZ_ERR_ARG = 1,            /* bad argument (null pointer, bad size or selector)          */
    MDZ_ERR_CUDA = 2,           /* CUDA runtime error or no device                             */
    MDZ_ERR_CAPACITY = 3,       /* marker count above the context's capacity                  */
    MDZ_ERR_UNSUPPORTED = 4,    /* an option outside the implemented subset (message says which) */
    MDZ_ERR_NOT_CONVERGED = 5,  /* local or global iteration did not converge                 */
    MDZ_ERR_NAN = 6,            /* NaN/Inf detected in a residual or a grid field              */
    MDZ_ERR_STATE = 7           /* call out of order (e.g. no markers uploaded)                */
} mdz_status;

/* Node sets, encoded as the reference's `centroid` argument. */
#define MDZ_NODES_CENTROIDS 1
#define MDZ_NODES_VERTICES 0
#define MDZ_NODES_VX (-1)
#define MDZ_NODES_VZ (-2)

/* The staggered grid: coordinates and boundary tags, exactly the arrays the
 * reference keeps in `grid` (SOURCE/header_MDOODZ.h:170-219).  Coordinates are
 * taken as given (the reference accumulates them, SOURCE/GridRoutines.c:230-300),
 * so that index formulas see the same values bit for bit. */
typedef struct mdz_grid_desc {
    int Nx, Nz;                         /* vertices per direction                    */
    double dx, dz;
    double xmin, xmax, zmin, zmax;
    const double *xg, *zg;              /* Nx, Nz        vertex lines                 */
    const double *xc, *zc;              /* Nx-1, Nz-1    centroid lines               */
    const double *xvz, *zvx;            /* Nx+1, Nz+1    ghosted lines (Vz x, Vx z)    */
    const signed char *BCu_type;        /* Nx*(Nz+1)                                  */
    const signed char *BCv_type;        /* (Nx+1)*Nz                                  */
    const signed char *BCp_type;        /* (Nx-1)*(Nz-1)                              */
    const signed char *BCg_type;        /* Nx*Nz                                      */
    const double *BCu_val, *BCv_val;    /* Dirichlet values on Vx / Vz nodes          */
    int isperiodic_x;                   /* only 0 is implemented                      */
} mdz_grid_desc;

typedef struct mdz_ctx mdz_ctx;

/* ---- context ------------------------------------------------------------ */

/* Create a context on the current CUDA device: copies the grid description to
 * the device and reserves room for `max_markers` markers.  Replaces the
 * reference's GridAlloc/PartAlloc (SOURCE/MemoryAllocFree.c:182,333) for the
 * device mirrors; the host arrays stay owned by the caller.  Grids of 3 to
 * 65 535 lines a side (MDZ_ERR_ARG otherwise). */
mdz_status mdz_create(mdz_ctx **ctx, const mdz_grid_desc *grid, int n_phases, long long max_markers);
void mdz_destroy(mdz_ctx *ctx);
const char *mdz_last_error(const mdz_ctx *ctx);
/* Number of kernels this context has launched so far (for launch accounting). */
long long mdz_kernel_launches(const mdz_ctx *ctx);

/* Upload markers (positions and phase) to the context's resident marker store
 * and mark the cell binning stale.  n <= max_markers. */
mdz_status mdz_set_markers(mdz_ctx *ctx, int n, const double *x, const double *z, const int *phase);
/* Number of resident markers (particles.Nb_part): the count set by
 * mdz_set_markers, grown by reseeding (mdz_CountPartCell, mdz_time_step). */
int mdz_marker_count(const mdz_ctx *ctx);
/* Breakpoint of the resident state (MakeBreakpointParticles /
 * LoadBreakpointParticles, SOURCE/InputOutput.c:515-1007, 160-514, for what
 * this library keeps between steps): markers (x, z, phase, Vx, Vz and the
 * MDZ_M_* attributes) and the grid u, v, p that start the next step, from
 * the device mirrors to one binary file ("MDZBRK02" header with the grid
 * sizes and the box, then the arrays in host byte order) and back into a
 * context of the same grid sizes and phase count; loading moves the
 * context's box to the saved one (a box moved by PureShearALE), as the
 * reference restores model.xmin..zmax.  A restart from it continues as the
 * uninterrupted run; the learned guess's weights are saved separately
 * (mdz_mlp_get_weights).  MDZ_ERR_ARG for an unreadable, foreign or
 * truncated file (the context is unchanged then), MDZ_ERR_CAPACITY when its
 * markers exceed the capacity. */
mdz_status mdz_save_breakpoint(mdz_ctx *ctx, const char *path);
mdz_status mdz_load_breakpoint(mdz_ctx *ctx, const char *path);

/* Flags and scales of the reference run that wrote a breakpoint: the model
 * switches that decide which sections its file holds (params free_surf,
 * iselastic, fstrain, aniso, rec_T_P_x_z) and its scale (scaling.L, .V, .S,
 * .T, .t). */
typedef struct {
    int free_surf, iselastic, fstrain, aniso, rec_T_P_x_z;
    double L, V, S, T, t;
} mdz_ref_breakpoint_desc;

/* Restart from the reference's own breakpoint file (Breakpoint%05d.dat of
 * MakeBreakpointParticles, SOURCE/InputOutput.c:515-903), read as
 * LoadBreakpointParticles (:160-514) reads it: marker positions, velocities,
 * phases, P, deviatoric stresses (iselastic), strain, plastic strain and T,
 * and u_in, v_in, p_in as the next step's starting u, v, p, divided by the
 * run's scales; the box is restored; MDZ_M_CMUL is set to 1.  dt and time
 * (scaled) are returned when the pointers are not NULL.  The file's length
 * must be the one the flags give for this context's grid and phase count:
 * MDZ_ERR_ARG otherwise (wrong flags, another grid, a truncated file), and
 * for phases outside -1..n_phases-1, with the context unchanged;
 * MDZ_ERR_CAPACITY when its markers exceed the capacity. */
mdz_status mdz_load_reference_breakpoint(mdz_ctx *ctx, const char *path, const mdz_ref_breakpoint_desc *desc,
                                         double *dt, double *time);
/* Upload the resident markers' velocities (particles.Vx, Vz; RK4 writes them,
 * reseeding copies them), e.g. when markers are restored from a saved state. */
mdz_status mdz_set_marker_velocity(mdz_ctx *ctx, int n, const double *vx, const double *vz);
/* Download resident marker positions / phases (any pointer may be NULL). */
mdz_status mdz_get_markers(mdz_ctx *ctx, int n, double *x, double *z, int *phase, double *vx, double *vz);

/* Page-lock (register) an existing host array, e.g. the reference's marker
 * arrays from PartAlloc (SOURCE/MemoryAllocFree.c:333), so that the marker
 * and field transfers above run as DMA copies instead of staged pageable
 * copies; mdz_host_unregister undoes it before the caller frees the array.
 * No counterpart in the reference (it keeps everything in host memory).
 * MDZ_ERR_ARG for a null pointer or zero size, MDZ_ERR_CUDA if CUDA refuses. */
mdz_status mdz_host_register(void *p, size_t bytes);
mdz_status mdz_host_unregister(void *p);

/* ---- marker -> grid projection ----------------------------------------- */

/* Drop-in for P2Mastah (SOURCE/ParticleRoutines.c:3226-3537) on the markers
 * last given to mdz_set_markers():
 *   mat_prop   flag 0: one value per phase (n_phases); flag 1: one value per marker
 *   node_field in/out, size of the selected node set; nodes with zero weight or
 *              tag 30/31 in node_type are left untouched (as the reference does)
 *   node_type  the tag array of that node set
 *   avg        0 arithmetic, 1 harmonic, 2 geometric
 *   prop       1: compute phase fractions into phase_perc instead of a field
 *   phase_perc n_phases x nnodes, row p = fraction of phase p (prop == 1 only;
 *              centroid and vertex node sets only, as in the reference)
 *   itp_stencil 1 (1-cell) or 9 (9-cell)
 * Host buffers; synchronous. */
mdz_status mdz_P2Mastah(mdz_ctx *ctx, const double *mat_prop, double *node_field, const signed char *node_type,
                        int flag, int avg, int prop, int centroid, int itp_stencil, double *phase_perc);

/* Batched device form: project up to MDZ_P2G_MAX_FIELDS per-marker fields
 * (d_values[f], length n_markers) onto one node set in a single marker pass,
 * each with its own averaging type; optionally also the phase fractions
 * (d_phase_perc != NULL).  Device pointers. */
mdz_status mdz_dev_p2g(mdz_ctx *ctx, int n_fields, const double *const *d_values, const int *avg,
                       double *const *d_out, double *d_phase_perc, int centroid, int itp_stencil, void *stream);

/* Marker binning (CountPartCell_Old counting, SOURCE/ParticleRoutines.c:4485-4980):
 * per-cell and per-vertex marker counts and per-(node, phase) counts, all
 * int32.  Any output may be NULL.  Host buffers. */
mdz_status mdz_count_markers(mdz_ctx *ctx, int *nb_part_cell, int *nb_part_vert, int *phase_count_cell,
                             int *phase_count_vert);

/* Marker reseeding: CountPartCell(particles, mesh, model, topo, topo_ini,
 * RESEED, scaling) (SOURCE/ParticleRoutines.c:3543-4480) on the resident
 * markers, with the result the reference gives on one OpenMP thread (its
 * thread slabs change which markers a new one may copy from).  reseed = 0
 * returns at once: the phase fractions CountPartCell also computes come from
 * mdz_P2Mastah with prop = 1.  reseed = 1: every quarter cell whose centroid
 * is not air and that holds fewer than (int)(ceil(min_part_cell) / 4) active
 * markers (particles.min_part_cell) gets one marker at its centre
 * (AddPartCell2 :977-1030).  The new marker copies the phase, velocity and
 * strains of the nearest marker within two quarter cells (FindClosestPhase2
 * :841-890); its T, pressure and stresses come from that marker
 * (direct_neighbour = 1) or from the grid fields T_n, sxxd_n, szzd_n, p_n
 * (centroids: p_n is the grid pressure p_in) and sxz_s (vertices)
 * (direct_neighbour = 0, model.DirectNeighbour; host arrays, which may be NULL
 * when direct_neighbour = 1) (AssignMarkerProperties :648-762).
 * New markers fill the slots of inactive markers (phase -1) first and are
 * then appended; n_added (may be NULL) receives their number.
 * MDZ_ERR_CAPACITY if they do not fit in the context's capacity (the
 * reference exits), MDZ_ERR_STATE if a deficient quarter cell has no marker
 * within two quarter cells (the reference exits with code 333); the markers
 * are unchanged then.  Free surface, sedimentation and periodic x are not
 * implemented (the context rejects them); MDZ_ERR_UNSUPPORTED for grids whose
 * (2 (Nx - 1) + 4)(2 (Nz - 1) + 4) quarter cells exceed 2^31. */
mdz_status mdz_CountPartCell(mdz_ctx *ctx, int reseed, int min_part_cell, int direct_neighbour, const double *T_n,
                             const double *sxxd_n, const double *szzd_n, const double *sxz_s, const double *p_n,
                             int *n_added);

/* ---- grid -> marker interpolation ---------------------------------------- */

/* Interp_Grid2P (SOURCE/ParticleRoutines.c:2439-2608): bilinear from a node set
 * whose x/z lines are given as node_set (0 vertices, -1 Vx, -2 Vz) with
 * tag 30/31 substitution.  Interp_Grid2P_centroids2
 * (SOURCE/ParticleRoutines.c:2612-2862): node_set = 1, centroid field
 * interpolated in the extended (ghost) centroid frame.  Host buffers. */
mdz_status mdz_Interp_Grid2P(mdz_ctx *ctx, const double *node_field, int node_set, double *marker_field);

/* RogerGuntherII (SOURCE/AdvectionRoutines.c:569-628): classic RK4 through the
 * staggered velocity (u: Nx*(Nz+1), v: (Nx+1)*Nz) on the resident markers;
 * markers leaving the box get phase -1.  Updates resident x, z, Vx, Vz, phase. */
mdz_status mdz_RogerGuntherII(mdz_ctx *ctx, const double *u, const double *v, double dt);

/* ---- local rheology ------------------------------------------------------ */

/* Per-phase material parameters: the subset of the reference's mat_prop
 * (SOURCE/header_MDOODZ.h:46-63) used by the implemented creep laws.
 * Implemented: constant viscosity (cstv), dislocation creep (pwlv), diffusion
 * creep (linv, constant grain size), Peierls creep (expv, below 1200 C),
 * grain-boundary sliding (gbsv), Maxwell elasticity, Drucker-Prager / von
 * Mises plasticity with the viscoplastic regularisation eta_vp, n_vp, and the
 * tension cut-off (is_tensile, tension pressure -25 MPa).
 * Not implemented (rejected with MDZ_ERR_UNSUPPORTED): grain-size evolution
 * (gs), reaction mixing (reac_soft, phase_mix). */
typedef struct mdz_materials {
    int n_phases;
    double R;                                           /* gas constant (mat_prop.R)           */
    int cstv[MDZ_MAX_PHASES], pwlv[MDZ_MAX_PHASES], linv[MDZ_MAX_PHASES];
    int expv[MDZ_MAX_PHASES], gbsv[MDZ_MAX_PHASES], gs[MDZ_MAX_PHASES], is_tensile[MDZ_MAX_PHASES];
    int reac_soft[MDZ_MAX_PHASES], phase_mix[MDZ_MAX_PHASES];
    double eta0[MDZ_MAX_PHASES], rho[MDZ_MAX_PHASES], alp[MDZ_MAX_PHASES], gs_ref[MDZ_MAX_PHASES];
    double Slim[MDZ_MAX_PHASES], eta_vp[MDZ_MAX_PHASES], n_vp[MDZ_MAX_PHASES];
    /* dislocation creep */
    double npwl[MDZ_MAX_PHASES], Apwl[MDZ_MAX_PHASES], Qpwl[MDZ_MAX_PHASES], Vpwl[MDZ_MAX_PHASES];
    double mpwl[MDZ_MAX_PHASES], rpwl[MDZ_MAX_PHASES], fpwl[MDZ_MAX_PHASES], apwl[MDZ_MAX_PHASES];
    double Fpwl[MDZ_MAX_PHASES], pref_pwl[MDZ_MAX_PHASES];
    /* diffusion creep */
    double nlin[MDZ_MAX_PHASES], Alin[MDZ_MAX_PHASES], Qlin[MDZ_MAX_PHASES], Vlin[MDZ_MAX_PHASES];
    double mlin[MDZ_MAX_PHASES], rlin[MDZ_MAX_PHASES], flin[MDZ_MAX_PHASES], alin[MDZ_MAX_PHASES];
    double Flin[MDZ_MAX_PHASES];
    /* grid-property inputs of the time step (ShearModCompExpGrid,
     * CohesionFrictionDilationGrid: SOURCE/RheologyDensity.c:1422-1791) */
    double mu[MDZ_MAX_PHASES], bet[MDZ_MAX_PHASES], C[MDZ_MAX_PHASES], phi[MDZ_MAX_PHASES], psi[MDZ_MAX_PHASES];
    double C_end[MDZ_MAX_PHASES], phi_end[MDZ_MAX_PHASES], psi_end[MDZ_MAX_PHASES];
    double pls_start[MDZ_MAX_PHASES], pls_end[MDZ_MAX_PHASES];
    int coh_soft[MDZ_MAX_PHASES], phi_soft[MDZ_MAX_PHASES], psi_soft[MDZ_MAX_PHASES];
    /* Peierls creep (expv): activation energy Qexp, Peierls stress Sexp,
     * reference strain rate Eexp, gamma Gexp (0 < Gexp < 1), stress exponent
     * nexp (Viscosity, SOURCE/RheologyDensity.c:181-199) */
    double Qexp[MDZ_MAX_PHASES], Sexp[MDZ_MAX_PHASES], Eexp[MDZ_MAX_PHASES], Gexp[MDZ_MAX_PHASES];
    double nexp[MDZ_MAX_PHASES];
    /* grain-boundary sliding (gbsv), a creep law of the dislocation form */
    double ngbs[MDZ_MAX_PHASES], Agbs[MDZ_MAX_PHASES], Qgbs[MDZ_MAX_PHASES], Vgbs[MDZ_MAX_PHASES];
    double mgbs[MDZ_MAX_PHASES], rgbs[MDZ_MAX_PHASES], fgbs[MDZ_MAX_PHASES], agbs[MDZ_MAX_PHASES];
    double Fgbs[MDZ_MAX_PHASES];
} mdz_materials;

/* Model switches and scales read by the rheology (params / scale in the reference). */
typedef struct mdz_rheo_params {
    double dt;
    int iselastic;          /* model.iselastic                                  */
    int step;               /* model.step (step 0 switches elasticity off)      */
    int eta_avg;            /* 0 arithmetic, 1 harmonic, 2 geometric phase mix   */
    double mineta, maxeta;  /* viscosity limiter                                */
    double scale_T, scale_E, scale_S, scale_eta, scale_L;
    int clamp_tangent;      /* 0: the reference's tangent, which differentiates the
                               unlimited viscosity also where the limiter is active;
                               1: zero tangent where mineta / maxeta clip (the
                               derivative of the limited law)                       */
} mdz_rheo_params;

/* Grid fields by the reference's names (grid, SOURCE/header_MDOODZ.h:170-219).
 * Suffix convention: no suffix or _n = centroids ((Nx-1)*(Nz-1)), _s and exz,
 * sxz, sxz0 = vertices (Nx*Nz), u / roger_x / ru = Vx nodes, v / roger_z / rv =
 * Vz nodes, p / p_corr / rhs_p / rp = centroids.  phase_perc_n/_s hold
 * n_phases rows.  Host calls read the fields a function consumes and write the
 * fields it produces; NULL pointers are skipped where a field is optional. */
typedef struct mdz_fields {
    double *u, *v, *p, *p_corr;
    double *div_u, *div_u_s, *exxd, *ezzd, *exz, *exz_n, *exxd_s, *ezzd_s;
    double *sxxd0, *szzd0, *sxz0, *sxxd0_s, *szzd0_s, *sxz0_n;
    double *mu_n, *mu_s, *T, *T_s, *P_s, *d0_n, *d0_s, *phi0_n, *phi0_s, *X0_n, *X0_s;
    double *strain_n, *strain_s, *dil_n, *dil_s, *fric_n, *fric_s, *C_n, *C_s, *p0_n, *p0_s;
    double *bet_n, *bet_s, *rho_n, *rho_s;
    double *phase_perc_n, *phase_perc_s;
    double *eta_n, *eta_s, *eta_phys_n, *eta_phys_s, *VE_n, *VE_s, *sxxd, *szzd, *sxz, *sxz_n;
    double *eII_el, *eII_pl, *eII_pwl, *eII_lin, *eII_cst, *d_n;
    double *exx_el, *ezz_el, *exz_el, *exx_diss, *ezz_diss, *exz_diss;
    double *detadexx_n, *detadezz_n, *detadgxz_n, *detadp_n;
    double *ddivpdexx_n, *ddivpdezz_n, *ddivpdgxz_n, *ddivpdp_n;
    double *detadexx_s, *detadezz_s, *detadgxz_s, *detadp_s;
    double *div_u_el, *div_u_pl, *div_u_r, *Wtot, *Wel, *Wdiss, *X_n, *X_s, *OverS_n, *OverS_s;
    double *D11_n, *D12_n, *D13_n, *D14_n, *D21_n, *D22_n, *D23_n, *D24_n;
    double *D31_s, *D32_s, *D33_s, *D34_s;
    double *roger_x, *roger_z, *rhs_p, *gx, *gz;
    double *ru, *rv, *rp;
    double *eII_exp, *eII_gbs;   /* centroid Peierls and grain-boundary-sliding rates */
    /* energy equation: conductivity on the Vx / Vz faces (kx, kz), heat
     * capacity Cv, radiogenic heat Qr, temperature increment dT and thermal
     * expansivity alp at the centroids */
    double *kx, *kz, *Cv, *Qr, *dT, *alp;
} mdz_fields;

/* Host-pointer drop-ins for the grid-side reference functions.  Each reads the
 * fields listed and writes the fields it produces in `f` (synchronous). */

/* StrainRateComponents (SOURCE/RheologyDensity.c:1902-1984): u, v ->
 * div_u, exxd, ezzd, exz, exz_n, exxd_s, ezzd_s. */
mdz_status mdz_StrainRateComponents(mdz_ctx *ctx, mdz_fields *f);

/* NonNewtonianViscosityGrid + Viscosity (SOURCE/RheologyDensity.c:961-1415,
 * 44-707): local VEP solve per node and phase, phase-fraction averaging, and
 * the consistent tangent.  Reads the strain rates, old stresses, mu, T, p, d0,
 * phi0, C, fric, dil, bet and phase_perc fields; writes eta, eta_phys, stresses,
 * strain-rate partition, detad*, ddivpd*, p_corr, W*, OverS.  Where the
 * reference exit()s on a failed local iteration, the count of such (node,
 * phase) solves is returned in *n_not_converged (may be NULL). */
mdz_status mdz_NonNewtonianViscosityGrid(mdz_ctx *ctx, const mdz_materials *mat, const mdz_rheo_params *prm,
                                         mdz_fields *f, int *n_not_converged);

/* ---- learned start of the local solves (no counterpart in the reference) --
 *
 * An 8 -> 64 -> 64 -> 2 ReLU network (BF16 weights and activations, FP32
 * accumulation, tensor-core kernels) maps (log10 strain-rate invariant [1/s],
 * T [K], P [Pa], log10 dt [s], one-hot phase of at most 4) to the local
 * Newton unknowns: y0 = ln(eta_ve / eta_up), the visco-elastic viscosity
 * relative to the plain iteration's start eta_up (smallest viscosity of the
 * active mechanisms), and y1 = gdot / (2 Eii).
 * Each local solve then starts there, takes at most two polish updates
 * (Halley steps in log eta_ve, Newton steps in gdot) and must pass the
 * reference's own convergence test; otherwise it reruns the plain solve from
 * the reference's start.  Parameters are MDZ_MLP_NPARAM FP32 values:
 * W1[64][8], b1[64], W2[64][64], b2[64], W3[2][64], b3[2]. */
#define MDZ_MLP_NPARAM 4866
/* He-uniform weights from the seed, zero biases, Adam state cleared. */
mdz_status mdz_mlp_init(mdz_ctx *ctx, unsigned long long seed);
mdz_status mdz_mlp_set_weights(mdz_ctx *ctx, const float *params);
mdz_status mdz_mlp_get_weights(mdz_ctx *ctx, float *params);
/* Input normalisation ranges lo[4], hi[4] of (log10 Eii, T, P, log10 dt):
 * x = 2 (v - lo) / (hi - lo) - 1, temperature as 1000 / T over
 * [1000 / hi, 1000 / lo]. */
mdz_status mdz_mlp_set_ranges(mdz_ctx *ctx, const double *lo, const double *hi);
/* Kernels of inference (mdz_mlp_infer, mdz_mlp_benchmark) and training
 * (mdz_mlp_train, mdz_mlp_gradients): 0 (default) tcgen05.mma on 128-row
 * tiles with the accumulators in tensor memory, 1 the warp-level mma.sync
 * kernels.  Both compute the same BF16 network with FP32 accumulation. */
mdz_status mdz_mlp_set_engine(mdz_ctx *ctx, int engine);
/* n training tuples on the device, drawn uniformly in the ranges (phase
 * uniform among the materials' phases) and labelled by the plain local solve
 * of these materials and switches (dt per tuple). */
mdz_status mdz_mlp_generate(mdz_ctx *ctx, const mdz_materials *mat, const mdz_rheo_params *prm, long long n,
                            unsigned long long seed, const double *lo, const double *hi);
/* Adam on the mean squared error over consecutive batches of the tuples,
 * learning rate decaying from lr to lr / 100 (cosine); *final_loss = mean loss
 * of the last 8 steps. */
mdz_status mdz_mlp_train(mdz_ctx *ctx, int steps, int batch, double lr, double *final_loss);
/* Gradient of the mean squared error over n host rows (x: n x 8 normalised
 * inputs, y: n x 2 labels) at the current weights, without an update:
 * grad[MDZ_MLP_NPARAM] and *loss. */
mdz_status mdz_mlp_gradients(mdz_ctx *ctx, int n, const float *x, const float *y, float *grad, double *loss);
/* Network outputs for n host rows (x: n x 8 normalised inputs -> y: n x 2). */
mdz_status mdz_mlp_infer(mdz_ctx *ctx, long long n, const float *x, float *y);
/* Device timing over the generated tuples: one inference pass (ms), one
 * training step of `batch` rows (ms), and the RMS error of the outputs against
 * the labels. */
mdz_status mdz_mlp_benchmark(mdz_ctx *ctx, int batch, int reps, double *ms_infer, double *ms_train_step,
                             double *rms_error);
/* NonNewtonianViscosityGrid with (learned = 1) or without the learned start;
 * stats[4] = not converged, learned starts that fell back to the plain solve,
 * learned starts, total local Newton updates. */
mdz_status mdz_NonNewtonianViscosityGrid_learned(mdz_ctx *ctx, const mdz_materials *mat, const mdz_rheo_params *prm,
                                                 mdz_fields *f, int learned, long long *stats);

/* ShearModCompExpGrid (SOURCE/RheologyDensity.c:1666-1791): harmonic phase
 * averages of the shear modulus and compressibility from phase_perc_n /
 * phase_perc_s -> mu_n, mu_s, bet_n, bet_s (0 on air nodes). */
mdz_status mdz_ShearModCompExpGrid(mdz_ctx *ctx, const mdz_materials *mat, mdz_fields *f);

/* CohesionFrictionDilationGrid (SOURCE/RheologyDensity.c:1422-1665): the
 * resident markers' plastic strain projected to the centroids (P2Mastah with
 * itp_stencil 1 or 9) and to the vertices (Interp_P2N, one-cell tent), the
 * smooth (erfc) softening of cohesion, friction and dilation per phase, and
 * arithmetic phase averages from phase_perc_n / phase_perc_s -> C_n, C_s,
 * fric_n, fric_s, dil_n, dil_s, strain_n, strain_s (0 on air nodes). */
mdz_status mdz_CohesionFrictionDilationGrid(mdz_ctx *ctx, const mdz_materials *mat, int itp_stencil, mdz_fields *f);

/* RheologicalOperators (SOURCE/RheologyDensity.c:713-954), isotropic:
 * Picard (jacobian = 0) or Newton (jacobian = 1) D11..D24 at centroids and
 * D31..D34 at vertices. */
mdz_status mdz_RheologicalOperators(mdz_ctx *ctx, const mdz_rheo_params *prm, mdz_fields *f, int jacobian);

/* EvaluateRHS (SOURCE/StokesRoutines.c:922-1133), incompressible and
 * non-polar: roger_x, roger_z (body force and elastic history), rhs_p. */
mdz_status mdz_EvaluateRHS(mdz_ctx *ctx, const mdz_rheo_params *prm, double gx, double gz, mdz_fields *f);

/* ---- decoupled Stokes ----------------------------------------------------- */

/* EvaluateStokesResidualDecoupled (SOURCE/StokesRoutines.c:839-920) with the
 * residual rows of BuildStokesOperatorDecoupled(Assemble = 0)
 * (SOURCE/StokesAssemblyDecoupled.c:1573-2150): reads u, v, p_corr, D11_n,
 * D22_n, D33_s (Picard operators), roger_x, roger_z, rhs_p; writes ru, rv, rp
 * (grid layout, zero off the equations) and norms3 = sqrt(sum F^2 / n) for the
 * x-momentum, z-momentum and continuity blocks.  MDZ_ERR_NAN where the
 * reference exit(122)s. */
mdz_status mdz_EvaluateStokesResidualDecoupled(mdz_ctx *ctx, mdz_fields *f, double *norms3);

/* The norms3 of EvaluateStokesResidualDecoupled from residual rows the caller
 * already holds on the device, without allocating anything and without a
 * context (no counterpart in the reference, which reduces on the host).
 * Device pointers in grid layout: ru (Nx*(Nz+1)), rv ((Nx+1)*Nz),
 * rp ((Nx-1)*(Nz-1)) and their tag arrays; norms3 is a device array of 3
 * doubles written on `stream` (a cudaStream_t; NULL = legacy default stream).
 * Scratch: a static device array of 8192 * 6 doubles (384 KiB), one slot per
 * index-box row; grids with Nz + 1 > 8192 rows, or whose Vx/Vz index
 * boxes exceed 32-bit indices, are rejected with MDZ_ERR_CAPACITY.  No
 * scratch value has to start at zero (every slot a call reads is written by
 * that call first) and the result is bitwise reproducible.  The first call on
 * a device looks the scratch address up (cudaGetSymbolAddress, with that
 * device current).  That address is kept for the life of the process; after a cudaDeviceReset (or anything else
 * that tears down the device's primary context) it is stale, and this entry
 * point must not be called again in that process.  The scratch is shared, so
 * calls that overlap in time (several streams or host threads on one device)
 * race and must be serialised.  Status only (no context for a message):
 * MDZ_ERR_ARG for a null pointer or Nx, Nz < 3, MDZ_ERR_CAPACITY for a grid
 * above the limits, MDZ_ERR_CUDA for a launch error -- including an earlier
 * asynchronous error still pending on the device, which the launch check
 * reports (and clears) here. */
mdz_status mdz_dev_residual_norms_noalloc(int Nx, int Nz, const double *ru, const double *rv, const double *rp,
                                          const signed char *BCu, const signed char *BCv, const signed char *BCp,
                                          double *norms3, void *stream);

/* Matrix-free linear operator, the product of the reference's assembled
 * blocks with a correction vector (x zero on non-equation nodes):
 * jacobian = 0: BuildStokesOperatorDecoupled(Assemble = 1) blocks [A B; C D];
 * jacobian = 1: BuildJacobianOperatorDecoupled (SOURCE/StokesAssemblyDecoupled.c:3834-4376).
 * Uses the D-tensor fields in f.  Host buffers in grid layout. */
mdz_status mdz_StokesOperatorApply(mdz_ctx *ctx, mdz_fields *f, int jacobian, const double *xu, const double *xv,
                                   const double *xp, double *yu, double *yv, double *yp);

/* Linear defect solve K dx = F, the job of SolveStokesDefectDecoupled ->
 * KillerSolver (SOURCE/StokesRoutines.c:700-764, SOURCE/Solvers.c:2226-2755),
 * done matrix-free: GCR preconditioned by a block-triangular operator whose
 * velocity block is one geometric-multigrid V-cycle on the Picard operator
 * (eta_n, eta_s) and whose pressure block is eta_n / cell volume.
 * K = Picard (jacobian = 0) or Newton Jacobian (jacobian = 1) from the
 * D-tensor in f.  precision 64: plain FP64; 32: FP32 stencils and V-cycles
 * inside FP64 iterative refinement.  Stops at ||F - K dx|| <= rtol ||F||;
 * MDZ_ERR_NOT_CONVERGED if maxit Krylov iterations do not reach it.  The
 * caller applies the update as the reference does: u <- u + alpha dx with
 * alpha = -1 without line search.  Host buffers in grid layout. */
mdz_status mdz_SolveStokesDefect(mdz_ctx *ctx, mdz_fields *f, int jacobian, int precision, double rtol, int maxit,
                                 const double *Fu, const double *Fv, const double *Fp, double *dxu, double *dxv,
                                 double *dxp, int *iterations, double *rel_residual);

/* Knobs of the defect solve (no counterpart in the reference, whose direct
 * factorisation has none): V-cycle pre/post Jacobi sweeps nu1 (1..16) and nu2
 * (0..16), Jacobi damping omega in (0, 2), GCR restart length (2..48), the
 * number of Krylov iterations between host-side convergence checks (1..64), and
 * mg_jacobian = 1 to build the multigrid hierarchy of a Newton solve from the
 * Jacobian's velocity block instead of the Picard block.
 * Defaults 2, 1, 0.7, 30, 1, 0. */
mdz_status mdz_set_solver_options(mdz_ctx *ctx, int nu1, int nu2, double omega, int restart, int check,
                                  int mg_jacobian);

/* Pressure block of the preconditioner in Newton (Jacobian) solves: mode 0
 * (default) scales the pressure residual by eta_n / cell volume, as in the
 * Picard solves; mode 1 by the Jacobian's own D11 / 2 (the tangent viscosity,
 * which the plastic part of the Newton tangent lowers below eta_n) wherever
 * that is positive, eta_n elsewhere.  No counterpart in the reference (its
 * defect solves are direct). */
mdz_status mdz_set_schur_scaling(mdz_ctx *ctx, int mode);

/* Multigrid stencils of one level after a solve (diagnostics and tests; no
 * counterpart in the reference).  31 coefficient planes per velocity row,
 * structure of arrays: su[31][Nx*(Nz+1)] for Vx rows, sv[31][(Nx+1)*Nz] for Vz
 * rows.  Vx row (k, l): planes 0..14 couple Vx (k+dk, l+dl), dk in -1..1,
 * dl in -2..2, plane (dk+1) + 3 (dl+2); planes 15..30 couple Vz (k+di, l+dj),
 * di in -1..2, dj in -2..1, plane 15 + (di+1) + 4 (dj+2).  Vz row (i, j):
 * planes 0..14 couple Vz (i+di, j+dj), di in -2..2, dj in -1..1, plane
 * (di+2) + 5 (dj+1); planes 15..30 couple Vx (i+dk, j+dl), dk in -2..1,
 * dl in -1..2, plane 15 + (dk+2) + 4 (dl+1).  Level 0 is the fine operator
 * (times the cell volume), level l > 0 the Galerkin product R A P.  su / sv may
 * be NULL to query the sizes and the number of levels. */
mdz_status mdz_mg_stencils(mdz_ctx *ctx, int precision, int level, int *levels, int *Nx, int *Nz, double *su,
                           double *sv);

/* ---- resident state and the whole time step ------------------------------- */

/* Per-marker attributes kept on the device next to x, z, phase (the marker
 * arrays of the reference, SOURCE/header_MDOODZ.h:66-78).  MDZ_M_CMUL is a
 * per-marker cohesion multiplier (harness extension: seeded cohesion noise;
 * 1 reproduces the reference).  MDZ_M_P is the marker pressure
 * (particles.P): the time step projects it to p0_n and adds the step's
 * pressure increment to it (UpdateParticlePressure). */
enum {
    MDZ_M_SXXD = 0, MDZ_M_SZZD = 1, MDZ_M_SXZ = 2, MDZ_M_STRAIN_PL = 3, MDZ_M_STRAIN = 4, MDZ_M_T = 5,
    MDZ_M_CMUL = 6, MDZ_M_P = 7, MDZ_M_NATTR = 8
};
/* UpdateParticlePressure (SOURCE/RheologyParticles.c:1004-1123) with
 * Plith_trick = 0 and no subgrid diffusion (subgrid_diff < 2, the reference's
 * defaults): dp = p - p0_n on every centroid whose tag is not 30 (f->p is the
 * reference's p_in, f->p0_n the pressure projected from the markers at the
 * start of the step; host arrays), interpolated to the resident active
 * markers (Interp_Grid2P_centroids2) and added to their MDZ_M_P. */
mdz_status mdz_UpdateParticlePressure(mdz_ctx *ctx, mdz_fields *f);
/* UpdateParticleStress (SOURCE/RheologyParticles.c:1124-1447), StressUpdate =
 * 0 without rotation and subgrid diffusion: the increments sxxd - sxxd0,
 * szzd - szzd0 (centroids, not on air) and sxz - sxz0 (vertices) of the host
 * fields in f, interpolated to the resident markers and added to MDZ_M_SXXD,
 * MDZ_M_SZZD, MDZ_M_SXZ. */
mdz_status mdz_UpdateParticleStress(mdz_ctx *ctx, mdz_fields *f);
/* AccumulatedStrainII (SOURCE/RheologyParticles.c:191-537): dt times the
 * centroid strain-rate invariants of f (eII_el + eII_pl + eII_pwl + eII_lin +
 * eII_cst, and eII_pl alone), interpolated to the resident markers and added
 * to MDZ_M_STRAIN and MDZ_M_STRAIN_PL. */
mdz_status mdz_AccumulatedStrainII(mdz_ctx *ctx, mdz_fields *f, double dt);
mdz_status mdz_set_marker_attr(mdz_ctx *ctx, int attr, int n, const double *values);
mdz_status mdz_get_marker_attr(mdz_ctx *ctx, int attr, int n, double *values);

/* Batched marker transfers for a host-side time loop (the reference keeps
 * its markers in host arrays): positions, phases and any of the MDZ_M_NATTR
 * attributes (attrs[a] null: attribute a not copied; attrs null: none) in one
 * call, the copies spread over several streams so that they run on several
 * copy engines at once.  set: makes n the resident marker count, as
 * mdz_set_markers.  get: any of x, z, phase, vx, vz may be null.  Both return
 * when the copies are done.  Register the host arrays (mdz_host_register) to
 * make them DMA transfers. */
/* Output preparation (the data-parallel part of WriteOutputHDF5,
 * SOURCE/HDF5Output.c:237-895; the HDF5 calls stay with the caller).
 *
 * mdz_Interp_Phase2VizGrid replaces Interp_Phase2VizGrid
 * (SOURCE/ParticleRoutines.c:3004-3095) as WriteOutputHDF5 calls it
 * (HDF5Output.c:266-297): the visualisation grid of res_fact times the grid
 * resolution, its lines built by accumulation from the first grid line
 * (xviz: res_fact*(Nx-1)+1 values, zviz: res_fact*(Nz-1)+1; either may be
 * null), and per visualisation cell the phase of the resident marker with the
 * largest tent weight (the first in index order among equal ones), markers in
 * air centroids (BCp 30 / 31) left out, -1 where none: compo holds
 * (nxviz-1)*(nzviz-1) values, the reference's "VizGrid/compo" (res_fact 1)
 * and "VizGrid/compo_hr" (res_fact 2).
 *
 * mdz_output_field: the resident grid field `name` (an mdz_fields member, e.g.
 * "u", "p", "sxxd", "eta_n", "rho_s", "T") cast to float and multiplied by
 * `scale` with the product rounded to float, as DoubleToFloat + ScaleBack
 * (HDF5Output.c:44-73) prepare each "Centers/..", "Vertices/..", "VxNodes/..",
 * "VzNodes/.." dataset; out holds the field's node count. */
mdz_status mdz_Interp_Phase2VizGrid(mdz_ctx *ctx, int res_fact, signed char *compo, double *xviz, double *zviz);
mdz_status mdz_output_field(mdz_ctx *ctx, const char *name, double scale, float *out);

mdz_status mdz_set_marker_state(mdz_ctx *ctx, int n, const double *x, const double *z, const int *phase,
                                const double *const *attrs);
mdz_status mdz_get_marker_state(mdz_ctx *ctx, int n, double *x, double *z, int *phase, double *vx, double *vz,
                                double *const *attrs);

/* Copy grid fields between the caller's host arrays and the context's device
 * mirrors: to_device = 1 uploads every non-NULL member, 0 downloads them. */
mdz_status mdz_sync_fields(mdz_ctx *ctx, mdz_fields *f, int to_device);

/* ---- energy equation ------------------------------------------------------ */

/* Thermal boundary description (the reference's BCT BCt): centroid tags
 * (-1 active, 30 air; ncx*ncz) and, per wall, a type and a value per
 * boundary cell: typS / typN / valS / valN over the Nx-1 columns, typW / typE
 * / valW / valE over the Nz-1 rows.  Type 1: Dirichlet temperature at the
 * wall; type 2 on the south wall: prescribed flux; type 0: zero flux. */
typedef struct mdz_thermal_bc {
    const signed char *type;
    const signed char *typW, *typE, *typS, *typN;
    const double *valW, *valE, *valS, *valN;
} mdz_thermal_bc;

/* EnergyDirectSolve (SOURCE/ThermalRoutines.c:72-551, one iteration, polar =
 * 0): the implicit (theta = 1) energy step rho Cv (T_new - T) / dt =
 * div(k grad T_new) + Qr [+ Wdiss with shear_heating = 1] [+ adiabatic heat,
 * adiab_heating = 1: T alp v gz rho_n, 2: T alp (p - p0_n) / dt] on the
 * centroids, with the reference's five-point conductances (kx on the west /
 * east faces, kz on the south / north faces) and boundary rows.  The
 * symmetric positive definite system is solved matrix-free by Jacobi-
 * preconditioned conjugate gradients in FP64 to a relative residual of
 * rel_tol (<= 0: 1e-13), in place of the reference's CHOLMOD factorisation.
 * Reads f->T, rho_n, Cv, Qr, kx, kz (and Wdiss, alp, v, p, p0_n as the
 * heating switches ask); writes f->T (the new temperature; zeroC / scale_T on
 * air cells) and f->dT.  iterations and rel_residual (may be NULL) report the
 * solve.  MDZ_ERR_UNSUPPORTED for centroid tags other than -1 / 30 (free
 * surface, periodic), MDZ_ERR_NOT_CONVERGED when max_iterations pass,
 * MDZ_ERR_STATE for a negative temperature (the reference exits there). */
mdz_status mdz_EnergyDirectSolve(mdz_ctx *ctx, mdz_fields *f, const mdz_thermal_bc *bc, double dt, double gz,
                                 int shear_heating, int adiab_heating, double scale_T, double rel_tol,
                                 int max_iterations, int *iterations, double *rel_residual);

/* PureShearALE (SOURCE/AdvectionRoutines.c:634-734, ispureshear_ale = 1,
 * no free surface): the mean Vx of the Dirichlet nodes (tag 0) of the west and
 * east walls (Vx rows 0..Nz-1) and the mean Vz of the Dirichlet nodes of the
 * south (tag 0) and north (tag 0 or 30) walls (Vz columns 0..Nx-1), each summed
 * in the reference's loop order, move xmin, xmax, zmin, zmax by dt times that
 * velocity; the grid lines are then regenerated over the new box as
 * SetGridCoordinates accumulates them.  u_in / v_in: host velocities, or NULL
 * for the resident ones.  bounds (4 doubles, may be NULL) receives the new
 * xmin, xmax, zmin, zmax.  The Dirichlet values are not changed
 * (mdz_set_boundary_values). */
mdz_status mdz_PureShearALE(mdz_ctx *ctx, const double *u_in, const double *v_in, double dt, double *bounds);
/* Replace the Dirichlet values of the Vx and Vz nodes (the BCu.val / BCv.val
 * arrays of the grid description; either may be NULL to keep it), as the
 * reference's SetBCs rewrites them at the start of every step. */
mdz_status mdz_set_boundary_values(mdz_ctx *ctx, const double *BCu_val, const double *BCv_val);
/* The grid the context works on now (after any PureShearALE): box[6] =
 * xmin, xmax, zmin, zmax, dx, dz, and the coordinate lines xg (Nx), zg (Nz),
 * xc (Nx-1), zc (Nz-1), xvz (Nx+1), zvx (Nz+1); any pointer may be NULL. */
mdz_status mdz_get_grid(mdz_ctx *ctx, double *box, double *xg, double *zg, double *xc, double *zc, double *xvz,
                        double *zvx);

/* Switches of one time step (the reference's params / Nparams keys). */
typedef struct mdz_model {
    mdz_rheo_params rheo;   /* dt, elasticity, averaging, viscosity limits, scales        */
    double gx, gz;          /* gravity                                                      */
    int newton;             /* 1: Newton linearisation (Jacobian), 0: Picard                */
    int nit_max;            /* non-linear iterations allowed (Nparams.nit_max)              */
    double rel_tol, abs_tol;/* non-linear tolerances on resx/resz/resp (rel_tol_u etc.)     */
    double lin_rtol;        /* relative tolerance of each linear defect solve               */
    int lin_maxit;
    int line_search;        /* 1: LineSearchDecoupled (6 trial steps)                      */
    double line_search_min;
    int precision;          /* 64: plain FP64; 32: FP32 stencils + V-cycles in FP64 refinement */
    int learned_guess;      /* local rheology starts (MLP weights loaded with mdz_mlp_*):
                               1: the MLP's guess in the first FP64 evaluation of the step,
                                  then each evaluation polishes the solutions the previous
                                  one converged to; 2: the MLP's guess in every evaluation;
                                  0: the reference's start                                  */
    int itp_stencil;        /* 1 or 9                                                        */
    int softening;          /* 0: smooth erfc law (reference); 1: linear law                 */
    int advect;             /* 1: update marker stress/strain and advect (RK4)               */
    /* Picard -> Newton switch of Main_DOODZ.c:728-743: with picard2newton = 1 the
     * step starts with Picard iterations and switches to the Jacobian once resx
     * or resz fell below pic2newt_cond times its first value, or after
     * nit_pic_max iterations (Nparams.Picard2Newton, Pic2NewtCond, nit_Pic_max). */
    int picard2newton;
    double pic2newt_cond;
    int nit_pic_max;
    int newton_maxit;       /* Krylov cap of a Jacobian solve before the Picard operator takes
                               that iteration over (0: lin_maxit)                              */
    /* 1: each defect solve asks only for the reduction the non-linear iteration
     * can use (Eisenstat-Walker forcing, eta_k = 0.9 (r_k / r_k-1)^2 within
     * [lin_rtol, 0.1], and no tighter than half the remaining distance to
     * rel_tol); 0: every solve to lin_rtol.  No counterpart in the reference,
     * whose direct solver has no tolerance. */
    int adaptive_lin_tol;
    /* the first fp32_rheology_its non-linear iterations evaluate the local
     * rheology in FP32 (FP64 where a solve fails); convergence decisions and
     * the final update always run in FP64.  0: FP64 throughout.  (FP32 stresses
     * put a floor of ~1e-7 of the stress level under the momentum residual, so
     * only the first, Picard-type iterations can use them.)  No counterpart in
     * the reference. */
    int fp32_rheology_its;
    /* > 0: a defect solve whose non-linear iteration has its largest relative
     * block residual below this value keeps the multigrid hierarchy of the
     * previous solve (the viscosities have nearly converged) instead of
     * rebuilding it.  0: rebuilt for every solve.  No counterpart in the
     * reference. */
    double mg_reuse_below;
    /* 1: after the advection, reseed the markers as CountPartCell(RESEED = 1)
     * (model.Reseed with cpc = 1, Main_DOODZ.c:1235; mdz_CountPartCell) with
     * particles.min_part_cell and model.DirectNeighbour; T and the stresses of
     * new markers then come from the step's grid fields T, sxxd, szzd, sxz. */
    int reseed;
    int min_part_cell;
    int direct_neighbour;
    /* 1: the box deforms with the flow (model.ispureshear_ale = 1, PureShearALE,
     * SOURCE/AdvectionRoutines.c:634-734, called before the marker advection,
     * Main_DOODZ.c:1107-1109): each wall moves by dt times the mean velocity of
     * its Dirichlet nodes and the grid lines are regenerated over the new box
     * (SetGridCoordinates, SOURCE/GridRoutines.c:230-300) before the markers are
     * advected on it.  The report returns the new box; the Dirichlet values of
     * the next step follow from it (the reference's SetBCs runs again on the new
     * coordinates): mdz_set_boundary_values.  0: fixed box. */
    int ispureshear_ale;
} mdz_model;

#define MDZ_HISTORY 32
typedef struct mdz_step_report {
    int nonlinear_its, linear_its, converged, stagnated;
    int picard_fallbacks;             /* Newton iterations solved with the Picard operator instead */
    double res0[3], res[3];           /* first and final resx, resz, resp                    */
    long long local_solves, local_fallbacks, local_failures;
    double ms_projection, ms_rheology, ms_residual, ms_solve, ms_line_search, ms_markers, ms_total;
    int newton_its;                   /* iterations solved with the Jacobian                  */
    long long local_iterations;       /* local Newton updates of all local rheology solves    */
    /* per non-linear iteration (the first MDZ_HISTORY; the reference prints the same
     * lines): resx, resz, resp before the solve, Krylov iterations and relative
     * residual of its defect solve, 1 where the Jacobian was used */
    double res_history[MDZ_HISTORY][3];
    int lin_its_history[MDZ_HISTORY];
    double lin_rel_history[MDZ_HISTORY];
    int newton_history[MDZ_HISTORY];
    int precision_fallbacks;          /* FP32-refined solves that missed min(10 x their tolerance, 0.5),
                                         redone in FP64 */
    int markers_added;                /* markers created by the reseeding (model.reseed)      */
    double xmin, xmax, zmin, zmax;    /* the box after the step (moves with ispureshear_ale)  */
} mdz_step_report;

/* One time step of Main_DOODZ.c's loop (SOURCE/Main_DOODZ.c:459-1320) on the
 * resident state: marker->grid projections, grid properties, the Newton (or
 * Picard) loop with matrix-free defect solves and optional line search, the
 * final rheology update, marker stress/strain updates and RK4 advection.
 * Velocities and pressure (mdz_fields u, v, p on the device) are the initial
 * guess and receive the solution. */
mdz_status mdz_time_step(mdz_ctx *ctx, const mdz_materials *mat, const mdz_model *model, mdz_step_report *rep);

/* Read back the resident velocity / pressure solution (any pointer may be NULL). */
mdz_status mdz_get_velocity(mdz_ctx *ctx, double *u, double *v, double *p);

/* Wait for all work queued on the context's stream. */
mdz_status mdz_sync(mdz_ctx *ctx);

/* Launch timing of the main kernel classes with CUDA events on the context's
 * stream (off by default; turning it on or off resets the totals).  Classes:
 * 0 local rheology, 1 Stokes operator apply inside the Krylov solver,
 * 2 multigrid V-cycle (the whole preconditioner application), 3 projection,
 * 4 learned-guess inference, 5 Krylov vector work of the GCR iterations
 * (orthogonalisation, dot products, updates), 6 multigrid set-up (level-0
 * stencils, Galerkin products, coarsest inverse).  Returns the summed time (ms), the summed
 * algorithmic bytes and the number of launches of one class. */
mdz_status mdz_set_profiling(mdz_ctx *ctx, int on);
mdz_status mdz_kernel_timing(mdz_ctx *ctx, int kernel_class, double *ms, double *bytes, long long *launches);

#ifdef __cplusplus
}
#endif
#endif /* MDOODZ_GPU_H */
