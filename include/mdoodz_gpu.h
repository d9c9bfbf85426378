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
 * device mirrors; the host arrays stay owned by the caller. */
mdz_status mdz_create(mdz_ctx **ctx, const mdz_grid_desc *grid, int n_phases, long long max_markers);
void mdz_destroy(mdz_ctx *ctx);
const char *mdz_last_error(const mdz_ctx *ctx);
/* Number of kernels this context has launched so far (for launch accounting). */
long long mdz_kernel_launches(const mdz_ctx *ctx);

/* Upload markers (positions and phase) to the context's resident marker store
 * and mark the cell binning stale.  n <= max_markers. */
mdz_status mdz_set_markers(mdz_ctx *ctx, int n, const double *x, const double *z, const int *phase);
/* Download resident marker positions / phases (any pointer may be NULL). */
mdz_status mdz_get_markers(mdz_ctx *ctx, int n, double *x, double *z, int *phase, double *vx, double *vz);

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

#ifdef __cplusplus
}
#endif
#endif /* MDOODZ_GPU_H */
