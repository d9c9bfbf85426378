/*
 * CPU oracle: a plain-C restatement of the MDOODZ 6.0 hot-path algorithms,
 * used ONLY as the reference for comparisons in tests/, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py.  The product library never links or calls it.
 *
 * Each function cites the reference function (path:line inside the MDOODZ 6.0
 * repository) whose arithmetic it restates.  The restatement is pinned against
 * the reference's own compiled functions through the golden fixtures in
 * tests/golden/ (generated by tests/golden/make_golden.py from
 * oracle/_ref/libmdoodz_ref.so).
 *
 * Grid and tag conventions are those of include/mdoodz_gpu.h.
 */
#ifndef MDZ_ORACLE_H
#define MDZ_ORACLE_H
#include "mdoodz_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* P2Mastah (SOURCE/ParticleRoutines.c:3226-3537), serial scatter form. */
int orc_p2g(const mdz_grid_desc *g, int n, const double *x, const double *z, const int *phase, int n_phases,
            const double *mat_prop, double *node_field, const signed char *node_type, int flag, int avg, int prop,
            int centroid, int itp_stencil, double *phase_perc);

/* CountPartCell_Old counting (SOURCE/ParticleRoutines.c:4530-4560 and 4898-4950). */
int orc_count(const mdz_grid_desc *g, int n, const double *x, const double *z, const int *phase, int n_phases,
              int *nb_part_cell, int *nb_part_vert, int *phase_count_cell, int *phase_count_vert);

/* Interp_Grid2P (SOURCE/ParticleRoutines.c:2439-2608) for node_set 0/-1/-2 and
 * Interp_Grid2P_centroids2 (SOURCE/ParticleRoutines.c:2612-2862) for node_set 1. */
int orc_g2p(const mdz_grid_desc *g, int n, const double *x, const double *z, const int *phase,
            const double *node_field, int node_set, double *out);

/* RogerGuntherII + V2P (TarasCorr = 0) + isoutPart
 * (SOURCE/AdvectionRoutines.c:569-628, SOURCE/ParticleRoutines.c:60-252,
 *  SOURCE/AdvectionRoutines.c:314-335).  Updates x, z, phase, vx, vz in place. */
int orc_rk4(const mdz_grid_desc *g, int n, double *x, double *z, int *phase, double *vx, double *vz,
            const double *u, const double *v, double dt);

/* Marker reseeding: CountPartCell with RESEED = 1, one OpenMP thread
 * (SOURCE/ParticleRoutines.c:3543-4480, 977-1030, 841-890, 648-762, 259-520).
 * attr: the MDZ_M_NATTR marker attribute arrays, all of length cap.  Returns
 * the new marker count, -1 for a deficient quarter cell without neighbours,
 * -2 when cap is too small; n_added receives the number of new markers. */
int orc_reseed(const mdz_grid_desc *g, int n, int cap, double *x, double *z, int *phase, double *vx, double *vz,
               double *const *attr, int min_part_cell, int direct, const double *T_n, const double *sxxd_n,
               const double *szzd_n, const double *sxz_s, const double *p_n, int *n_added);

#ifdef __cplusplus
}
#endif
#endif

#ifdef __cplusplus
extern "C" {
#endif
/* StrainRateComponents (SOURCE/RheologyDensity.c:1902-1984), incl. the two
 * InterpCentroidsToVerticesDouble calls at its end. */
int orc_strain_rates(const mdz_grid_desc *g, mdz_fields *f);
/* InterpCentroidsToVerticesDouble (SOURCE/GridRoutines.c:106-198), non-periodic. */
int orc_c2v(const mdz_grid_desc *g, const double *cen, double *ver);
/* InterpVerticesToCentroidsDouble (SOURCE/GridRoutines.c:204-228). */
int orc_v2c(const mdz_grid_desc *g, double *cen, const double *ver);
/* NonNewtonianViscosityGrid + Viscosity, isotropic (SOURCE/RheologyDensity.c:961-1415, 44-707).
 * not_conv (optional, 2 ints) receives the number of local visco-elastic and
 * visco-plastic solves that hit the 20-iteration cap. */
int orc_viscosity_grid(const mdz_grid_desc *g, const mdz_materials *mat, const mdz_rheo_params *prm, mdz_fields *f,
                       int *not_conv);
/* RheologicalOperators, isotropic (SOURCE/RheologyDensity.c:713-954). */
int orc_rheo_operators(const mdz_grid_desc *g, const mdz_rheo_params *prm, mdz_fields *f, int jacobian);
/* EvaluateRHS, incompressible, non-polar (SOURCE/StokesRoutines.c:922-1133). */
int orc_rhs(const mdz_grid_desc *g, const mdz_rheo_params *prm, double gx, double gz, mdz_fields *f);
#ifdef __cplusplus
}
#endif

#ifdef __cplusplus
extern "C" {
#endif
/* Decoupled Stokes rows (SOURCE/StokesAssemblyDecoupled.c): y = K x (residual = 0)
 * or y = K x - b (residual = 1), Picard (jacobian = 0) or Newton (jacobian = 1),
 * every row times the cell volume; non-equation entries set to 0. */
int orc_stokes_apply(const mdz_grid_desc *g, const mdz_fields *f, int jacobian, int residual, const double *u,
                     const double *v, const double *p, double *yu, double *yv, double *yp);
/* EvaluateStokesResidualDecoupled (SOURCE/StokesRoutines.c:839-920). */
int orc_residual(const mdz_grid_desc *g, mdz_fields *f, double *norms3);
#ifdef __cplusplus
}
#endif
