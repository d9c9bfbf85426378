/*
 * mdoodz_refshim.h -- set-up entry points of the reference-signature
 * drop-ins (mdoodz6.0_gb300/refshim/mdz_refshim.c), which define P2Mastah,
 * CountPartCell, StrainRateComponents, NonNewtonianViscosityGrid,
 * RheologicalOperators, UpdateNonLinearity, BuildStokesOperatorDecoupled,
 * BuildJacobianOperatorDecoupled, EvaluateStokesResidualDecoupled,
 * SolveStokesDefectDecoupled, LineSearchDecoupled, Interp_Grid2P,
 * Interp_Grid2P_centroids2, RogerGuntherII, UpdateParticleStress and
 * AccumulatedStrainII with the argument lists of the reference's
 * SOURCE/header_MDOODZ.h (lines 340-592), computed on the GPU.
 *
 * No counterpart in the reference: these four manage the GPU context the
 * drop-ins share.  The structure tags are those of the reference's header
 * (or of the generated layout view, include/mdoodz_ref_types.h).
 */
#ifndef MDOODZ_REFSHIM_H
#define MDOODZ_REFSHIM_H

#ifdef __cplusplus
extern "C" {
#endif

struct _params;
struct _grid;
struct _p_markers;

/* Create the GPU context for the caller's grid (coordinates, boundary tags;
 * the grid must not change afterwards) with room for the markers' Nb_part_max.
 * Optional: the first drop-in that receives a params argument makes it.
 * Returns 0 or an mdz_status.  MDZ_REFSHIM_PRECISION=32 in the environment
 * selects the FP32-refined defect solves. */
int mdz_gpu_init(const struct _params *model, const struct _grid *mesh, const struct _p_markers *particles);
/* Release the context and the drop-ins' host buffers. */
void mdz_gpu_finalize(void);
/* mdz_status of the last drop-in (every failure also prints and exits as the
 * reference does at the same points). */
int mdz_gpu_last_status(void);
/* The drop-ins return with their outputs in the caller's arrays (synchronous);
 * this waits for any device work still queued and returns its status. */
int mdz_gpu_sync_to_host(unsigned int fieldmask);

#ifdef __cplusplus
}
#endif
#endif
