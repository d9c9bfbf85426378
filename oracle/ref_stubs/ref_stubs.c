/*
 * Aborting definitions for the symbols that the reference's hot-path object
 * files reference but that live in files this harness does not build
 * (SuiteSparse solvers, HDF5 output, the thermal solver).  None of them is on
 * the projection / rheology / residual / advection path; if one is ever
 * reached the harness aborts loudly rather than returning garbage.
 *
 * Test infrastructure only: linked into oracle/_ref/libmdoodz_ref.so, never
 * into the product library.
 */
#include <stdio.h>
#include <stdlib.h>

#define MDZ_REF_STUB(name)                                                     \
    void name(void) {                                                          \
        fprintf(stderr, "reference harness: stub '%s' reached\n", #name);     \
        abort();                                                               \
    }

MDZ_REF_STUB(AddFieldToGroup_generic)
MDZ_REF_STUB(AddGroup_to_hdf5)
MDZ_REF_STUB(create_output_hdf5)
MDZ_REF_STUB(DirectStokes)
MDZ_REF_STUB(DirectStokesDecoupled)
MDZ_REF_STUB(DirectStokesDecoupledComp)
MDZ_REF_STUB(KSPStokesDecoupled)
MDZ_REF_STUB(KillerSolver)
MDZ_REF_STUB(ScaleBackD)
MDZ_REF_STUB(FactorEnergyCHOLMOD)
MDZ_REF_STUB(SolveEnergyCHOLMOD)
MDZ_REF_STUB(TransposeA)
MDZ_REF_STUB(cholmod_start)
MDZ_REF_STUB(cholmod_finish)
MDZ_REF_STUB(cholmod_free_factor)
MDZ_REF_STUB(cs_spfree)
