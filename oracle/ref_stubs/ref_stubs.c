/*
 * Aborting definitions for the symbols that the reference's hot-path object
 * files reference but that live in files this harness does not build
 * (SuiteSparse solvers, HDF5 output).  None of them is on the projection /
 * rheology / residual / advection path; if one is ever reached the harness
 * aborts loudly rather than returning garbage.  The thermal solver's
 * CHOLMOD calls have stand-ins in ref_harness.c instead.
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
