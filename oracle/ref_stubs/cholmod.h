/* Minimal stand-in declarations so that the reference's hot-path sources
 * compile without SuiteSparse.  Only opaque struct types are declared: no
 * CHOLMOD routine is ever called on the hot path, and the few symbols the
 * reference references are defined in ref_stubs.c as aborting stubs. */
#ifndef MDZ_REF_STUB_CHOLMOD_H
#define MDZ_REF_STUB_CHOLMOD_H
typedef struct { int stub_unused; } cholmod_common;
typedef struct { int stub_unused; } cholmod_factor;
typedef struct { int stub_unused; } cholmod_sparse;
typedef struct { int stub_unused; } cholmod_dense;
#endif
