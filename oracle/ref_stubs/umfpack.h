/* Stand-in for UMFPACK's header: nothing on the hot path uses it. */
#ifndef MDZ_REF_STUB_UMFPACK_H
#define MDZ_REF_STUB_UMFPACK_H
#endif
