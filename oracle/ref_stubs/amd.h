/* Stand-in for AMD's header: nothing on the hot path uses it. */
#ifndef MDZ_REF_STUB_AMD_H
#define MDZ_REF_STUB_AMD_H
#endif
