/* Stand-in for CXSparse's header: opaque types only (see cholmod.h here). */
#ifndef MDZ_REF_STUB_CS_H
#define MDZ_REF_STUB_CS_H
typedef struct { int stub_unused; } cs_di;
typedef cs_di cs;
#endif
