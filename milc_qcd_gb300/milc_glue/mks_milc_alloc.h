/* mks_milc_alloc.h -- prototypes of the two host allocators that MILC's
 * link-construction files name when compiled with -DUSE_FL_GPU
 * (generic_ks/fermion_links_hisq_load_milc.c:21-27, fn_links_milc.c:11-17,
 * fermion_links_from_site.c:10-55 through include/generic_quda.h).  A MILC
 * build that binds libmilc_ks_gb300 instead of QUDA force-includes this
 * header (-include mks_milc_alloc.h); mks_milc_glue.c defines them. */
#ifndef MKS_MILC_ALLOC_H
#define MKS_MILC_ALLOC_H
#include <stddef.h>
void *qudaAllocatePinned(size_t bytes);
void qudaFreePinned(void *ptr);
#endif
