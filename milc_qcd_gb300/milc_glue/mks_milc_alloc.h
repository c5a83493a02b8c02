/* mks_milc_alloc.h -- prototypes of the helpers that MILC's files name
 * when compiled with -DUSE_FL_GPU / -DUSE_FF_GPU and that a QUDA build takes
 * from include/generic_quda.h (all under HAVE_QUDA there):
 *   qudaAllocatePinned / qudaFreePinned and their "Managed" aliases
 *     (generic_ks/fermion_links_hisq_load_milc.c:21-27, fn_links_milc.c:11-17,
 *     generic/make_lattice.c:27, ks_imp_rhmc/update_rhmc.c:150-153);
 *   create_G_from_site_quda / destroy_G_quda
 *     (generic_ks/fermion_links_from_site.c:14-58).
 * A MILC build that binds libmilc_ks_gb300 instead of QUDA force-includes
 * this header (-include mks_milc_alloc.h); mks_milc_glue.c defines them.
 * The link-array helpers return and take void * here because MILC's types
 * are not yet declared where this header is included. */
#ifndef MKS_MILC_ALLOC_H
#define MKS_MILC_ALLOC_H
#include <stddef.h>
void *qudaAllocatePinned(size_t bytes);
void qudaFreePinned(void *ptr);
#ifndef qudaAllocateManaged
#define qudaAllocateManaged qudaAllocatePinned
#define qudaFreeManaged qudaFreePinned
#endif
void *create_G_from_site_quda(void);
void destroy_G_quda(void *links);
#endif
