// mks_pending.cu -- entry points whose kernels are not in this build yet.
// They fail loudly with MKS_ERR_UNSUPPORTED; nothing falls back to a CPU path.
#include "mks_internal.cuh"

extern "C" {
int mks_fermion_force_multi_hisq(double, const double *, const double *const *, int, const int *, int, double *) {
  return MKS_ERR_UNSUPPORTED;
}
}
