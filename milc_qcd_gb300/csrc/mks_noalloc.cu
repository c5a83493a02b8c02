// mks_noalloc.cu -- D_eo for callers that cannot allocate device memory.
//
// mks_dslash_fn_field_dev stages its input and output in structure-of-
// arrays buffers that the library allocates with cudaMalloc on first use.
// Some callers cannot allow that: an application that hands nearly all
// device memory to its own pool allocator before calling in, or code that
// must not run a device-wide synchronising call such as cudaMalloc at that
// point.  mks_dslash_fn_field_dev_noalloc runs the same layout-conversion
// kernels and the FP64 D_eo with the staging buffers placed in the fixed
// array below, so it allocates nothing.  It launches the plain one-source
// D_eo kernel (k_dslash with one source per thread, 256-thread blocks), not
// the autotuned shape of the allocating entry point: the results agree to
// rounding, the speed may differ.
//
// Limits and sharing: the array holds MKS_NOALLOC_SCRATCH_BYTES (32 MiB),
// the FP64 input and output staging for lattices of up to 349,525 sites
// (e.g. 16^3x64 or 24^4); larger lattices are rejected with MKS_ERR_ARG.
// Every GPU that loads this library keeps the array until the process
// exits.  All calls share it and it keeps the last call's contents; every
// byte a call reads is written earlier in the same call, so nothing needs
// clearing, but two calls that overlap on the GPU (from different host
// threads, or through another stream) race on it.
//
// Set-up: mks_init (with the library's device current) resolves the
// array's device address with cudaGetSymbolAddress and loads the kernel
// this file launches, so the array and the kernel's code are resident
// before the caller's pool allocator takes the device memory, and no call
// of the entry point loads a module.  mks_finalize forgets the address; the
// next mks_init looks it up again.
#include <cstring>
#include "mks_internal.cuh"
#include "mks_dslash.cuh"

namespace mks {

constexpr size_t MKS_NOALLOC_SCRATCH_BYTES = (size_t)32 << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[MKS_NOALLOC_SCRATCH_BYTES];
static void *g_noalloc_addr = nullptr;  // device address of the array on the library's device

// the one D_eo kernel this file launches
static void (*const noalloc_kernel)(const LinkF64, const LinkF64, const DslashArgs<VecF64, VecF64, VecF64>,
                                    const NoFinish) =
    k_dslash<double, LinkF64, VecF64, VecF64, 1, EPI_PLAIN, 0, NoFinish>;

// called by mks_init after cudaSetDevice
int noalloc_prepare() {
  void *p = nullptr;
  MKS_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
  cudaFuncAttributes fa;
  MKS_CUDA(cudaFuncGetAttributes(&fa, noalloc_kernel));
  g_noalloc_addr = p;
  return MKS_OK;
}

// called by mks_finalize
void noalloc_forget() { g_noalloc_addr = nullptr; }

// out (one parity, SoA) = D in (other parity, SoA), FP64, one source
static int noalloc_dslash64(const LinkSlot &sl, int out_par, double2 *in, double2 *out) {
  Context &c = ctx();
  DslashArgs<VecF64, VecF64, VecF64> a;
  memset(&a, 0, sizeof a);
  a.g = c.geom;
  a.out_par = out_par;
  a.nsrc = 1;
  a.groups = 1;
  a.in[0].p = in;
  a.out[0].p = out;
  LinkF64 fat = {sl.fat64}, lng = {sl.lng64};
  timing_begin(MKS_K_DSLASH_F64);  // counts the launch (and times it when timing is on)
  noalloc_kernel<<<grid_for(c.Vh, 256), 256, 0, c.stream>>>(fat, lng, a, NoFinish());
  timing_end(MKS_K_DSLASH_F64);
  MKS_CUDA(cudaGetLastError());
  return MKS_OK;
}

}  // namespace mks

using namespace mks;

extern "C" int mks_dslash_fn_field_dev_noalloc(const double *src_dev, double *dst_dev, int parity, int slot) {
  MKS_TRY(check_ready());
  Context &c = ctx();
  if (2 * c.V * 6 * sizeof(double) > MKS_NOALLOC_SCRATCH_BYTES) return MKS_ERR_ARG;
  if (slot < 0 || slot >= MKS_MAX_SLOTS) return MKS_ERR_ARG;
  if (!c.slots[slot].valid) return MKS_ERR_STATE;
  if (!src_dev || !dst_dev || parity < MKS_ODD || parity > MKS_EVENANDODD) return MKS_ERR_ARG;
  if (!g_noalloc_addr) return MKS_ERR_STATE;  // mks_init resolves it
  double2 *in = (double2 *)g_noalloc_addr;  // full-lattice SoA input  [2][3][Vh]
  double2 *out = in + 6 * c.Vh;             // full-lattice SoA output [2][3][Vh]
  const LinkSlot &sl = c.slots[slot];
  for (int op = 0; op < 2; op++) {
    bool want = (parity == MKS_EVENANDODD) || (parity == MKS_EVEN && op == 0) || (parity == MKS_ODD && op == 1);
    if (!want) continue;
    MKS_TRY(vec_aos_to_soa64(src_dev, in + (size_t)(1 - op) * 3 * c.Vh, 1 - op));
  }
  for (int op = 0; op < 2; op++) {
    bool want = (parity == MKS_EVENANDODD) || (parity == MKS_EVEN && op == 0) || (parity == MKS_ODD && op == 1);
    if (!want) continue;
    double2 *pin = in + (size_t)(1 - op) * 3 * c.Vh, *pout = out + (size_t)op * 3 * c.Vh;
    MKS_TRY(noalloc_dslash64(sl, op, pin, pout));
    MKS_TRY(vec_soa64_to_aos(pout, dst_dev, op));
  }
  MKS_CUDA(cudaStreamSynchronize(c.stream));
  return MKS_OK;
}
