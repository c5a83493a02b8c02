// mks_context.cu -- library context, errors, timing, layout conversion and
// fermion-link residency (the part of the C ABI that replaces MILC's QUDA
// set-up and link cache: generic/milc_to_quda_utilities.c:11-41,
// generic_ks/fermion_links_fn_load_gpu.c:19-78, include/fn_links.h:9-17).
#include <cstring>
#include <cstdlib>
#include <cmath>
#include <string>
#include "mks_internal.cuh"

namespace mks {

static Context g_ctx;
static char g_errmsg[512] = "";

Context &ctx() { return g_ctx; }

void set_last_error(cudaError_t e, const char *what, const char *file, int line) {
  snprintf(g_errmsg, sizeof g_errmsg, "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
}

int check_ready(bool need_lattice) {
  if (!g_ctx.initialised) return MKS_ERR_STATE;
  if (need_lattice && g_ctx.V == 0) return MKS_ERR_STATE;
  return MKS_OK;
}

int dev_alloc(void **p, size_t bytes) {
  *p = nullptr;
  if (bytes == 0) return MKS_OK;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    set_last_error(e, "cudaMalloc", __FILE__, __LINE__);
    cudaGetLastError();
    return MKS_ERR_NOMEM;
  }
  return MKS_OK;
}

void dev_free(void *p) {
  if (p) cudaFree(p);
}

// ---------------- timing ----------------
static const int EV_POOL = 4096;

void timing_begin(int family) {
  Context &c = g_ctx;
  if (c.capture) {
    Capture &k = *c.capture;
    k.family.push_back(family);
    if (k.timed) {
      cudaEvent_t e0, e1;
      cudaEventCreate(&e0);
      cudaEventCreate(&e1);
      k.ev.push_back(e0);
      k.ev.push_back(e1);
      // an external record becomes an event-record node that fires on every replay
      cudaEventRecordWithFlags(e0, c.stream, cudaEventRecordExternal);
    }
    return;
  }
  c.launches++;
  c.kernel_launches[family]++;
  if (!c.timing) return;
  if (c.ev_used >= EV_POOL) timing_flush();
  cudaEventRecord(c.ev_pool[2 * c.ev_used], c.stream);
  c.ev_family[c.ev_used] = family;
}

void timing_end(int family) {
  Context &c = g_ctx;
  (void)family;
  if (c.capture) {
    if (c.capture->timed) cudaEventRecordWithFlags(c.capture->ev.back(), c.stream, cudaEventRecordExternal);
    return;
  }
  if (!c.timing) return;
  cudaEventRecord(c.ev_pool[2 * c.ev_used + 1], c.stream);
  c.ev_used++;
}

int timing_flush() {
  Context &c = g_ctx;
  if (c.ev_used == 0) return MKS_OK;
  MKS_CUDA(cudaStreamSynchronize(c.stream));
  for (int i = 0; i < c.ev_used; i++) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c.ev_pool[2 * i], c.ev_pool[2 * i + 1]);
    c.kernel_ms[c.ev_family[i]] += ms;
  }
  c.ev_used = 0;
  return MKS_OK;
}

void capture_account(const Capture &k) {
  Context &c = g_ctx;
  for (size_t i = 0; i < k.family.size(); i++) {
    c.launches++;
    c.kernel_launches[k.family[i]]++;
    if (k.timed && c.timing) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, k.ev[2 * i], k.ev[2 * i + 1]);
      c.kernel_ms[k.family[i]] += ms;
    }
  }
}

// Scratch for a reduction of nsum sums per block over `blocks` blocks
// (grid_reduce_last in mks_reduce.cuh): block rows + group rows, and the
// top counter + one counter per group.  Grown, never shrunk; counters are
// zeroed when (re)allocated and are left at zero by every launch.
int ensure_red(int nsum, int blocks) {
  Context &c = g_ctx;
  const size_t ngroups = ((size_t)blocks + RED_GROUP - 1) / RED_GROUP;
  const size_t need = (size_t)nsum * ((size_t)blocks + ngroups), need_count = 1 + ngroups;
  if (c.red.max_partials < need) {
    dev_free(c.red.partials);
    c.red.partials = nullptr;
    c.red.max_partials = 0;
    const size_t n = need < 65536 ? 65536 : need;
    MKS_TRY(dev_alloc((void **)&c.red.partials, n * sizeof(double)));
    c.red.max_partials = n;
  }
  if (!c.red.err) {
    MKS_TRY(dev_alloc((void **)&c.red.err, sizeof(int)));
    MKS_CUDA(cudaMemsetAsync(c.red.err, 0, sizeof(int), c.stream));
  }
  if (c.red.max_count < need_count) {
    dev_free(c.red.count);
    c.red.count = nullptr;
    c.red.max_count = 0;
    const size_t n = need_count < 4096 ? 4096 : need_count;
    MKS_TRY(dev_alloc((void **)&c.red.count, n * sizeof(unsigned int)));
    MKS_CUDA(cudaMemsetAsync(c.red.count, 0, n * sizeof(unsigned int), c.stream));
    c.red.max_count = n;
  }
  return MKS_OK;
}

int red_check() {
  Context &c = g_ctx;
  if (!c.red.err) return MKS_OK;
  int e = 0;
  MKS_CUDA(cudaMemcpyAsync(&e, c.red.err, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
  MKS_CUDA(cudaStreamSynchronize(c.stream));
  if (!e) return MKS_OK;
  MKS_CUDA(cudaMemsetAsync(c.red.err, 0, sizeof(int), c.stream));
  if (e & 6) {
    // value 2: a TMA-staged D_eo tile gave up waiting for its links (it
    // computed nothing); value 4: its copies were still in flight after the
    // second wait.  The staged kernel is off from now on.
    tma_disable();
    snprintf(g_errmsg, sizeof g_errmsg,
             "TMA-staged D_eo: link staging did not complete within its wait limit (%s); the staged kernel is "
             "switched off for this process",
             (e & 4) ? "copies still in flight" : "tile skipped");
    return MKS_ERR_TIMEOUT;
  }
  snprintf(g_errmsg, sizeof g_errmsg, "reduction scratch too small for a launch (internal sizing error)");
  return MKS_ERR_CUDA;
}

// ---------------- layout conversion kernels ----------------
// full AoS vector field [V][6] -> one parity SoA double2 [3][Vh].  One
// complex number per thread: the parity half of a MILC field is 3*Vh
// consecutive complex numbers, taken in order, so the reads (and in
// k_vec_soa_to_aos the writes) of the AoS side are contiguous across a warp
// -- the AoS side is often a page-locked host array read over the host link.
// 16-byte accesses where the array allows them.
__device__ __forceinline__ double2 aos_get(const double *base, size_t t) {
  if (((uintptr_t)base & 15) == 0) return reinterpret_cast<const double2 *>(base)[t];
  return make_double2(base[2 * t], base[2 * t + 1]);
}
__global__ void k_vec_aos_to_soa(const double *__restrict__ aos, double2 *__restrict__ soa, int par, int Vh) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= 3 * (size_t)Vh) return;
  const size_t h = t / 3;
  const int c = (int)(t - 3 * h);
  soa[(size_t)c * Vh + h] = aos_get(aos + (size_t)par * Vh * 6, t);
}
__global__ void k_vec_soa_to_aos(const double2 *__restrict__ soa, double *__restrict__ aos, int par, int Vh) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= 3 * (size_t)Vh) return;
  const size_t h = t / 3;
  const int c = (int)(t - 3 * h);
  const double2 v = soa[(size_t)c * Vh + h];
  double *base = aos + (size_t)par * Vh * 6;
  if (((uintptr_t)base & 15) == 0) {
    reinterpret_cast<double2 *>(base)[t] = v;
  } else {
    base[2 * t] = v.x;
    base[2 * t + 1] = v.y;
  }
}
// links [V][4][18] -> [2][4][9][Vh]
__global__ void k_links_aos_to_soa(const double *__restrict__ aos, double2 *__restrict__ soa, int Vh) {
  int h = blockIdx.x * blockDim.x + threadIdx.x;
  int par = blockIdx.y, dir = blockIdx.z;
  if (h >= Vh) return;
  const double *s = aos + (((size_t)par * Vh + h) * 4 + dir) * 18;
  double2 *d = soa + ((size_t)(par * 4 + dir) * 9) * Vh + h;
#pragma unroll
  for (int k = 0; k < 9; k++) d[(size_t)k * Vh] = make_double2(s[2 * k], s[2 * k + 1]);
}
__global__ void k_links_soa_to_aos(const double2 *__restrict__ soa, double *__restrict__ aos, int Vh) {
  int h = blockIdx.x * blockDim.x + threadIdx.x;
  int par = blockIdx.y, dir = blockIdx.z;
  if (h >= Vh) return;
  double *d = aos + (((size_t)par * Vh + h) * 4 + dir) * 18;
  const double2 *s = soa + ((size_t)(par * 4 + dir) * 9) * Vh + h;
#pragma unroll
  for (int k = 0; k < 9; k++) { double2 v = s[(size_t)k * Vh]; d[2 * k] = v.x; d[2 * k + 1] = v.y; }
}
__global__ void k_links_to_f32(const double2 *__restrict__ src, float4 *__restrict__ a, float2 *__restrict__ b, int Vh) {
  int h = blockIdx.x * blockDim.x + threadIdx.x;
  int pd = blockIdx.y;  // par*4+dir
  if (h >= Vh) return;
  const double2 *s = src + ((size_t)pd * 9) * Vh + h;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    double2 u = s[(size_t)(2 * k) * Vh], v = s[(size_t)(2 * k + 1) * Vh];
    a[((size_t)pd * 4 + k) * Vh + h] = make_float4((float)u.x, (float)u.y, (float)v.x, (float)v.y);
  }
  double2 w = s[(size_t)8 * Vh];
  b[(size_t)pd * Vh + h] = make_float2((float)w.x, (float)w.y);
}
__global__ void k_links_maxabs(const double2 *__restrict__ src, size_t n, unsigned long long *out) {
  double m = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double2 v = src[i];
    m = fmax(m, fmax(fabs(v.x), fabs(v.y)));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}
__global__ void k_links_to_f16(const double2 *__restrict__ src, uint4 *__restrict__ a, __half2 *__restrict__ b,
                               const unsigned long long *maxbits, int Vh) {
  int h = blockIdx.x * blockDim.x + threadIdx.x;
  int pd = blockIdx.y;
  if (h >= Vh) return;
  double mx = __longlong_as_double((long long)*maxbits);
  float inv = mx > 0 ? (float)(1.0 / mx) : 0.f;
  const double2 *s = src + ((size_t)pd * 9) * Vh + h;
#pragma unroll
  for (int k = 0; k < 2; k++) {
    unsigned w[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      double2 u = s[(size_t)(4 * k + j) * Vh];
      __half2 hv = __floats2half2_rn((float)u.x * inv, (float)u.y * inv);
      w[j] = *reinterpret_cast<unsigned *>(&hv);
    }
    a[((size_t)pd * 2 + k) * Vh + h] = make_uint4(w[0], w[1], w[2], w[3]);
  }
  double2 u = s[(size_t)8 * Vh];
  b[(size_t)pd * Vh + h] = __floats2half2_rn((float)u.x * inv, (float)u.y * inv);
}

int vec_aos_to_soa64(const double *aos_dev, double2 *soa, int par) {
  Context &c = g_ctx;
  int Vh = (int)c.Vh;
  k_vec_aos_to_soa<<<grid_for(3 * Vh, 256), 256, 0, c.stream>>>(aos_dev, soa, par, Vh);
  c.launches++;
  MKS_CUDA(cudaGetLastError());
  return MKS_OK;
}
__global__ void k_vec_aos_to_soa32(const double *__restrict__ aos, float2 *__restrict__ soa, int par, int Vh) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= 3 * (size_t)Vh) return;
  const size_t h = t / 3;
  const int c = (int)(t - 3 * h);
  const double2 v = aos_get(aos + (size_t)par * Vh * 6, t);
  soa[(size_t)c * Vh + h] = make_float2((float)v.x, (float)v.y);
}
int vec_aos_to_soa32(const double *aos_dev, float2 *soa, int par) {
  Context &c = g_ctx;
  int Vh = (int)c.Vh;
  k_vec_aos_to_soa32<<<grid_for(3 * Vh, 256), 256, 0, c.stream>>>(aos_dev, soa, par, Vh);
  c.launches++;
  MKS_CUDA(cudaGetLastError());
  return MKS_OK;
}
int vec_soa64_to_aos(const double2 *soa, double *aos_dev, int par) {
  Context &c = g_ctx;
  int Vh = (int)c.Vh;
  k_vec_soa_to_aos<<<grid_for(3 * Vh, 256), 256, 0, c.stream>>>(soa, aos_dev, par, Vh);
  c.launches++;
  MKS_CUDA(cudaGetLastError());
  return MKS_OK;
}
int links_aos_to_soa64(const double *aos_dev, double2 *soa) {
  Context &c = g_ctx;
  int Vh = (int)c.Vh;
  k_links_aos_to_soa<<<dim3(grid_for(Vh, 128), 2, 4), 128, 0, c.stream>>>(aos_dev, soa, Vh);
  c.launches++;
  MKS_CUDA(cudaGetLastError());
  return MKS_OK;
}
int links_soa64_to_aos(const double2 *soa, double *aos_dev) {
  Context &c = g_ctx;
  int Vh = (int)c.Vh;
  k_links_soa_to_aos<<<dim3(grid_for(Vh, 128), 2, 4), 128, 0, c.stream>>>(soa, aos_dev, Vh);
  c.launches++;
  MKS_CUDA(cudaGetLastError());
  return MKS_OK;
}

static void free_slot(LinkSlot &s) {
  dev_free(s.fat64); dev_free(s.lng64);
  dev_free(s.fat32a); dev_free(s.lng32a); dev_free(s.fat32b); dev_free(s.lng32b);
  dev_free(s.fat16a); dev_free(s.lng16a); dev_free(s.fat16b); dev_free(s.lng16b);
  s = LinkSlot();
}

static int make_f16(const double2 *src, uint4 **a, __half2 **b, float *scale) {
  Context &c = g_ctx;
  int Vh = (int)c.Vh;
  size_t n = (size_t)8 * 9 * Vh;
  unsigned long long *mx;
  MKS_TRY(dev_alloc((void **)&mx, sizeof(unsigned long long)));
  MKS_CUDA(cudaMemsetAsync(mx, 0, sizeof(unsigned long long), c.stream));
  k_links_maxabs<<<c.sm_count * 4, 256, 0, c.stream>>>(src, n, mx);
  k_links_to_f16<<<dim3(grid_for(Vh, 256), 8), 256, 0, c.stream>>>(src, *a, *b, mx, Vh);
  c.launches += 2;
  unsigned long long bits = 0;
  MKS_CUDA(cudaMemcpyAsync(&bits, mx, sizeof bits, cudaMemcpyDeviceToHost, c.stream));
  MKS_CUDA(cudaStreamSynchronize(c.stream));
  dev_free(mx);
  double m;
  memcpy(&m, &bits, sizeof m);
  *scale = (float)m;
  MKS_CUDA(cudaGetLastError());
  return MKS_OK;
}

int links_make_lowprec(LinkSlot &s) {
  Context &c = g_ctx;
  int Vh = (int)c.Vh;
  size_t n32a = (size_t)8 * 4 * Vh, n32b = (size_t)8 * Vh;
  if (!s.fat32a) {
    MKS_TRY(dev_alloc((void **)&s.fat32a, n32a * sizeof(float4)));
    MKS_TRY(dev_alloc((void **)&s.lng32a, n32a * sizeof(float4)));
    MKS_TRY(dev_alloc((void **)&s.fat32b, n32b * sizeof(float2)));
    MKS_TRY(dev_alloc((void **)&s.lng32b, n32b * sizeof(float2)));
    MKS_TRY(dev_alloc((void **)&s.fat16a, (size_t)8 * 2 * Vh * sizeof(uint4)));
    MKS_TRY(dev_alloc((void **)&s.lng16a, (size_t)8 * 2 * Vh * sizeof(uint4)));
    MKS_TRY(dev_alloc((void **)&s.fat16b, n32b * sizeof(__half2)));
    MKS_TRY(dev_alloc((void **)&s.lng16b, n32b * sizeof(__half2)));
  }
  k_links_to_f32<<<dim3(grid_for(Vh, 256), 8), 256, 0, c.stream>>>(s.fat64, s.fat32a, s.fat32b, Vh);
  k_links_to_f32<<<dim3(grid_for(Vh, 256), 8), 256, 0, c.stream>>>(s.lng64, s.lng32a, s.lng32b, Vh);
  c.launches += 2;
  MKS_CUDA(cudaGetLastError());
  MKS_TRY(make_f16(s.fat64, &s.fat16a, &s.fat16b, &s.fat16scale));
  MKS_TRY(make_f16(s.lng64, &s.lng16a, &s.lng16b, &s.lng16scale));
  return MKS_OK;
}

static int load_slot_from_dev(int slot, const double *fat_dev, const double *lng_dev, double eps) {
  Context &c = g_ctx;
  LinkSlot &s = c.slots[slot];
  size_t nsoa = (size_t)8 * 9 * c.Vh;
  if (!s.fat64) {
    MKS_TRY(dev_alloc((void **)&s.fat64, nsoa * sizeof(double2)));
    MKS_TRY(dev_alloc((void **)&s.lng64, nsoa * sizeof(double2)));
  }
  MKS_TRY(links_aos_to_soa64(fat_dev, s.fat64));
  MKS_TRY(links_aos_to_soa64(lng_dev, s.lng64));
  MKS_TRY(links_make_lowprec(s));
  s.eps_naik = eps;
  s.valid = true;
  return MKS_OK;
}

}  // namespace mks

using namespace mks;

extern "C" {

const char *mks_error_string(int status) {
  switch (status) {
  case MKS_OK: return "ok";
  case MKS_ERR_ARG: return "invalid argument";
  case MKS_ERR_CUDA: return g_errmsg[0] ? g_errmsg : "CUDA error";
  case MKS_ERR_NOMEM: return g_errmsg[0] ? g_errmsg : "device allocation failed";
  case MKS_ERR_STATE: return "library not initialised, lattice not set or links not loaded";
  case MKS_ERR_TIMEOUT: return g_errmsg[0] ? g_errmsg : "bounded device wait gave up";
  case MKS_ERR_NUMERIC: return "non-finite value in a solver recurrence";
  case MKS_ERR_UNSUPPORTED: return "unsupported option";
  default: return "unknown status";
  }
}

int mks_init(int device) {
  Context &c = g_ctx;
  if (c.initialised) return MKS_OK;
  int n = 0;
  MKS_CUDA(cudaGetDeviceCount(&n));
  if (device < 0 || device >= n) return MKS_ERR_ARG;
  MKS_CUDA(cudaSetDevice(device));
  cudaDeviceProp prop;
  MKS_CUDA(cudaGetDeviceProperties(&prop, device));
  if (prop.major < 10) {
    snprintf(g_errmsg, sizeof g_errmsg, "device %d is sm_%d%d; the library is compiled for sm_103a", device,
             prop.major, prop.minor);
    return MKS_ERR_UNSUPPORTED;
  }
  c.device = device;
  c.sm_count = prop.multiProcessorCount;
  MKS_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
  c.ev_pool.resize(2 * EV_POOL);
  c.ev_family.resize(EV_POOL);
  for (auto &e : c.ev_pool) MKS_CUDA(cudaEventCreate(&e));
  // the allocation-free D_eo takes no device memory after this point: its
  // fixed array and the kernels it launches are loaded now
  cudaFuncAttributes fa;
  MKS_CUDA(cudaFuncGetAttributes(&fa, k_vec_aos_to_soa));
  MKS_CUDA(cudaFuncGetAttributes(&fa, k_vec_soa_to_aos));
  MKS_TRY(noalloc_prepare());
  c.initialised = true;
  return MKS_OK;
}

static void free_lattice_fields() {
  Context &c = g_ctx;
  for (auto &s : c.slots) free_slot(s);
  ws_free_all();
  dev_free(c.auxU); dev_free(c.auxV); dev_free(c.auxW);
  c.auxU = c.auxV = c.auxW = nullptr;
  c.aux_action = 0;
  dev_free(c.mom);
  c.mom = nullptr;
  gauge_free();
  rhmc_free();
}

int mks_finalize(void) {
  Context &c = g_ctx;
  if (!c.initialised) return MKS_OK;
  cudaStreamSynchronize(c.stream);
  free_lattice_fields();
  dev_free(c.red.partials); dev_free(c.red.count); dev_free(c.red.err);
  c.red = RedScratch();
  for (auto &e : c.ev_pool) cudaEventDestroy(e);
  c.ev_pool.clear();
  cudaStreamDestroy(c.stream);
  noalloc_forget();
  c = Context();
  return MKS_OK;
}

int mks_set_lattice(const int dims[4]) {
  MKS_TRY(check_ready(false));
  if (!dims) return MKS_ERR_ARG;
  // even extents of at least 4: the Naik term reaches 3 sites, and a hop of
  // 3 must wrap at most once
  for (int d = 0; d < 4; d++)
    if (dims[d] < 4 || (dims[d] & 1)) return MKS_ERR_ARG;
  Context &c = g_ctx;
  size_t V = (size_t)dims[0] * dims[1] * dims[2] * dims[3];
  if (V / 2 > (size_t)0x3fffffff) return MKS_ERR_ARG;  // checkerboard index is 32-bit
  bool same = V == c.V && !memcmp(dims, c.dims, sizeof c.dims);
  if (!same) {
    MKS_CUDA(cudaStreamSynchronize(c.stream));
    free_lattice_fields();
  }
  memcpy(c.dims, dims, sizeof c.dims);
  c.V = V;
  c.Vh = V / 2;
  c.geom.nx = dims[0]; c.geom.ny = dims[1]; c.geom.nz = dims[2]; c.geom.nt = dims[3];
  c.geom.Vh = (int)c.Vh;
  c.geom.sx = 1; c.geom.sy = dims[0]; c.geom.sz = dims[0] * dims[1]; c.geom.st = dims[0] * dims[1] * dims[2];
  // Reduction scratch for the largest reducing launch on this lattice, so
  // that it is never reallocated while a solver batch is being captured:
  // D_eo epilogues (up to 16 threads per site in blocks of >= 128 threads,
  // 16 sources x 3 sums) and the BLAS site kernels (up to 4 blocks per SM
  // per source row, 32 rows x 3 sums).
  MKS_TRY(ensure_red(16 * 3, (int)((c.Vh * 16 + 127) / 128)));
  MKS_TRY(ensure_red(32 * 3, c.sm_count * 4 * 32));
  return MKS_OK;
}

int mks_load_fn_links_dev(int slot, const double *fat_dev, const double *lng_dev, double eps_naik) {
  MKS_TRY(check_ready());
  if (slot < 0 || slot >= MKS_MAX_SLOTS || !fat_dev || !lng_dev) return MKS_ERR_ARG;
  MKS_TRY(load_slot_from_dev(slot, fat_dev, lng_dev, eps_naik));
  MKS_CUDA(cudaStreamSynchronize(g_ctx.stream));
  return MKS_OK;
}

int mks_load_fn_links(int slot, const double *fat, const double *lng, double eps_naik) {
  MKS_TRY(check_ready());
  if (slot < 0 || slot >= MKS_MAX_SLOTS || !fat || !lng) return MKS_ERR_ARG;
  Context &c = g_ctx;
  size_t bytes = c.V * 4 * 18 * sizeof(double);
  double *tmp;
  MKS_TRY(dev_alloc((void **)&tmp, 2 * bytes));
  MKS_CUDA(cudaMemcpyAsync(tmp, fat, bytes, cudaMemcpyHostToDevice, c.stream));
  MKS_CUDA(cudaMemcpyAsync(tmp + c.V * 72, lng, bytes, cudaMemcpyHostToDevice, c.stream));
  int rc = load_slot_from_dev(slot, tmp, tmp + c.V * 72, eps_naik);
  cudaStreamSynchronize(c.stream);
  dev_free(tmp);
  return rc;
}

int mks_invalidate_fn_links(int slot) {
  MKS_TRY(check_ready(false));
  if (slot < 0 || slot >= MKS_MAX_SLOTS) return MKS_ERR_ARG;
  g_ctx.slots[slot].valid = false;
  return MKS_OK;
}

int mks_get_fn_links(int slot, double *fat, double *lng) {
  MKS_TRY(check_ready());
  if (slot < 0 || slot >= MKS_MAX_SLOTS) return MKS_ERR_ARG;
  Context &c = g_ctx;
  LinkSlot &s = c.slots[slot];
  if (!s.valid) return MKS_ERR_STATE;
  size_t bytes = c.V * 4 * 18 * sizeof(double);
  double *tmp;
  MKS_TRY(dev_alloc((void **)&tmp, bytes));
  int rc = MKS_OK;
  if (fat) {
    MKS_TRY(links_soa64_to_aos(s.fat64, tmp));
    MKS_CUDA(cudaMemcpyAsync(fat, tmp, bytes, cudaMemcpyDeviceToHost, c.stream));
    MKS_CUDA(cudaStreamSynchronize(c.stream));
  }
  if (lng) {
    MKS_TRY(links_soa64_to_aos(s.lng64, tmp));
    MKS_CUDA(cudaMemcpyAsync(lng, tmp, bytes, cudaMemcpyDeviceToHost, c.stream));
    MKS_CUDA(cudaStreamSynchronize(c.stream));
  }
  dev_free(tmp);
  return rc;
}

int mks_timing_enable(int on) {
  MKS_TRY(check_ready(false));
  if (!on) MKS_TRY(timing_flush());
  g_ctx.timing = on != 0;
  return MKS_OK;
}

int mks_timing_reset(void) {
  MKS_TRY(check_ready(false));
  MKS_TRY(timing_flush());
  Context &c = g_ctx;
  for (int k = 0; k < MKS_K_COUNT; k++) { c.kernel_ms[k] = 0; c.kernel_launches[k] = 0; }
  c.launches = 0;
  return MKS_OK;
}

int mks_timing_get(int family, double *total_ms, long long *launches) {
  MKS_TRY(check_ready(false));
  if (family < 0 || family >= MKS_K_COUNT) return MKS_ERR_ARG;
  MKS_TRY(timing_flush());
  if (total_ms) *total_ms = g_ctx.kernel_ms[family];
  if (launches) *launches = g_ctx.kernel_launches[family];
  return MKS_OK;
}

long long mks_launch_count(void) { return g_ctx.launches; }

void *mks_stream(void) { return (void *)g_ctx.stream; }

}  // extern "C"
