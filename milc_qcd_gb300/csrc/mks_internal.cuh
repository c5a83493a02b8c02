// mks_internal.cuh -- device data types, field layouts and the library
// context shared by the CUDA translation units.
//
// HBM layout (one GPU, whole lattice resident):
//   * a colour-vector field of one parity is structure-of-arrays, one
//     array per colour component, indexed by the checkerboard index h
//     (MILC index = parity*Vh + h, even parity first):
//       FP64  double2 [3][Vh]            (16-byte loads)
//       FP32  float2  [3][Vh]
//       FP16  __half2 [3][Vh] + float norm[Vh]  (per-site max-abs scale)
//   * a link field of one parity and direction (9 complex entries):
//       FP64  double2 [9][Vh]
//       FP32  float4  [4][Vh] (entries 0..7) + float2 [Vh] (entry 8)
//       FP16  uint4   [2][Vh] (entries 0..7 as 16 halves) + __half2 [Vh],
//             scaled by one global factor per link type
//     stored [parity][dir][...], so D_eo streams forward links at h and
//     backward links of the other parity at the neighbour index: every link
//     is read exactly once per application, without back-link copies.
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>
#include <stdio.h>
#include <vector>
#include "milc_ks_gb300.h"

#define MKS_CUDA(call)                                                        \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess) {                                                  \
      mks::set_last_error(e_, #call, __FILE__, __LINE__);                     \
      return MKS_ERR_CUDA;                                                    \
    }                                                                         \
  } while (0)

#define MKS_TRY(call)                                                         \
  do {                                                                        \
    int s_ = (call);                                                          \
    if (s_ < 0) return s_;                                                    \
  } while (0)

namespace mks {

void set_last_error(cudaError_t e, const char *what, const char *file, int line);

// ------------------------------------------------------------------
// complex / SU(3) arithmetic
template <typename R> struct cplx { R re, im; };
template <typename R> struct V3 { cplx<R> c[3]; };
template <typename R> struct M3 { cplx<R> e[3][3]; };

template <typename R> __device__ __forceinline__ cplx<R> cmul(cplx<R> a, cplx<R> b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}

// o += m v
template <typename R> __device__ __forceinline__ void mv_acc(const M3<R> &m, const V3<R> &v, V3<R> &o) {
#pragma unroll
  for (int i = 0; i < 3; i++) {
    R re = o.c[i].re, im = o.c[i].im;
#pragma unroll
    for (int j = 0; j < 3; j++) {
      re = fma(m.e[i][j].re, v.c[j].re, re);
      re = fma(-m.e[i][j].im, v.c[j].im, re);
      im = fma(m.e[i][j].re, v.c[j].im, im);
      im = fma(m.e[i][j].im, v.c[j].re, im);
    }
    o.c[i].re = re; o.c[i].im = im;
  }
}
// o -= m^dag v
template <typename R> __device__ __forceinline__ void amv_sub(const M3<R> &m, const V3<R> &v, V3<R> &o) {
#pragma unroll
  for (int i = 0; i < 3; i++) {
    R re = o.c[i].re, im = o.c[i].im;
#pragma unroll
    for (int j = 0; j < 3; j++) {
      // conj(m[j][i]) * v[j]
      re = fma(-m.e[j][i].re, v.c[j].re, re);
      re = fma(-m.e[j][i].im, v.c[j].im, re);
      im = fma(-m.e[j][i].re, v.c[j].im, im);
      im = fma(m.e[j][i].im, v.c[j].re, im);
    }
    o.c[i].re = re; o.c[i].im = im;
  }
}

// ------------------------------------------------------------------
// lattice geometry on the device
struct Geom {
  int nx, ny, nz, nt;
  int Vh;
  int sx, sy, sz, st;   // lexicographic strides 1, nx, nx*ny, nx*ny*nz
};

// coordinates of checkerboard site h of parity par (0 even, 1 odd)
__device__ __forceinline__ void site_coords(const Geom &g, int par, int h, int &x, int &y, int &z, int &t) {
  int q = 2 * h;
  int xe = q % g.nx;
  int r = q / g.nx;
  y = r % g.ny;
  r /= g.ny;
  z = r % g.nz;
  t = r / g.nz;
  x = xe + ((xe + y + z + t + par) & 1);
}

// checkerboard index of (x,y,z,t) (parity implied)
__device__ __forceinline__ int cb_index(const Geom &g, int x, int y, int z, int t) {
  return (x + g.nx * (y + g.ny * (z + g.nz * t))) >> 1;
}

// lexicographic offset of a hop of k (|k| <= 3) along mu, with wrap
__device__ __forceinline__ int wrap_add(int c, int k, int n) {
  int r = c + k;
  r += (r < 0) ? n : 0;
  r -= (r >= n) ? n : 0;
  return r;
}

// ------------------------------------------------------------------
// field accessors

// ask L2 for the 128-byte line holding address a (a hint: no register is
// held and nothing is returned)
__device__ __forceinline__ void prefetch_l2(const void *a) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(a));
}

struct VecF64 {
  double2 *p;  // [3][Vh]
  // lines of the 16 sites h..h+15 (h a multiple of 16)
  __device__ __forceinline__ void prefetch16(int h, int Vh) const {
#pragma unroll
    for (int c = 0; c < 3; c++) {
      prefetch_l2(p + (size_t)c * Vh + h);
      if (h + 8 < Vh) prefetch_l2(p + (size_t)c * Vh + h + 8);
    }
  }
  __device__ __forceinline__ V3<double> load(int h, int Vh) const {
    V3<double> v;
#pragma unroll
    for (int c = 0; c < 3; c++) { double2 a = __ldg(p + (size_t)c * Vh + h); v.c[c] = {a.x, a.y}; }
    return v;
  }
  __device__ __forceinline__ void store(int h, int Vh, const V3<double> &v) const {
#pragma unroll
    for (int c = 0; c < 3; c++) p[(size_t)c * Vh + h] = make_double2(v.c[c].re, v.c[c].im);
  }
  __device__ __forceinline__ void store_stream(int h, int Vh, const V3<double> &v) const {
#pragma unroll
    for (int c = 0; c < 3; c++) __stcs(p + (size_t)c * Vh + h, make_double2(v.c[c].re, v.c[c].im));
  }
};
struct VecF32 {
  float2 *p;  // [3][Vh]
  // lines of the 16 sites h..h+15 (h a multiple of 16)
  __device__ __forceinline__ void prefetch16(int h, int Vh) const {
#pragma unroll
    for (int c = 0; c < 3; c++) prefetch_l2(p + (size_t)c * Vh + h);
  }
  __device__ __forceinline__ V3<float> load(int h, int Vh) const {
    V3<float> v;
#pragma unroll
    for (int c = 0; c < 3; c++) { float2 a = __ldg(p + (size_t)c * Vh + h); v.c[c] = {a.x, a.y}; }
    return v;
  }
  __device__ __forceinline__ void store(int h, int Vh, const V3<float> &v) const {
#pragma unroll
    for (int c = 0; c < 3; c++) p[(size_t)c * Vh + h] = make_float2(v.c[c].re, v.c[c].im);
  }
  // the same as a streaming (evict-first) store, for results that the next
  // kernel reads once
  __device__ __forceinline__ void store_stream(int h, int Vh, const V3<float> &v) const {
#pragma unroll
    for (int c = 0; c < 3; c++) __stcs(p + (size_t)c * Vh + h, make_float2(v.c[c].re, v.c[c].im));
  }
  __device__ __forceinline__ V3<float> load_mul(int h, int Vh, float f) const {
    V3<float> v = load(h, Vh);
#pragma unroll
    for (int c = 0; c < 3; c++) { v.c[c].re *= f; v.c[c].im *= f; }
    return v;
  }
};
struct VecF16 {
  __half2 *p;   // [3][Vh]
  float *norm;  // [Vh]
  __device__ __forceinline__ V3<float> load(int h, int Vh) const {
    V3<float> v;
    float s = __ldg(norm + h);
#pragma unroll
    for (int c = 0; c < 3; c++) {
      float2 a = __half22float2(__ldg(p + (size_t)c * Vh + h));
      v.c[c] = {a.x * s, a.y * s};
    }
    return v;
  }
  __device__ __forceinline__ V3<float> load_mul(int h, int Vh, float f) const {
    V3<float> v;
    float s = __ldg(norm + h) * f;
#pragma unroll
    for (int c = 0; c < 3; c++) {
      float2 a = __half22float2(__ldg(p + (size_t)c * Vh + h));
      v.c[c] = {a.x * s, a.y * s};
    }
    return v;
  }
  __device__ __forceinline__ void store(int h, int Vh, const V3<float> &v) const {
    float m = 0.f;
#pragma unroll
    for (int c = 0; c < 3; c++) m = fmaxf(m, fmaxf(fabsf(v.c[c].re), fabsf(v.c[c].im)));
    float inv = m > 0.f ? 1.0f / m : 0.f;
    norm[h] = m;
#pragma unroll
    for (int c = 0; c < 3; c++) p[(size_t)c * Vh + h] = __floats2half2_rn(v.c[c].re * inv, v.c[c].im * inv);
  }
  __device__ __forceinline__ void store_stream(int h, int Vh, const V3<float> &v) const { store(h, Vh, v); }
};

// Link loads of D_eo: every link is read once per application, so they are
// loaded as streaming data (evict-first in L1 and L2) and leave the L2 to the
// colour vectors, which 16 sites read each (the t-neighbours up to six
// time slices apart)
#ifndef MKS_LINK_LD
#define MKS_LINK_LD __ldcs
#endif
struct LinkF64 {
  static constexpr bool scaled = false;
  const double2 *p;  // [par][dir][9][Vh]
  __device__ __forceinline__ M3<double> load(int par, int dir, int h, int Vh) const {
    const double2 *b = p + ((size_t)(par * 4 + dir) * 9) * Vh + h;
    M3<double> m;
#pragma unroll
    for (int k = 0; k < 9; k++) { double2 a = MKS_LINK_LD(b + (size_t)k * Vh); m.e[k / 3][k % 3] = {a.x, a.y}; }
    return m;
  }
};
struct LinkF32 {
  static constexpr bool scaled = false;
  const float4 *a;  // [par][dir][4][Vh]
  const float2 *b;  // [par][dir][Vh]
  __device__ __forceinline__ M3<float> load(int par, int dir, int h, int Vh) const {
    const float4 *pa = a + ((size_t)(par * 4 + dir) * 4) * Vh + h;
    float2 l = MKS_LINK_LD(b + (size_t)(par * 4 + dir) * Vh + h);
    M3<float> m;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      float4 q = MKS_LINK_LD(pa + (size_t)k * Vh);
      m.e[(2 * k) / 3][(2 * k) % 3] = {q.x, q.y};
      m.e[(2 * k + 1) / 3][(2 * k + 1) % 3] = {q.z, q.w};
    }
    m.e[2][2] = {l.x, l.y};
    return m;
  }
};
struct LinkF16 {
  static constexpr bool scaled = true;  // entries are stored divided by `scale`
  const uint4 *a;     // [par][dir][2][Vh]: entries 0..7 as 16 halves
  const __half2 *b;   // [par][dir][Vh]: entry 8
  float scale;
  // unscaled entries: U = scale * load_raw(); D_eo folds `scale` into the vector
  __device__ __forceinline__ M3<float> load_raw(int par, int dir, int h, int Vh) const {
    const uint4 *pa = a + ((size_t)(par * 4 + dir) * 2) * Vh + h;
    M3<float> m;
#pragma unroll
    for (int k = 0; k < 2; k++) {
      uint4 q = MKS_LINK_LD(pa + (size_t)k * Vh);
      unsigned w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
      for (int j = 0; j < 4; j++) {
        __half2 hv = *reinterpret_cast<__half2 *>(&w[j]);
        float2 f = __half22float2(hv);
        int e = 4 * k + j;
        m.e[e / 3][e % 3] = {f.x, f.y};
      }
    }
    float2 f = __half22float2(MKS_LINK_LD(b + (size_t)(par * 4 + dir) * Vh + h));
    m.e[2][2] = {f.x, f.y};
    return m;
  }
  __device__ __forceinline__ M3<float> load(int par, int dir, int h, int Vh) const {
    const uint4 *pa = a + ((size_t)(par * 4 + dir) * 2) * Vh + h;
    M3<float> m;
#pragma unroll
    for (int k = 0; k < 2; k++) {
      uint4 q = MKS_LINK_LD(pa + (size_t)k * Vh);
      unsigned w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
      for (int j = 0; j < 4; j++) {
        __half2 hv = *reinterpret_cast<__half2 *>(&w[j]);
        float2 f = __half22float2(hv);
        int e = 4 * k + j;
        m.e[e / 3][e % 3] = {f.x * scale, f.y * scale};
      }
    }
    float2 f = __half22float2(MKS_LINK_LD(b + (size_t)(par * 4 + dir) * Vh + h));
    m.e[2][2] = {f.x * scale, f.y * scale};
    return m;
  }
};

// ------------------------------------------------------------------
// device-side reduction scratch for grid_reduce_last: per-block and
// per-group rows of partial sums, and the arrival counters (top + one per
// group of blocks), which return to 0 at the end of every launch
constexpr int RED_GROUP = 64;  // blocks per first-level group
struct RedScratch {
  double *partials;     // capacity: max_partials doubles
  unsigned int *count;  // capacity: max_count counters
  size_t max_partials;
  size_t max_count;
  int *err;             // set on the device when a launch would overrun the scratch
};
// reads and clears the device error flag: MKS_ERR_CUDA if a reduction
// overran its scratch, MKS_ERR_TIMEOUT (after tma_disable) if a TMA-staged
// D_eo tile gave up waiting for its links
int red_check();
// switch the TMA-staged D_eo off for the rest of the process (mks_solvers.cu)
void tma_disable();

// gauge side of the molecular dynamics (mks_gauge.cu), on the resident
// thin links and momenta
void gauge_free();
void rhmc_free();
int gauge_force_dev(double eps, double beta, double u0, int nflavors, int prec);
int gauge_action_dev(double beta, double u0, int nflavors, double *action);
int mom_action_dev(double *h);
int plaquette_dev(double *ss, double *st);
int update_u_dev(double eps);
int reunitarize_dev();
int ranmom_dev();
int gauss_vec_dev(int parity, double *v_dev);
int norm2_aos_dev(const double *v_dev, int par, double *out);
int lincomb_aos_dev(int par, const double *src, const double *const *x, const double *a, int n, double *out);
int prn_seed_dev(int seed);
// fat/long links of slots 0..n_naiks-1 from the resident thin links (mks_links.cu)
int links_from_aux(int action, int n_naiks, const double *eps_naik, double u0);
// fermion force on device SoA solution fields (mks_force.cu)
int force_dev(double eps, const double *residues, double2 *const *xs, int nterms, const int *orders, int n_naiks,
              double *mom_dev, double2 *ku_out);
// the same in the FP32 molecular-dynamics setting with the solutions already
// FP32 SoA, full lattice [2][3][Vh] per term
int force_dev32(double eps, const double *residues, float2 *const *xs32, int nterms, const int *orders,
                int n_naiks, double *mom_dev);
// FP32 multi-source D on one parity: out_s (parity out_par) = D in_s (other
// parity), SoA [3][Vh] fields, slot's FP32 links, any number of sources
int dslash32_multi(int slot, int out_par, int nsrc, float2 *const *in, float2 *const *out);

// ------------------------------------------------------------------
// host-side context
struct LinkSlot {
  bool valid = false;
  double eps_naik = 0.0;
  double2 *fat64 = nullptr, *lng64 = nullptr;            // [2][4][9][Vh]
  float4 *fat32a = nullptr, *lng32a = nullptr;           // [2][4][4][Vh]
  float2 *fat32b = nullptr, *lng32b = nullptr;           // [2][4][Vh]
  uint4 *fat16a = nullptr, *lng16a = nullptr;            // [2][4][2][Vh]
  __half2 *fat16b = nullptr, *lng16b = nullptr;          // [2][4][Vh]
  float fat16scale = 1.f, lng16scale = 1.f;
};

struct Context {
  bool initialised = false;
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  int dims[4] = {0, 0, 0, 0};
  size_t V = 0, Vh = 0;
  Geom geom{};
  LinkSlot slots[MKS_MAX_SLOTS];
  RedScratch red{};
  // thin links (auxU, phases in) and the HISQ smearing stages V, W (FP64,
  // device, [2][4][9][Vh] SoA like fat64), with the action and tadpole
  // factor the fat/long links of slot 0 were built with (0: unknown)
  double2 *auxU = nullptr, *auxV = nullptr, *auxW = nullptr;
  int aux_action = 0;
  double aux_u0 = 1.0;
  // gauge momenta of the molecular dynamics (anti_hermitmat[V][4], device)
  double *mom = nullptr;
  // arithmetic of the staple products in link construction and the fermion
  // force (MKS_PREC_DOUBLE, or MKS_PREC_SINGLE inside a molecular-dynamics
  // integration), and the one the current fermion links were built with
  int md_prec = MKS_PREC_DOUBLE;
  int links_prec = MKS_PREC_DOUBLE;
  // timing
  bool timing = false;
  double kernel_ms[MKS_K_COUNT] = {0};
  long long kernel_launches[MKS_K_COUNT] = {0};
  long long launches = 0;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<int> ev_family;  // family per pair
  int ev_used = 0;
  // CUDA-graph capture of solver iterations: while `capture` is set,
  // launches are recorded into it instead of the event pool
  struct Capture *capture = nullptr;
};

Context &ctx();
int check_ready(bool need_lattice = true);

// A captured batch of launches: per kernel node its family and (when the
// batch was captured with timing on) its own event pair, so each replay of
// the graph can be timed and counted like eager launches.
struct Capture {
  std::vector<int> family;
  std::vector<cudaEvent_t> ev;  // 2 per node when timed
  bool timed = false;
};
void capture_account(const Capture &cap);  // after a replay has completed

// timed launch helpers
void timing_begin(int family);
void timing_end(int family);
int timing_flush();

// memory helpers (stream-ordered)
int dev_alloc(void **p, size_t bytes);
void dev_free(void *p);

// named workspace buffers of the solvers (mks_solvers.cu)
void ws_free_all();

// reduction scratch sized for `nsum` sums and `blocks` blocks
int ensure_red(int nsum, int blocks);

inline int grid_for(size_t n, int block) { return (int)((n + block - 1) / block); }

// allocation-free D_eo (mks_noalloc.cu): resolve its fixed device array and
// load its kernel at mks_init; forget the address at mks_finalize
int noalloc_prepare();
void noalloc_forget();

// layout conversion (mks_context.cu)
int vec_aos_to_soa64(const double *aos_dev, double2 *soa, int par);   // one parity from a full AoS field
int vec_soa64_to_aos(const double2 *soa, double *aos_dev, int par);
int vec_aos_to_soa32(const double *aos_dev, float2 *soa, int par);    // one parity, rounded to FP32
int links_aos_to_soa64(const double *aos_dev, double2 *soa);          // [V][4][18] -> [2][4][9][Vh]
int links_soa64_to_aos(const double2 *soa, double *aos_dev);
int links_make_lowprec(LinkSlot &s);

// D_eo entry points (mks_dslash.cu).  All take device SoA fields.
// out_par: parity of the output sites; input read on the other parity.
int dslash_f64(int slot, const double2 *in, double2 *out, int out_par);
int dslash_f32(int slot, const float2 *in, float2 *out, int out_par);
int dslash_f16(int slot, const __half2 *in, const float *in_norm, float2 *out, int out_par);

}  // namespace mks
