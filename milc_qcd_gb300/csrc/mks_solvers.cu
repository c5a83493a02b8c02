// mks_solvers.cu -- D_eo launchers and the Krylov solvers behind the C ABI:
//   mks_dslash_fn_field*          (generic_ks/dslash_fn.c:302-358)
//   mks_ks_congrad_parity*        (generic_ks/d_congrad5_fn_milc.c:61-407,
//                                  generic_ks/d_congrad5_fn_gpu.c:35-165)
//   mks_ks_congrad_block_parity*  (generic_ks/d_congrad5_fn_gpu.c:167-305)
//   mks_mat_invert_uml_field / mks_mat_invert_block_uml (generic_ks/mat_invert.c:328-483)
//   mks_ks_multicg_offset_field*  (generic_ks/ks_multicg_offset.c:63-505,
//                                  generic_ks/ks_multicg.c:170-228)
//
// Every iteration is device resident: the two D applications carry the
// CG axpy and dot products in their epilogue, the solver scalars are
// updated by the last block of each reduction, and kernels return at once
// while a device flag asks for host attention (restart, reliable update,
// convergence).  The host only polls that flag every few iterations.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <cstdlib>
#include <map>
#include <string>
#include <type_traits>
#include <vector>
#include "mks_internal.cuh"
#include "mks_dslash.cuh"
#include "mks_blas.cuh"

namespace mks {

// ------------------------------------------------------------------
// workspace: named device buffers kept across calls
struct WsBuf { void *p = nullptr; size_t bytes = 0; };
static std::map<std::string, WsBuf> g_ws;

static int ws(const std::string &name, size_t bytes, void **out) {
  WsBuf &b = g_ws[name];
  if (b.bytes < bytes) {
    dev_free(b.p);
    b.p = nullptr;
    b.bytes = 0;
    MKS_TRY(dev_alloc(&b.p, bytes));
    b.bytes = bytes;
  }
  *out = b.p;
  return MKS_OK;
}

void graphs_free_all();
static void shapes_reset();

// on a lattice change: graphs, workspace and the tuned launch shapes go
void ws_free_all() {
  graphs_free_all();
  shapes_reset();
  for (auto &kv : g_ws) dev_free(kv.second.p);
  g_ws.clear();
}

template <typename T> static int wsv(const std::string &name, size_t n, T **out) {
  void *p;
  MKS_TRY(ws(name, n * sizeof(T), &p));
  *out = (T *)p;
  return MKS_OK;
}

// ------------------------------------------------------------------
// solver scalars, one per source
enum { ST_RUN = 0, ST_HOST = 1, ST_DONE = 4 };

struct CgState {
  double rsq;          // MILC 'rsq' (FEWSUMS estimate between true residuals)
  double actual_rsq;   // true |r|^2 of the iterated residual
  double a, b;
  double source_norm;
  double rsqmin, relrsqmin;
  double size_r, size_relr;
  double final_rsq, final_relrsq;
  double maxrr, delta;
  int iter, niter, max_cg, status;
  int nrestart, max_restarts, mixed, converged;
  int reliable;
};

struct Solver {
  CgState *st = nullptr;   // device [nsrc]
  int *skip = nullptr;     // device: non-zero while any source needs the host
};

// ---------- finishers ----------
// after the second D of an iteration: pkp, c_tr, c_tt -> a, rsq, b
// (generic_ks/d_congrad5_fn_milc.c:278-357 with FEWSUMS)
struct FinCgAlpha {
  CgState *st;
  __device__ void operator()(const double *t, int nsrc) const {
    int s = threadIdx.x;
    if (s >= nsrc) return;
    CgState &c = st[s];
    if (c.status != ST_RUN) { c.a = 0; c.b = 0; return; }
    double pkp = t[3 * s], c_tr = t[3 * s + 1], c_tt = t[3 * s + 2];
    double oldrsq = c.actual_rsq;
    double a = -c.rsq / pkp;
    c.iter++;
    c.a = a;
    c.rsq = oldrsq + 2.0 * a * c_tr + a * a * c_tt;
    c.b = c.rsq / oldrsq;
    if (!isfinite(c.rsq) || !isfinite(a)) c.status = ST_HOST;
  }
};

// after the update: true |r|^2 -> stop / restart / reliable-update checks.
// FP64 CG: restart when iter % niter == 0 or the iterated residual meets
// the target (d_congrad5_fn_milc.c:173-181).  Mixed precision: ask for a
// reliable update when |r| fell below delta * max|r| since the last one,
// or the iterated residual meets the target, or the iteration cap is hit.
struct FinCgUpdate {
  CgState *st;
  int *skip;
  __device__ void operator()(const double *t, int nsrc) const {
    int s = threadIdx.x;
    if (s < nsrc) {
      CgState &c = st[s];
      if (c.status == ST_RUN) {
        c.actual_rsq = t[s];
        c.size_r = c.rsq / c.source_norm;
        if (c.mixed) {
          double rn = sqrt(c.actual_rsq);
          if (rn > c.maxrr) c.maxrr = rn;
          if (rn < c.delta * c.maxrr || c.actual_rsq < c.rsqmin * c.source_norm || c.iter >= c.max_cg ||
              !isfinite(c.actual_rsq))
            c.status = ST_HOST;
        } else {
          if ((c.iter % c.niter == 0) || (c.rsqmin <= 0 || c.rsqmin > c.size_r) || !isfinite(c.actual_rsq))
            c.status = ST_HOST;
        }
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int any = 0;
      for (int i = 0; i < nsrc; i++) any |= (st[i].status == ST_HOST);
      *skip = any;
    }
  }
};

// source norm, and generic "store totals" finisher
struct FinNone {
  __device__ void operator()(const double *, int) const {}
};

// ---------- BLAS site operations ----------
template <typename T> struct VT;
template <> struct VT<double> { typedef double2 v2; };
template <> struct VT<float> { typedef float2 v2; };

struct PtrSet64 { double2 *p[BLAS_MAXSRC]; };
struct PtrSet32 { float2 *p[BLAS_MAXSRC]; };
struct PtrSet16 { __half2 *p[BLAS_MAXSRC]; float *n[BLAS_MAXSRC]; };

// |v|^2
template <typename T2> struct OpNorm {
  T2 *v[2 * BLAS_MAXSRC];
  int Vh;
  __device__ void operator()(int h, int s, double *out) const {
    double a = 0;
#pragma unroll
    for (int c = 0; c < 3; c++) {
      T2 q = v[s][(size_t)c * Vh + h];
      a += (double)q.x * q.x + (double)q.y * q.y;
    }
    out[0] = a;
  }
};

// CG restart / reliable update residual (FP64):
//   ttt <- ttt - 4m^2 x ; r <- src + ttt ; sum |r|^2, and the relative residual
//   sum |r|^2/|x|^2 (d_congrad5_fn_milc.c:196-216).  Optionally p <- r.
// Entry s of the op works on source map[s]; when tzero[s] is set the
// source's x is known to be zero and D D x is not computed (ttt taken as 0).
struct OpResid64 {
  double2 *ttt[BLAS_MAXSRC], *x[BLAS_MAXSRC], *src[BLAS_MAXSRC], *r[BLAS_MAXSRC], *p[BLAS_MAXSRC];
  const CgState *st;
  double msq4[BLAS_MAXSRC];
  int map[BLAS_MAXSRC], tzero[BLAS_MAXSRC];
  int Vh, setp;
  __device__ void operator()(int h, int s, double *out) const {
    if (st && st[map[s]].status != ST_HOST) { out[0] = 0; out[1] = 0; return; }
    double a = 0, xx = 0;
#pragma unroll
    for (int c = 0; c < 3; c++) {
      size_t i = (size_t)c * Vh + h;
      double2 t = tzero[s] ? make_double2(0.0, 0.0) : ttt[s][i], xv = x[s][i], sv = src[s][i];
      double2 rv = make_double2(sv.x + (t.x + (-msq4[s]) * xv.x), sv.y + (t.y + (-msq4[s]) * xv.y));
      r[s][i] = rv;
      if (setp) p[s][i] = rv;
      a += rv.x * rv.x + rv.y * rv.y;
      xx += xv.x * xv.x + xv.y * xv.y;
    }
    out[0] = a;
    out[1] = (xx == 0) ? 1.0 : a / xx;
  }
};

struct FinResid {
  CgState *st;
  int *skip;
  int map[BLAS_MAXSRC];
  __device__ void operator()(const double *t, int nsrc) const {
    int s = threadIdx.x;
    if (s < nsrc) {
      CgState &c = st[map[s]];
      if (c.status == ST_HOST) {
        c.rsq = t[2 * s];
        c.actual_rsq = t[2 * s];
        c.final_rsq = c.rsq / c.source_norm;
        c.maxrr = sqrt(c.rsq);
        c.iter++;
      }
    }
  }
};

// CG update, FP64 or FP32 storage: x += a p; r += a ttt; sum |r|^2 (+ rel);
// p = r + b p (d_congrad5_fn_milc.c:315-368).  Optional FP16 shadow of p.
template <typename R> struct OpUpdate {
  typedef typename VT<R>::v2 T2;
  T2 *x[BLAS_MAXSRC], *p[BLAS_MAXSRC], *r[BLAS_MAXSRC], *ttt[BLAS_MAXSRC];
  __half2 *p16[BLAS_MAXSRC];
  float *p16n[BLAS_MAXSRC];
  const CgState *st;
  int Vh, relres;
  // split epilogue: ttt holds D D p only and the update forms
  // ttt - msq4 p itself (the same fma as the fused D_eo epilogue)
  int fold;
  double msq4[BLAS_MAXSRC];
  __device__ void operator()(int h, int s, double *out) const {
    const CgState &c = st[s];
    if (c.status != ST_RUN) { out[0] = 0; if (relres) out[1] = 0; return; }
    const R a = (R)c.a, b = (R)c.b, cf = -(R)msq4[s];
    R rr = 0, xx = 0;  // per-site sums in the storage precision (FP64 is slow on GB300)
    V3<R> pn;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      size_t i = (size_t)k * Vh + h;
      T2 xv = x[s][i], pv = p[s][i], rv = r[s][i], tv = ttt[s][i];
      if (fold) { tv.x = fma(cf, pv.x, tv.x); tv.y = fma(cf, pv.y, tv.y); }
      xv.x = xv.x + a * pv.x; xv.y = xv.y + a * pv.y;
      rv.x = rv.x + a * tv.x; rv.y = rv.y + a * tv.y;
      rr += rv.x * rv.x + rv.y * rv.y;
      xx += xv.x * xv.x + xv.y * xv.y;
      pv.x = rv.x + b * pv.x; pv.y = rv.y + b * pv.y;
      x[s][i] = xv; r[s][i] = rv; p[s][i] = pv;
      pn.c[k] = {(R)pv.x, (R)pv.y};
    }
    if (p16[s]) {
      float m = 0.f;
#pragma unroll
      for (int k = 0; k < 3; k++) m = fmaxf(m, fmaxf(fabsf((float)pn.c[k].re), fabsf((float)pn.c[k].im)));
      float inv = m > 0.f ? 1.f / m : 0.f;
      p16n[s][h] = m;
#pragma unroll
      for (int k = 0; k < 3; k++)
        p16[s][(size_t)k * Vh + h] = __floats2half2_rn((float)pn.c[k].re * inv, (float)pn.c[k].im * inv);
    }
    out[0] = rr;
    if (relres) out[1] = (xx == 0) ? 1.0 : rr / xx;
  }
};

// split epilogue of the CG iteration: with ttt = D D p - msq4 p formed on
// the fly from the plain D's output, the FEWSUMS set <p,ttt>, <ttt,r>,
// <ttt,ttt> (what the fused D_eo epilogue computes), FP32 per site
template <typename R> struct OpDots3 {
  typedef typename VT<R>::v2 T2;
  const T2 *p[BLAS_MAXSRC], *r[BLAS_MAXSRC], *ttt[BLAS_MAXSRC];
  double msq4[BLAS_MAXSRC];
  int Vh;
  __device__ void operator()(int h, int s, double *out) const {
    const R cf = -(R)msq4[s];
    R d0 = 0, d1 = 0, d2 = 0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      size_t i = (size_t)k * Vh + h;
      const T2 pv = p[s][i], rv = r[s][i];
      T2 tv = ttt[s][i];
      tv.x = fma(cf, pv.x, tv.x);
      tv.y = fma(cf, pv.y, tv.y);
      d0 += pv.x * tv.x + pv.y * tv.y;
      d1 += tv.x * rv.x + tv.y * rv.y;
      d2 += tv.x * tv.x + tv.y * tv.y;
    }
    out[0] = d0; out[1] = d1; out[2] = d2;
  }
};

// x64 += x32 ; x32 = 0 (reliable update), for flagged sources
struct OpAccumX {
  double2 *x64[BLAS_MAXSRC];
  float2 *x32[BLAS_MAXSRC];
  const CgState *st;
  int Vh;
  __device__ void operator()(int h, int s, double *) const {
    if (st[s].status != ST_HOST) return;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      size_t i = (size_t)k * Vh + h;
      double2 a = x64[s][i];
      float2 b = x32[s][i];
      x64[s][i] = make_double2(a.x + (double)b.x, a.y + (double)b.y);
      x32[s][i] = make_float2(0.f, 0.f);
    }
  }
};

// r32 = r64, and (when setp) p32 = r32, p16 = r32, for flagged sources
struct OpDemote {
  double2 *r64[BLAS_MAXSRC];
  float2 *r32[BLAS_MAXSRC], *p32[BLAS_MAXSRC];
  __half2 *p16[BLAS_MAXSRC];
  float *p16n[BLAS_MAXSRC];
  const CgState *st;
  int Vh, setp;
  __device__ void operator()(int h, int s, double *) const {
    if (st[s].status != ST_HOST) return;
    float2 v[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      size_t i = (size_t)k * Vh + h;
      double2 a = r64[s][i];
      v[k] = make_float2((float)a.x, (float)a.y);
      r32[s][i] = v[k];
      if (setp) p32[s][i] = v[k];
    }
    if (setp && p16[s]) {
      float m = 0.f;
#pragma unroll
      for (int k = 0; k < 3; k++) m = fmaxf(m, fmaxf(fabsf(v[k].x), fabsf(v[k].y)));
      float inv = m > 0.f ? 1.f / m : 0.f;
      p16n[s][h] = m;
#pragma unroll
      for (int k = 0; k < 3; k++) p16[s][(size_t)k * Vh + h] = __floats2half2_rn(v[k].x * inv, v[k].y * inv);
    }
  }
};

// zero a vector (one parity)
template <typename T2> struct OpZero {
  T2 *v[BLAS_MAXSRC];
  int Vh;
  __device__ void operator()(int h, int s, double *) const {
#pragma unroll
    for (int k = 0; k < 3; k++) { T2 z; z.x = 0; z.y = 0; v[s][(size_t)k * Vh + h] = z; }
  }
};

template <class Op, int NSUM, class Fin>
static int launch_site(int family, const Op &op, const Fin &fin, const int *skip, int nsrc, double *totals = nullptr) {
  Context &c = ctx();
  int Vh = (int)c.Vh;
  int gx = grid_for(Vh, 256);
  // Blocks per SM and source row: about 16 per SM over all rows, 1 to 4 per
  // row.  Every block ends with a block reduction and a row of partial sums,
  // so for many sources fewer, longer blocks win (8 sources on 32^3x64: the
  // CG's update and dot kernels 111 ms per solve of 8 with 2 per row, 117
  // with 4, 129 with 8), while the one-row multi-shift update needs the 4
  // (100 ms against 116 with 2).  MKS_SITE_BLOCKS fixes the count per row.
  static int forced = -1;
  if (forced < 0) {
    const char *e = getenv("MKS_SITE_BLOCKS");
    forced = e && atoi(e) > 0 ? atoi(e) : 0;
  }
  int per_sm = forced ? forced : 16 / (nsrc > 0 ? nsrc : 1);
  if (!forced) per_sm = per_sm < 1 ? 1 : per_sm > 4 ? 4 : per_sm;
  int cap = c.sm_count * per_sm;
  if (gx > cap) gx = cap;
  MKS_TRY(ensure_red(NSUM > 0 ? NSUM * nsrc : 1, gx * nsrc));  // one row per block of the (gx, nsrc) grid
  timing_begin(family);
  k_site<Op, NSUM, Fin><<<dim3(gx, nsrc), 256, 0, c.stream>>>(op, fin, skip, Vh, c.red,
                                                             totals);
  timing_end(family);
  MKS_CUDA(cudaGetLastError());
  return MKS_OK;
}

// ------------------------------------------------------------------
// D_eo launchers
struct LinkSet64 { LinkF64 fat, lng; };
struct LinkSet32 { LinkF32 fat, lng; };
struct LinkSet16 { LinkF16 fat, lng; };

static LinkSet64 links64(const LinkSlot &s) { return {{s.fat64}, {s.lng64}}; }
static LinkSet32 links32(const LinkSlot &s) { return {{s.fat32a, s.fat32b}, {s.lng32a, s.lng32b}}; }
static LinkSet16 links16(const LinkSlot &s) {
  return {{s.fat16a, s.fat16b, s.fat16scale}, {s.lng16a, s.lng16b, s.lng16scale}};
}

// ------------------------------------------------------------------
// D_eo launch shapes and their autotuner.
// A shape is (G threads per site, NB sources per thread, block size).  The
// first launch for a given (link precision, class of source counts: 1, 2,
// 3-4, 5-8, 9-16) times the candidates with G*NB >= the class's widest
// count (and at most 2x padding) on the live links and scratch vectors,
// over at most 2^20 sites, keeps the fastest, and reuses it for every count
// of the class; plain and fused-epilogue launches are tuned apart.
// MKS_TUNE=0 turns tuning off (fixed table); the choices can be read back
// with mks_tuned_shape().
// launch shape: G threads per site, NB sources per thread, block size;
// tma = 1: the FP32 kernel that stages each tile's links in shared memory
// (NB = 1, block = T G for a tile of T sites); pipe = 1: the kernel whose
// link loads are software-pipelined one term deep (k_dslash_p)
// persist = 1: a persistent grid (as many CTAs as fit on the GPU at once)
// that loops over the site blocks, so a fused-epilogue launch reduces its
// dot products once per CTA rather than once per site block
// as = 2 or 3: FP32 links fetched ahead into shared memory by cp.async with
// that many link buffers per site (k_dslash_a)
struct Shape { int G, NB, block, tma, pipe, persist, as; };
static Shape g_shape[3][MAXSRC + 1];      // [prec][nsrc], G == 0: not chosen yet
static Shape g_shape_epi[3][MAXSRC + 1];  // the same for the fused-epilogue launches
static void shapes_reset() {
  memset(g_shape, 0, sizeof g_shape);
  memset(g_shape_epi, 0, sizeof g_shape_epi);
}

// The TMA-staged kernel is switched off for the rest of the process once one
// of its staging waits ran out (red_check reports it): the shapes that use
// it are dropped (re-chosen without it at the next launch) with the graphs
// that bake them in, and the solver entry points repeat their work once.
static bool g_tma_off = false, g_tma_retry = false;
void tma_disable() {
  g_tma_off = true;
  g_tma_retry = true;
  for (auto *tab : {g_shape, g_shape_epi})
    for (int p = 0; p < 3; p++)
      for (int n = 0; n <= MAXSRC; n++)
        if (tab[p][n].tma) tab[p][n] = Shape{0, 0, 0, 0, 0, 0, 0};
  graphs_free_all();
}
// true once after tma_disable: the failed call may be repeated
static bool take_tma_retry() {
  const bool r = g_tma_retry;
  g_tma_retry = false;
  return r;
}

static int tune_class(int nsrc) {
  return nsrc <= 2 ? nsrc : nsrc <= 4 ? 4 : nsrc <= 8 ? 8 : MAXSRC;
}

// Tuning launches cover at most this many output sites (the first ones):
// enough site blocks for many waves on every shape, and on large lattices a
// fraction of a full launch (a 16-source FP64 D_eo on 48^3x96 takes 80 ms).
constexpr size_t TUNE_SITES = size_t(1) << 20;

static Shape default_shape(int nsrc) {
  if (nsrc <= 1) return {1, 1, 256, 0, 0};
  if (nsrc <= 2) return {1, 2, 256, 0, 0};
  if (nsrc <= 4) return {1, 4, 256, 0, 0};
  if (nsrc <= 8) return {2, 4, 256, 0, 0};
  return {4, 4, 256, 0, 0};
}

// tile of the TMA kernel for G threads per site: R complete x-rows of nx/2
// sites (R dividing ny), T G <= 256 threads, a whole number of warps; the
// bulk copies need nx/2 even (16-byte aligned row segments).  false when
// the lattice admits no such tile.
constexpr int TMA_MAX_SMEM = 200 * 1024;  // dynamic shared memory of the staged links, bytes
static bool tma_tile(const Geom &g, int G, int *T, int *R) {
  if (g.nx % 4 || g.ny < 4 || g.nz < 4 || g.nt < 4 || G < 1 || G > 16) return false;
  const int nx2 = g.nx / 2;
  for (int r = g.ny; r >= 1; r--) {
    if (g.ny % r) continue;
    const int t = r * nx2;
    if (t * G > 256 || (t * G) % 32 || (size_t)t * 1152 > (size_t)TMA_MAX_SMEM) continue;
    *T = t;
    *R = r;
    return true;
  }
  return false;
}

template <class LinkT> struct PrecOf;
template <> struct PrecOf<LinkF64> { enum { v = MKS_PREC_DOUBLE }; typedef VecF64 In; typedef VecF64 Out; typedef double R; };
template <> struct PrecOf<LinkF32> { enum { v = MKS_PREC_SINGLE }; typedef VecF32 In; typedef VecF32 Out; typedef float R; };
template <> struct PrecOf<LinkF16> { enum { v = MKS_PREC_HALF }; typedef VecF16 In; typedef VecF32 Out; typedef float R; };

// CTAs of `kernel` with `block` threads that fit on one SM at once
template <class K> static int resident_blocks(K kernel, int block) {
  static std::map<std::pair<const void *, int>, int> cache;
  const auto key = std::make_pair((const void *)kernel, block);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, block, 0) != cudaSuccess || n < 1) {
    cudaGetLastError();
    n = 1;
  }
  cache[key] = n;
  return n;
}

// The variant kernels (software-pipelined, persistent grid, cp.async link
// buffers) are built for the FP32 plain D_eo only, the launch where they
// were measured; elsewhere a shape that asks for one runs the direct kernel.
template <class LinkT, int EPI> constexpr bool has_variants() {
  return std::is_same<LinkT, LinkF32>::value && EPI == EPI_PLAIN;
}

template <typename R, class LinkT, class InT, class OutT, int NB, int EPI, int NSUM, class Fin>
static int launch_dslash_nb(int family, const LinkT &fat, const LinkT &lng,
                            DslashArgs<InT, OutT, typename EpiLoad<R>::type> &a, const Fin &fin, int block,
                            bool pipe, bool persist, int as = 0) {
  Context &c = ctx();
  const size_t sites = family == MKS_K_TUNE && c.Vh > TUNE_SITES ? TUNE_SITES : c.Vh;
  size_t threads = sites * a.groups;
  const int nvb = (int)((threads + block - 1) / block);
  if constexpr (has_variants<LinkT, EPI>()) {
    if (as == 2 || as == 3) {
      const int grid = nvb;
      a.nvb = 0;
      const size_t smem = (size_t)as * 72 * (block / a.groups);
      if (NSUM > 0) {
        MKS_TRY(ensure_red(NSUM * a.groups * NB, grid));
        a.red = c.red;
      }
      auto ka = as == 2 ? k_dslash_a<InT, OutT, NB, EPI, NSUM, Fin, 2> : k_dslash_a<InT, OutT, NB, EPI, NSUM, Fin, 3>;
      static bool attr[2] = {false, false};
      if (smem > 48 * 1024 && !attr[as - 2]) {
        MKS_CUDA(cudaFuncSetAttribute(ka, cudaFuncAttributeMaxDynamicSharedMemorySize, 3 * 72 * 256));
        attr[as - 2] = true;
      }
      timing_begin(family);
      ka<<<grid, block, smem, c.stream>>>(fat, lng, a, fin);
      timing_end(family);
      MKS_CUDA(cudaGetLastError());
      return MKS_OK;
    }
  }
  auto k1 = k_dslash1<R, LinkT, InT, OutT, EPI, NSUM, Fin>;
  auto kd = k_dslash<R, LinkT, InT, OutT, NB, EPI, NSUM, Fin>;
  if constexpr (!has_variants<LinkT, EPI>()) {
    pipe = false;
    persist = false;
  }
  if (persist) pipe = false;  // the persistent kernel loads directly
  const bool one = !pipe && !persist && NB == 1 && a.groups == 1 && block == 256;
  int grid = nvb;
  a.nvb = 0;
  if constexpr (has_variants<LinkT, EPI>()) {
    if (persist) {
      const int cap = resident_blocks(k_dslash_g<R, LinkT, InT, OutT, NB, EPI, NSUM, Fin>, block) * c.sm_count;
      if (cap < nvb) grid = cap;
      a.nvb = nvb;
    }
  }
  if (NSUM > 0) {
    MKS_TRY(ensure_red(NSUM * a.groups * NB, grid));
    a.red = c.red;
  }
  timing_begin(family);
  if constexpr (has_variants<LinkT, EPI>()) {
    if (persist)
      k_dslash_g<R, LinkT, InT, OutT, NB, EPI, NSUM, Fin><<<grid, block, 0, c.stream>>>(fat, lng, a, fin);
    else if (pipe)
      k_dslash_p<R, LinkT, InT, OutT, NB, EPI, NSUM, Fin><<<grid, block, 0, c.stream>>>(fat, lng, a, fin);
    else if (one)
      k1<<<grid, block, 0, c.stream>>>(fat, lng, a, fin);
    else
      kd<<<grid, block, 0, c.stream>>>(fat, lng, a, fin);
  } else {
    if (one)
      k1<<<grid, block, 0, c.stream>>>(fat, lng, a, fin);
    else
      kd<<<grid, block, 0, c.stream>>>(fat, lng, a, fin);
  }
  timing_end(family);
  MKS_CUDA(cudaGetLastError());
  return MKS_OK;
}

template <typename R, class LinkT, class InT, class OutT, int EPI, int NSUM, class Fin>
static int launch_shape(int family, const LinkT &fat, const LinkT &lng,
                        DslashArgs<InT, OutT, typename EpiLoad<R>::type> &a, const Fin &fin, const Shape &sh) {
  a.groups = sh.G;
  a.g = ctx().geom;
  if (EPI == EPI_PLAIN) a.rev = 1;
  if constexpr (std::is_same<LinkT, LinkF32>::value && std::is_same<InT, VecF32>::value &&
                std::is_same<OutT, VecF32>::value) {
    if (sh.tma) {
      Context &c = ctx();
      int T, Rr;
      if (sh.NB != 1 || !tma_tile(a.g, sh.G, &T, &Rr) || a.nsrc > sh.G) return MKS_ERR_ARG;
      const int grid = (int)((family == MKS_K_TUNE && c.Vh > TUNE_SITES ? TUNE_SITES : c.Vh) / T);
      const size_t smem = (size_t)T * 1152;
      static bool attr = false;
      if (!attr) {
        MKS_CUDA(cudaFuncSetAttribute(k_dslash_tma<EPI, NSUM, Fin>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      TMA_MAX_SMEM));
        attr = true;
      }
      MKS_TRY(ensure_red(NSUM > 0 ? NSUM * sh.G : 1, grid));
      a.red = c.red;
      timing_begin(family);
      k_dslash_tma<EPI, NSUM, Fin><<<grid, T * sh.G, smem, c.stream>>>(fat, lng, a, fin, T, Rr);
      timing_end(family);
      MKS_CUDA(cudaGetLastError());
      return MKS_OK;
    }
  }
  const bool pipe = sh.pipe != 0, persist = sh.persist != 0;
  switch (sh.NB) {
  case 1:
    return launch_dslash_nb<R, LinkT, InT, OutT, 1, EPI, NSUM, Fin>(family, fat, lng, a, fin, sh.block, pipe, persist,
                                                                   sh.as);
  case 2:
    return launch_dslash_nb<R, LinkT, InT, OutT, 2, EPI, NSUM, Fin>(family, fat, lng, a, fin, sh.block, pipe, persist,
                                                                   sh.as);
  case 4:
    return launch_dslash_nb<R, LinkT, InT, OutT, 4, EPI, NSUM, Fin>(family, fat, lng, a, fin, sh.block, pipe, persist,
                                                                   sh.as);
  default:
    return launch_dslash_nb<R, LinkT, InT, OutT, 8, EPI, NSUM, Fin>(family, fat, lng, a, fin, sh.block, pipe, persist,
                                                                   sh.as);
  }
}

__global__ void k_fill_tune(float *v, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    v[i] = 0.25f * (float)((i * 2654435761u) >> 24 & 255) / 255.0f;
}

static bool tuning_enabled() {
  static int v = -1;
  if (v < 0) {
    const char *e = getenv("MKS_TUNE");
    v = e ? atoi(e) : 1;
  }
  return v != 0;
}

// The FP32 CG iteration runs its second D_eo as a plain D and the FEWSUMS
// dot products in a separate site kernel (the update forms ttt - 4m^2 p
// itself); MKS_SPLIT_EPI=0 fuses axpy and dot products into the D_eo
// instead.  Measured on GB300 (8 sources, 32^3x64, 1e-10): 0.0641 against
// 0.0663 s per solved source -- the fused-epilogue D_eo holds 73 registers
// (3 resident blocks per SM against 4 for the plain D) and its extra loads
// sit at the end of the latency-bound site loop, while the dot kernel
// streams at the HBM rate.
static bool split_epilogue() {
  static int v = -1;
  if (v < 0) {
    const char *e = getenv("MKS_SPLIT_EPI");
    v = e ? atoi(e) : 1;
  }
  return v != 0;
}

// MKS_ASYNC=1 adds the cp.async link-prefetch D_eo kernel (k_dslash_a) to the
// tuner's candidates.  Off by default: measured on GB300 (8 sources,
// 32^3x64) its D_eo took 350 ms (2 stages) and 415 ms (3 stages) per solve
// of 8 against 230 ms for k_dslash, and one source 112 against 103 ms.
static bool async_enabled() {
  static int v = -1;
  if (v < 0) {
    const char *e = getenv("MKS_ASYNC");
    v = e ? atoi(e) : 0;
  }
  return v != 0;
}

// MKS_PIPE=1 and MKS_PERSIST=1 add the software-pipelined (k_dslash_p) and
// the persistent-grid (k_dslash_g) D_eo kernels to the tuner's candidates.
// Off by default: on GB300 neither beat k_dslash on a solve (8 sources,
// 32^3x64: 0.0713-0.0733 and 0.0745-0.0793 against 0.0669 s per source),
// and every extra candidate costs tuning launches at the first use of each
// source count (on 48^3x96 a trajectory's tuning took 84 s with both on).
static bool pipe_enabled() {
  static int v = -1;
  if (v < 0) {
    const char *e = getenv("MKS_PIPE");
    v = e ? atoi(e) : 0;
  }
  return v != 0;
}
static bool persist_enabled() {
  static int v = -1;
  if (v < 0) {
    const char *e = getenv("MKS_PERSIST");
    v = e ? atoi(e) : 0;
  }
  return v != 0;
}

// The sloppy multi-shift stops on the lowest shift's iterated residual, as
// the FP64 solve does; the FP64 check of every shift follows.
// MKS_MS_TRUE_STOP=1 makes it stop only when that shift's residual,
// recomputed in FP64 by a reliable update, meets the target -- measured on
// GB300 (11 offsets, 32^3x64, 1e-10) it buys nothing: 0.432 against 0.430 s,
// the lowest shift then passing the check with one refinement iteration
// either way.
static bool ms_true_stop() {
  static int v = -1;
  if (v < 0) {
    const char *e = getenv("MKS_MS_TRUE_STOP");
    v = e ? atoi(e) : 0;
  }
  return v != 0;
}

// For targets below 1e-7 the sloppy single-field multi-shift keeps the
// shifts' search directions p_j and solutions x_j in FP64 (residual, D_eo
// and the lowest shift's D_eo input in FP32).  The update kernel then moves
// twice the bytes per shift, but fewer shifts miss a tight target after
// the sloppy phase, so the block-CG refinement that follows shrinks.
// Measured on GB300 (11 offsets, 32^3x64, 1e-10): 0.392 against 0.425 s
// (329 against 352 iterations for the slowest shift).  The batched-field
// solves of the RHMC trajectory keep FP32: the 2+1+1 48^3x96 trajectory
// took 39.9 s so, 40.4 s with FP64 storage in its 1e-10 solves and 46.6 s
// with it in every solve.  MKS_MS_SHIFT64=1 / 0 forces FP64 / FP32.
static bool ms_shift64(double resid, bool batched) {
  static int v = -2;
  if (v == -2) {
    const char *e = getenv("MKS_MS_SHIFT64");
    v = e ? atoi(e) : -1;
  }
  return v < 0 ? (!batched && resid < 1e-7) : v != 0;
}

static void set_vec(VecF64 &v, float *p, float *) { v.p = (double2 *)p; }
static void set_vec(VecF32 &v, float *p, float *) { v.p = (float2 *)p; }
static void set_vec(VecF16 &v, float *p, float *n) { v.p = (__half2 *)p; v.norm = n; }

// EPI = EPI_AXPY times the fused CG epilogue (3 sums, no finisher): its
// block reduction and extra reads can favour another shape than plain D
template <class LinkT, int EPI = EPI_PLAIN>
static int tune_shape(const LinkT &fat, const LinkT &lng, int nsrc, Shape *best) {
  typedef PrecOf<LinkT> P;
  typedef typename P::R R;
  typedef typename P::In InT;
  typedef typename P::Out OutT;
  Context &c = ctx();
  *best = default_shape(nsrc);
  if (!tuning_enabled()) return MKS_OK;
  const size_t n = 3 * c.Vh;
  DslashArgs<InT, OutT, typename EpiLoad<R>::type> a;
  memset(&a, 0, sizeof a);
  a.nsrc = nsrc;
  a.out_par = 0;
  for (int s = 0; s < nsrc; s++) {
    float *in, *out, *nrm;
    MKS_TRY(wsv("tune_in" + std::to_string(s), n * 4, &in));     // large enough for any precision
    MKS_TRY(wsv("tune_out" + std::to_string(s), n * 4, &out));
    MKS_TRY(wsv("tune_nrm" + std::to_string(s), c.Vh, &nrm));
    k_fill_tune<<<c.sm_count * 4, 256, 0, c.stream>>>(in, n * 4);
    c.launches++;
    k_fill_tune<<<c.sm_count * 4, 256, 0, c.stream>>>(nrm, c.Vh);
    c.launches++;
    set_vec(a.in[s], in, nrm);
    set_vec(a.out[s], out, nrm);
    if (EPI == EPI_AXPY) {
      float *pp, *rr;
      MKS_TRY(wsv("tune_p" + std::to_string(s), n * 4, &pp));
      MKS_TRY(wsv("tune_r" + std::to_string(s), n * 4, &rr));
      k_fill_tune<<<c.sm_count * 4, 256, 0, c.stream>>>(pp, n * 4);
      c.launches++;
      k_fill_tune<<<c.sm_count * 4, 256, 0, c.stream>>>(rr, n * 4);
      c.launches++;
      a.p[s].p = (decltype(a.p[s].p))pp;
      a.r[s].p = (decltype(a.r[s].p))rr;
      a.coef[s] = -0.01;
    }
  }
  if (EPI == EPI_AXPY) {
    float *tot;
    MKS_TRY(wsv("tune_totals", 2 * MAXSRC * 3, &tot));
    a.totals = (double *)tot;
  }
  MKS_CUDA(cudaGetLastError());
  cudaEvent_t e0, e1;
  MKS_CUDA(cudaEventCreate(&e0));
  MKS_CUDA(cudaEventCreate(&e1));
  // One launch per candidate first; a candidate more than 1.5x slower than
  // the best average so far is dropped after it, the others are timed over
  // 3 more launches.  The default shape goes first so that slow candidates
  // (spilling source counts per thread, wide G) cost one launch each.
  float best_ms = 1e30f;
  auto time_one = [&](const Shape &sh, float *ms) -> int {
    MKS_CUDA(cudaEventRecord(e0, c.stream));
    MKS_TRY((launch_shape<R, LinkT, InT, OutT, EPI, (EPI == EPI_AXPY ? 3 : 0)>(MKS_K_TUNE, fat, lng, a, NoFinish(),
                                                                                sh)));
    MKS_CUDA(cudaEventRecord(e1, c.stream));
    MKS_CUDA(cudaEventSynchronize(e1));
    MKS_CUDA(cudaEventElapsedTime(ms, e0, e1));
    return MKS_OK;
  };
  auto try_shape = [&](const Shape &sh) -> int {
    float first, ms, tot = 0;
    MKS_TRY(time_one(sh, &first));
    if (sh.tma) MKS_TRY(red_check());
    if (first > 1.5f * best_ms) return MKS_OK;
    for (int it = 0; it < 3; it++) {
      MKS_TRY(time_one(sh, &ms));
      tot += ms;
    }
    if (sh.tma) MKS_TRY(red_check());
    if (tot / 3 < best_ms) { best_ms = tot / 3; *best = sh; }
    return MKS_OK;
  };
  const Shape def = *best;
  MKS_TRY(try_shape(def));
  const int nbs[4] = {1, 2, 4, 8};
  for (int ib = 0; ib < 4; ib++) {
    for (int G = 1; G <= 16; G *= 2) {
      const int NB = nbs[ib];
      if (G * NB < nsrc || G * NB > MAXSRC || (G * NB >= 2 * nsrc && G * NB > 1)) continue;
      for (int cand = 0; cand < 12; cand++) {
        // 0-7: block x pipelined x persistent; 8-11: block x cp.async stages 2, 3 (FP32 links)
        const int block = (cand & 1) ? 256 : 128;
        const int pipe = cand < 8 ? (cand >> 1) & 1 : 0, persist = cand < 8 ? (cand >> 2) & 1 : 0;
        const int as = cand < 8 ? 0 : 2 + ((cand >> 1) & 1);
        if ((pipe && !pipe_enabled()) || (persist && !persist_enabled()) || (pipe && persist)) continue;
        if (as && !async_enabled()) continue;
        if ((pipe || persist || as) && !has_variants<LinkT, EPI>()) continue;
        Shape sh = {G, NB, block, 0, pipe, persist, as};
        if (memcmp(&sh, &def, sizeof sh) == 0) continue;
        MKS_TRY(try_shape(sh));
      }
    }
  }
  if constexpr (std::is_same<LinkT, LinkF32>::value) {
    // the TMA-staged kernel: one source per thread, G = nsrc rounded up to a power of two
    int G = 1;
    while (G < nsrc) G *= 2;
    int T, Rr;
    if (nsrc >= 2 && !g_tma_off && tma_tile(c.geom, G, &T, &Rr)) {
      Shape sh = {G, 1, T * G, 1};
      MKS_TRY(try_shape(sh));
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return MKS_OK;
}

// MKS_SHAPE="prec:nsrc:G:NB:block[,...]" fixes shapes by hand (a tuning
// cache written by the user); entries must satisfy G*NB >= nsrc, G*NB <= 16,
// NB in {1,2,4,8}, G a power of two, block in {128,256}.  The entry
// "prec:nsrc:G:1:tma" (prec 1, FP32) selects the TMA-staged kernel with G
// threads per site, where the lattice admits its tiles.  A trailing ":p"
// selects the software-pipelined kernel, ":g" the persistent grid, ":a2" or
// ":a3" the cp.async link buffers (FP32 plain D only).  A leading "d" or "e"
// limits an entry to the plain D or to the fused-epilogue launches.
static bool shape_override(int prec, int nsrc, bool epi, Shape *out) {
  const char *e = getenv("MKS_SHAPE");
  if (!e) return false;
  std::string str(e);
  size_t pos = 0;
  while (pos < str.size()) {
    size_t end = str.find(',', pos);
    if (end == std::string::npos) end = str.size();
    std::string item = str.substr(pos, end - pos);
    if (!item.empty() && (item[0] == 'd' || item[0] == 'e')) {
      const bool for_epi = item[0] == 'e';
      item = item.substr(1);
      if (for_epi != epi) {
        pos = end + 1;
        continue;
      }
    }
    int p, n, G, NB, B;
    if (sscanf(item.c_str(), "%d:%d:%d:%d:%d", &p, &n, &G, &NB, &B) == 5 && p == prec &&
        n == nsrc && G >= 1 && G <= 16 && (G & (G - 1)) == 0 && (NB == 1 || NB == 2 || NB == 4 || NB == 8) &&
        G * NB >= nsrc && G * NB <= MAXSRC && (B == 128 || B == 256)) {
      const size_t f = item.find_first_not_of("0123456789:");
      const std::string flags = f == std::string::npos ? "" : item.substr(f);
      // the variant kernels exist for the FP32 plain D_eo only
      const bool var = prec == MKS_PREC_SINGLE && !epi;
      const int pipe = var && flags.find('p') != std::string::npos;
      const int persist = var && flags.find('g') != std::string::npos;
      const size_t fa = flags.find('a');
      const int as = (fa != std::string::npos && fa + 1 < flags.size()) ? flags[fa + 1] - '0' : 0;
      *out = {G, NB, B, 0, pipe, persist, var && (as == 2 || as == 3) ? as : 0};
      return true;
    }
    int T, Rr;
    if (!g_tma_off && sscanf(item.c_str(), "%d:%d:%d:%d:", &p, &n, &G, &NB) == 4 && item.size() > 4 &&
        item.compare(item.size() - 4, 4, ":tma") == 0 && p == MKS_PREC_SINGLE && p == prec && n == nsrc &&
        NB == 1 && G >= nsrc && G <= 16 && (G & (G - 1)) == 0 && tma_tile(ctx().geom, G, &T, &Rr)) {
      *out = {G, 1, T * G, 1};
      return true;
    }
    pos = end + 1;
  }
  return false;
}

template <typename R, class LinkT, class InT, class OutT, int EPI, int NSUM, class Fin>
static int launch_dslash(int family, const LinkT &fat, const LinkT &lng,
                         DslashArgs<InT, OutT, typename EpiLoad<R>::type> &a, const Fin &fin) {
  const int pk = PrecOf<LinkT>::v;
  Shape(&tab)[MAXSRC + 1] = (EPI == EPI_AXPY ? g_shape_epi : g_shape)[pk];
  Shape &sh = tab[a.nsrc];
  if (sh.G == 0) {
    Shape t;
    if (!shape_override(pk, a.nsrc, EPI == EPI_AXPY, &t)) {
      // source counts are tuned in classes 1, 2, 3-4, 5-8, 9-16: the shape
      // tuned for a class's widest count serves every count of the class
      // (the unused source slots of a thread are masked)
      const int cls = tune_class(a.nsrc);
      if (tab[cls].G == 0) {
        if (EPI == EPI_AXPY) MKS_TRY((tune_shape<LinkT, EPI_AXPY>(fat, lng, cls, &tab[cls])));
        else MKS_TRY(tune_shape(fat, lng, cls, &tab[cls]));
      }
      t = tab[cls];
    }
    sh = t;
  }
  if (a.nsrc > 1 && family != MKS_K_DSLASH_F64) family = MKS_K_DSLASH_MRHS;
  return launch_shape<R, LinkT, InT, OutT, EPI, NSUM, Fin>(family, fat, lng, a, fin, sh);
}

// plain D on FP64 SoA fields, nsrc sources
static int dslash64(const LinkSlot &sl, int out_par, int nsrc, double2 *const *in, double2 *const *out,
                    const int *skip = nullptr) {
  DslashArgs<VecF64, VecF64, VecF64> a;
  memset(&a, 0, sizeof a);
  a.out_par = out_par; a.nsrc = nsrc; a.skip = skip;
  for (int s = 0; s < nsrc; s++) { a.in[s].p = in[s]; a.out[s].p = out[s]; }
  LinkSet64 L = links64(sl);
  return launch_dslash<double, LinkF64, VecF64, VecF64, EPI_PLAIN, 0>(MKS_K_DSLASH_F64, L.fat, L.lng, a, FinNone());
}

// ------------------------------------------------------------------
// per-parity field views inside one contiguous "full" SoA buffer:
// full field = [2][3][Vh] double2; parity par starts at par*3*Vh
static inline double2 *par64(double2 *full, int par) { return full + (size_t)par * 3 * ctx().Vh; }

static int parity_index(int parity, int *par) {
  if (parity == MKS_EVEN) *par = 0;
  else if (parity == MKS_ODD) *par = 1;
  else return MKS_ERR_ARG;
  return MKS_OK;
}

static int slot_ok(int slot) {
  if (slot < 0 || slot >= MKS_MAX_SLOTS) return MKS_ERR_ARG;
  if (!ctx().slots[slot].valid) return MKS_ERR_STATE;
  return MKS_OK;
}

// ------------------------------------------------------------------
// public D
static int dslash_dev_impl(const double *src_dev, double *dst_dev, int parity, int slot) {
  Context &c = ctx();
  double2 *in, *out;
  MKS_TRY(wsv("ds_in", 6 * c.Vh, &in));
  MKS_TRY(wsv("ds_out", 6 * c.Vh, &out));
  const LinkSlot &sl = c.slots[slot];
  for (int op = 0; op < 2; op++) {
    int out_par = op;
    bool want = (parity == MKS_EVENANDODD) || (parity == MKS_EVEN && op == 0) || (parity == MKS_ODD && op == 1);
    if (!want) continue;
    MKS_TRY(vec_aos_to_soa64(src_dev, par64(in, 1 - out_par), 1 - out_par));
  }
  for (int op = 0; op < 2; op++) {
    bool want = (parity == MKS_EVENANDODD) || (parity == MKS_EVEN && op == 0) || (parity == MKS_ODD && op == 1);
    if (!want) continue;
    double2 *pin = par64(in, 1 - op), *pout = par64(out, op);
    MKS_TRY(dslash64(sl, op, 1, &pin, &pout));
    MKS_TRY(vec_soa64_to_aos(pout, dst_dev, op));
  }
  return MKS_OK;
}

}  // namespace mks

using namespace mks;

extern "C" int mks_dslash_fn_field_dev(const double *src_dev, double *dst_dev, int parity, int slot) {
  MKS_TRY(check_ready());
  MKS_TRY(slot_ok(slot));
  if (!src_dev || !dst_dev || parity < MKS_ODD || parity > MKS_EVENANDODD) return MKS_ERR_ARG;
  MKS_TRY(dslash_dev_impl(src_dev, dst_dev, parity, slot));
  MKS_CUDA(cudaStreamSynchronize(ctx().stream));
  return MKS_OK;
}

extern "C" int mks_dslash_fn_field(const double *src, double *dst, int parity, int slot) {
  MKS_TRY(check_ready());
  MKS_TRY(slot_ok(slot));
  if (!src || !dst || parity < MKS_ODD || parity > MKS_EVENANDODD) return MKS_ERR_ARG;
  Context &c = ctx();
  size_t bytes = c.V * 6 * sizeof(double);
  double *ds, *dd;
  MKS_TRY(wsv("host_src", 6 * c.V, &ds));
  MKS_TRY(wsv("host_dst", 6 * c.V, &dd));
  MKS_CUDA(cudaMemcpyAsync(ds, src, bytes, cudaMemcpyHostToDevice, c.stream));
  MKS_CUDA(cudaMemcpyAsync(dd, dst, bytes, cudaMemcpyHostToDevice, c.stream));
  MKS_TRY(dslash_dev_impl(ds, dd, parity, slot));
  MKS_CUDA(cudaMemcpyAsync(dst, dd, bytes, cudaMemcpyDeviceToHost, c.stream));
  MKS_CUDA(cudaStreamSynchronize(c.stream));
  return MKS_OK;
}

namespace mks {

// ------------------------------------------------------------------
// block CG driver (nsrc = 1 is the single-source solver)
struct CgFields {
  // FP64, one parity [3][Vh] per source
  double2 *src[MAXSRC], *x[MAXSRC], *r[MAXSRC], *p[MAXSRC], *ttt[MAXSRC], *t[MAXSRC];  // t: other parity
  // sloppy
  float2 *x32[MAXSRC], *r32[MAXSRC], *p32[MAXSRC], *ttt32[MAXSRC], *t32[MAXSRC];
  __half2 *p16[MAXSRC], *t16[MAXSRC];
  float *p16n[MAXSRC], *t16n[MAXSRC];
};

static int alloc_cg_fields(CgFields &f, int nsrc, int prec) {
  Context &c = ctx();
  size_t n = 3 * c.Vh;
  for (int s = 0; s < nsrc; s++) {
    std::string k = std::to_string(s);
    MKS_TRY(wsv("cg_src" + k, n, &f.src[s]));
    MKS_TRY(wsv("cg_x" + k, n, &f.x[s]));
    MKS_TRY(wsv("cg_r" + k, n, &f.r[s]));
    MKS_TRY(wsv("cg_p" + k, n, &f.p[s]));
    MKS_TRY(wsv("cg_ttt" + k, n, &f.ttt[s]));
    MKS_TRY(wsv("cg_t" + k, n, &f.t[s]));
    if (prec != MKS_PREC_DOUBLE) {
      MKS_TRY(wsv("cg_x32" + k, n, &f.x32[s]));
      MKS_TRY(wsv("cg_r32" + k, n, &f.r32[s]));
      MKS_TRY(wsv("cg_p32" + k, n, &f.p32[s]));
      MKS_TRY(wsv("cg_ttt32" + k, n, &f.ttt32[s]));
      MKS_TRY(wsv("cg_t32" + k, n, &f.t32[s]));
      if (prec == MKS_PREC_HALF) {
        MKS_TRY(wsv("cg_p16" + k, n, &f.p16[s]));
        MKS_TRY(wsv("cg_t16" + k, n, &f.t16[s]));
        MKS_TRY(wsv("cg_p16n" + k, c.Vh, &f.p16n[s]));
        MKS_TRY(wsv("cg_t16n" + k, c.Vh, &f.t16n[s]));
      } else {
        f.p16[s] = nullptr; f.t16[s] = nullptr; f.p16n[s] = nullptr; f.t16n[s] = nullptr;
      }
    }
  }
  return MKS_OK;
}

int dslash32_multi(int slot, int out_par, int nsrc, float2 *const *in, float2 *const *out) {
  MKS_TRY(slot_ok(slot));
  const LinkSlot &sl = ctx().slots[slot];
  if (!sl.valid || !sl.fat32a) return MKS_ERR_STATE;
  LinkSet32 L = links32(sl);
  for (int b0 = 0; b0 < nsrc; b0 += MAXSRC) {
    const int nb = nsrc - b0 < MAXSRC ? nsrc - b0 : MAXSRC;
    DslashArgs<VecF32, VecF32, VecF32> a;
    memset(&a, 0, sizeof a);
    a.out_par = out_par; a.nsrc = nb;
    for (int q = 0; q < nb; q++) { a.in[q].p = in[b0 + q]; a.out[q].p = out[b0 + q]; }
    MKS_TRY((launch_dslash<float, LinkF32, VecF32, VecF32, EPI_PLAIN, 0>(MKS_K_DSLASH_F32, L.fat, L.lng, a,
                                                                       FinNone())));
  }
  return MKS_OK;
}

// ttt <- D_par D_opar x  (FP64) for the sources listed
static int apply_DD64(const LinkSlot &sl, int par, int nsrc, double2 *const *x, double2 *const *t,
                      double2 *const *ttt) {
  MKS_TRY(dslash64(sl, 1 - par, nsrc, x, t));
  MKS_TRY(dslash64(sl, par, nsrc, t, ttt));
  return MKS_OK;
}

static int read_states(Solver &S, int nsrc, CgState *h) {
  Context &c = ctx();
  MKS_CUDA(cudaMemcpyAsync(h, S.st, nsrc * sizeof(CgState), cudaMemcpyDeviceToHost, c.stream));
  MKS_CUDA(cudaStreamSynchronize(c.stream));
  return red_check();
}
static int write_states(Solver &S, int nsrc, const CgState *h, int skip) {
  Context &c = ctx();
  MKS_CUDA(cudaMemcpyAsync(S.st, h, nsrc * sizeof(CgState), cudaMemcpyHostToDevice, c.stream));
  MKS_CUDA(cudaMemcpyAsync(S.skip, &skip, sizeof(int), cudaMemcpyHostToDevice, c.stream));
  MKS_CUDA(cudaStreamSynchronize(c.stream));
  return MKS_OK;
}

// one sloppy or FP64 CG iteration for all running sources (3 launches)
static int cg_iteration(const LinkSlot &sl, int par, int nsrc, int prec, const double *msq4, CgFields &f, Solver &S) {
  if (prec == MKS_PREC_DOUBLE) {
    DslashArgs<VecF64, VecF64, VecF64> a1;
    memset(&a1, 0, sizeof a1);
    a1.out_par = 1 - par; a1.nsrc = nsrc; a1.skip = S.skip;
    for (int s = 0; s < nsrc; s++) { a1.in[s].p = f.p[s]; a1.out[s].p = f.t[s]; }
    LinkSet64 L = links64(sl);
    MKS_TRY((launch_dslash<double, LinkF64, VecF64, VecF64, EPI_PLAIN, 0>(MKS_K_DSLASH_F64, L.fat, L.lng, a1, FinNone())));
    DslashArgs<VecF64, VecF64, VecF64> a2;
    memset(&a2, 0, sizeof a2);
    a2.out_par = par; a2.nsrc = nsrc; a2.skip = S.skip;
    for (int s = 0; s < nsrc; s++) {
      a2.in[s].p = f.t[s]; a2.out[s].p = f.ttt[s]; a2.p[s].p = f.p[s]; a2.r[s].p = f.r[s]; a2.coef[s] = -msq4[s];
    }
    double *tot;
    MKS_TRY(wsv("cg_tot", 3 * MAXSRC, &tot));
    a2.totals = tot;
    MKS_TRY((launch_dslash<double, LinkF64, VecF64, VecF64, EPI_AXPY, 3>(MKS_K_DSLASH_F64, L.fat, L.lng, a2, FinCgAlpha{S.st})));
    OpUpdate<double> up;
    memset(&up, 0, sizeof up);
    for (int s = 0; s < nsrc; s++) { up.x[s] = f.x[s]; up.p[s] = f.p[s]; up.r[s] = f.r[s]; up.ttt[s] = f.ttt[s]; }
    up.st = S.st; up.Vh = (int)ctx().Vh; up.relres = 0;
    MKS_TRY((launch_site<OpUpdate<double>, 1, FinCgUpdate>(MKS_K_BLAS, up, FinCgUpdate{S.st, S.skip}, S.skip, nsrc)));
    return MKS_OK;
  }
  const int fam = prec == MKS_PREC_SINGLE ? MKS_K_DSLASH_F32 : MKS_K_DSLASH_F16;
  if (prec == MKS_PREC_SINGLE) {
    LinkSet32 L = links32(sl);
    DslashArgs<VecF32, VecF32, VecF32> a1;
    memset(&a1, 0, sizeof a1);
    a1.out_par = 1 - par; a1.nsrc = nsrc; a1.skip = S.skip;
    for (int s = 0; s < nsrc; s++) { a1.in[s].p = f.p32[s]; a1.out[s].p = f.t32[s]; }
    MKS_TRY((launch_dslash<float, LinkF32, VecF32, VecF32, EPI_PLAIN, 0>(fam, L.fat, L.lng, a1, FinNone())));
    DslashArgs<VecF32, VecF32, VecF32> a2;
    memset(&a2, 0, sizeof a2);
    a2.out_par = par; a2.nsrc = nsrc; a2.skip = S.skip;
    double *tot;
    MKS_TRY(wsv("cg_tot", 3 * MAXSRC, &tot));
    if (split_epilogue()) {
      // plain D (ttt = D t), then the dot products in a site kernel; the
      // update forms ttt - msq4 p itself
      for (int s = 0; s < nsrc; s++) { a2.in[s].p = f.t32[s]; a2.out[s].p = f.ttt32[s]; }
      MKS_TRY((launch_dslash<float, LinkF32, VecF32, VecF32, EPI_PLAIN, 0>(fam, L.fat, L.lng, a2, FinNone())));
      OpDots3<float> dt;
      memset(&dt, 0, sizeof dt);
      for (int s = 0; s < nsrc; s++) {
        dt.p[s] = f.p32[s]; dt.r[s] = f.r32[s]; dt.ttt[s] = f.ttt32[s]; dt.msq4[s] = msq4[s];
      }
      dt.Vh = (int)ctx().Vh;
      MKS_TRY((launch_site<OpDots3<float>, 3, FinCgAlpha>(MKS_K_BLAS, dt, FinCgAlpha{S.st}, S.skip, nsrc, tot)));
    } else {
      for (int s = 0; s < nsrc; s++) {
        a2.in[s].p = f.t32[s]; a2.out[s].p = f.ttt32[s]; a2.p[s].p = f.p32[s]; a2.r[s].p = f.r32[s];
        a2.coef[s] = -msq4[s];
      }
      a2.totals = tot;
      MKS_TRY((launch_dslash<float, LinkF32, VecF32, VecF32, EPI_AXPY, 3>(fam, L.fat, L.lng, a2, FinCgAlpha{S.st})));
    }
  } else {
    LinkSet16 L = links16(sl);
    DslashArgs<VecF16, VecF16, VecF32> a1;
    memset(&a1, 0, sizeof a1);
    a1.out_par = 1 - par; a1.nsrc = nsrc; a1.skip = S.skip;
    for (int s = 0; s < nsrc; s++) {
      a1.in[s].p = f.p16[s]; a1.in[s].norm = f.p16n[s]; a1.out[s].p = f.t16[s]; a1.out[s].norm = f.t16n[s];
    }
    MKS_TRY((launch_dslash<float, LinkF16, VecF16, VecF16, EPI_PLAIN, 0>(fam, L.fat, L.lng, a1, FinNone())));
    DslashArgs<VecF16, VecF32, VecF32> a2;
    memset(&a2, 0, sizeof a2);
    a2.out_par = par; a2.nsrc = nsrc; a2.skip = S.skip;
    for (int s = 0; s < nsrc; s++) {
      a2.in[s].p = f.t16[s]; a2.in[s].norm = f.t16n[s]; a2.out[s].p = f.ttt32[s];
      a2.p[s].p = f.p32[s]; a2.r[s].p = f.r32[s]; a2.coef[s] = -msq4[s];
    }
    double *tot;
    MKS_TRY(wsv("cg_tot", 3 * MAXSRC, &tot));
    a2.totals = tot;
    MKS_TRY((launch_dslash<float, LinkF16, VecF16, VecF32, EPI_AXPY, 3>(fam, L.fat, L.lng, a2, FinCgAlpha{S.st})));
  }
  OpUpdate<float> up;
  memset(&up, 0, sizeof up);
  for (int s = 0; s < nsrc; s++) {
    up.x[s] = f.x32[s]; up.p[s] = f.p32[s]; up.r[s] = f.r32[s]; up.ttt[s] = f.ttt32[s];
    up.p16[s] = f.p16[s]; up.p16n[s] = f.p16n[s]; up.msq4[s] = msq4[s];
  }
  up.fold = prec == MKS_PREC_SINGLE && split_epilogue();
  up.st = S.st; up.Vh = (int)ctx().Vh; up.relres = 0;
  MKS_TRY((launch_site<OpUpdate<float>, 1, FinCgUpdate>(MKS_K_BLAS, up, FinCgUpdate{S.st, S.skip}, S.skip, nsrc)));
  return MKS_OK;
}

// FP64 true residual for sources with status ST_HOST: r = src - M^dag M x,
// |r|^2 -> state (rsq, actual_rsq, final_rsq, iter++).  setp: p <- r.
// ------------------------------------------------------------------
// CUDA graphs for the solver iterations.  A batch of poll_interval()
// iterations (3 launches each) is captured once per configuration and then
// replayed with one cudaGraphLaunch; the first batch of a configuration runs
// eagerly so that the autotuner and the scratch buffers are settled before
// capture.  The key holds every pointer and scalar the launches bake in.
struct GraphEntry {
  std::vector<uint64_t> key;
  int seen = 0;
  cudaGraphExec_t exec = nullptr;
  Capture cap;
};
static std::vector<GraphEntry> g_graphs;

static bool graphs_enabled() {
  static int v = -1;
  if (v < 0) {
    const char *e = getenv("MKS_GRAPH");
    v = e ? atoi(e) : 1;
  }
  return v != 0;
}

static void free_graph(GraphEntry &e) {
  if (e.exec) cudaGraphExecDestroy(e.exec);
  for (auto ev : e.cap.ev) cudaEventDestroy(ev);
  e.exec = nullptr;
  e.cap = Capture();
}

void graphs_free_all() {
  for (auto &e : g_graphs) free_graph(e);
  g_graphs.clear();
}

template <typename T> static void key_push(std::vector<uint64_t> &k, const T &v) {
  uint64_t u = 0;
  memcpy(&u, &v, sizeof(T) < 8 ? sizeof(T) : 8);
  k.push_back(u);
}

static int cg_iteration(const LinkSlot &sl, int par, int nsrc, int prec, const double *msq4, CgFields &f, Solver &S);

// Run `issue` (a batch of launches on the context stream) through the graph
// cache: eagerly the first time a key is seen, captured and instantiated the
// second time, replayed afterwards.  The key must hold every pointer and
// scalar the launches bake in.
template <class F>
static int graph_batch(const std::vector<uint64_t> &key, F issue) {
  Context &c = ctx();
  if (!graphs_enabled()) return issue();
  // least recently used entries are dropped first (the list is kept in
  // order of use); the solves of a trajectory meet many distinct batches
  // (active-source sets of the refinements), and a dropped entry costs an
  // eager run and a new capture when it comes back
  GraphEntry *e = nullptr;
  for (size_t i = 0; i < g_graphs.size(); i++)
    if (g_graphs[i].key == key) {
      if (i + 1 < g_graphs.size()) std::rotate(g_graphs.begin() + i, g_graphs.begin() + i + 1, g_graphs.end());
      e = &g_graphs.back();
      break;
    }
  if (!e) {
    if (g_graphs.size() >= 128) { free_graph(g_graphs.front()); g_graphs.erase(g_graphs.begin()); }
    g_graphs.emplace_back();
    e = &g_graphs.back();
    e->key = key;
  }
  if (!e->exec) {
    if (e->seen++ == 0) return issue();
    Capture cap;
    cap.timed = c.timing;
    c.capture = &cap;
    int rc = MKS_OK;
    cudaError_t e0 = cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeRelaxed);
    if (e0 == cudaSuccess) rc = issue();
    cudaGraph_t graph = nullptr;
    cudaError_t e1 = e0 == cudaSuccess ? cudaStreamEndCapture(c.stream, &graph) : e0;
    c.capture = nullptr;
    if (rc < 0 || e1 != cudaSuccess || !graph) {
      if (graph) cudaGraphDestroy(graph);
      for (auto ev : cap.ev) cudaEventDestroy(ev);
      cudaGetLastError();
      if (rc < 0) return rc;
      set_last_error(e1, "cudaStreamEndCapture", __FILE__, __LINE__);
      return MKS_ERR_CUDA;
    }
    cudaError_t e2 = cudaGraphInstantiate(&e->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e2 != cudaSuccess) {
      for (auto ev : cap.ev) cudaEventDestroy(ev);
      e->exec = nullptr;
      set_last_error(e2, "cudaGraphInstantiate", __FILE__, __LINE__);
      return MKS_ERR_CUDA;
    }
    e->cap = cap;
  }
  MKS_CUDA(cudaGraphLaunch(e->exec, c.stream));
  MKS_CUDA(cudaStreamSynchronize(c.stream));
  capture_account(e->cap);
  return MKS_OK;
}

static int run_batch(const LinkSlot &sl, int par, int nsrc, int prec, const double *msq4, CgFields &f, Solver &S,
                     int np) {
  Context &c = ctx();
  auto issue = [&]() -> int {
    for (int k = 0; k < np; k++) MKS_TRY(cg_iteration(sl, par, nsrc, prec, msq4, f, S));
    return MKS_OK;
  };
  if (!graphs_enabled()) return issue();
  std::vector<uint64_t> key;
  key_push(key, nsrc); key_push(key, prec); key_push(key, par); key_push(key, np); key_push(key, (int)c.timing);
  key_push(key, c.geom.Vh); key_push(key, c.geom.nx); key_push(key, c.geom.ny); key_push(key, c.geom.nz);
  key_push(key, c.geom.nt);
  key_push(key, sl.fat64); key_push(key, sl.lng64); key_push(key, sl.fat32a); key_push(key, sl.lng32a);
  key_push(key, sl.fat32b); key_push(key, sl.lng32b); key_push(key, sl.fat16a); key_push(key, sl.lng16a);
  key_push(key, sl.fat16b); key_push(key, sl.lng16b); key_push(key, sl.fat16scale); key_push(key, sl.lng16scale);
  key_push(key, S.st); key_push(key, S.skip); key_push(key, c.red.partials); key_push(key, c.red.count);
  for (int s = 0; s < nsrc; s++) {
    key_push(key, msq4[s]);
    key_push(key, f.x[s]); key_push(key, f.p[s]); key_push(key, f.r[s]); key_push(key, f.ttt[s]); key_push(key, f.t[s]);
    key_push(key, f.x32[s]); key_push(key, f.p32[s]); key_push(key, f.r32[s]); key_push(key, f.ttt32[s]);
    key_push(key, f.t32[s]); key_push(key, f.p16[s]); key_push(key, f.t16[s]); key_push(key, f.p16n[s]);
    key_push(key, f.t16n[s]);
  }
  return graph_batch(key, issue);
}

// FP64 true residual r = src - (sigma - D D) x for the sources flagged
// (need[s]); xzero[s] marks sources whose x is exactly zero (D D x skipped).
static int true_residual(const LinkSlot &sl, int par, int nsrc, const double *msq4, CgFields &f, Solver &S, int setp,
                         const std::vector<int> &need, const std::vector<int> &xzero, std::vector<double> *relrsq) {
  int idx[MAXSRC], nd = 0, ndd = 0;
  double2 *xs[MAXSRC], *ts[MAXSRC], *tts[MAXSRC];
  for (int s = 0; s < nsrc; s++) {
    if (!need[s]) continue;
    idx[nd++] = s;
    if (!xzero[s]) { xs[ndd] = f.x[s]; ts[ndd] = f.t[s]; tts[ndd] = f.ttt[s]; ndd++; }
  }
  if (nd == 0) return MKS_OK;
  if (ndd > 0) MKS_TRY(apply_DD64(sl, par, ndd, xs, ts, tts));
  OpResid64 op;
  memset(&op, 0, sizeof op);
  FinResid fin;
  memset(&fin, 0, sizeof fin);
  for (int k = 0; k < nd; k++) {
    int s = idx[k];
    op.ttt[k] = f.ttt[s]; op.x[k] = f.x[s]; op.src[k] = f.src[s]; op.r[k] = f.r[s]; op.p[k] = f.p[s];
    op.msq4[k] = msq4[s]; op.map[k] = s; op.tzero[k] = xzero[s];
    fin.map[k] = s;
  }
  op.st = S.st; op.Vh = (int)ctx().Vh; op.setp = setp;
  fin.st = S.st; fin.skip = S.skip;
  double *tot;
  MKS_TRY(wsv("cg_tot2", 2 * MAXSRC, &tot));
  MKS_TRY((launch_site<OpResid64, 2, FinResid>(MKS_K_BLAS, op, fin, nullptr, nd, tot)));
  if (relrsq) {
    std::vector<double> h(2 * nd);
    Context &c = ctx();
    MKS_CUDA(cudaMemcpyAsync(h.data(), tot, 2 * nd * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    MKS_CUDA(cudaStreamSynchronize(c.stream));
    relrsq->assign(nsrc, 0.0);
    for (int k = 0; k < nd; k++) (*relrsq)[idx[k]] = sqrt(2.0 * h[2 * k + 1] / (double)c.V);
  }
  return MKS_OK;
}

// Reliable-update batching factor f (MKS_RU_JOIN, default 3; 1 = off): when
// a source of a mixed-precision block asks for its FP64 reliable update (|r|
// fell below delta * max|r|), every running source with |r| < f * delta *
// max|r| takes its update in the same FP64 launch.  Measured on GB300 (8
// sources, 32^3x64): the FP64 launches per solve fall from 42 to 20, their
// time stays the same (the FP64 D is FP64-rate bound per source), and the
// fewer host polls save 0.7 % of the solve; iteration and update counts are
// unchanged.  Only blocks whose sources share one shift take part: sources
// of one operator reach their triggers together, while the shifts of a
// multi-shift refinement do not, and joining them early adds updates (11
// offsets, 32^3x64: FP64 D 146 ms with the joins, 107 ms without).
static double ru_join() {
  static double v = -1;
  if (v < 0) {
    const char *e = getenv("MKS_RU_JOIN");
    v = e ? atof(e) : 3.0;
    if (!(v >= 1.0)) v = 1.0;
  }
  return v;
}

static int poll_interval() {
  static int v = -1;
  if (v < 0) {
    const char *e = getenv("MKS_POLL");
    v = e ? atoi(e) : 8;
    if (v < 1) v = 1;
  }
  return v;
}

// Solve (sigma_s - D_par D_opar) x_s = src_s on parity par for nsrc sources
// held in FP64 SoA device fields f.src/f.x (x = initial guess on entry);
// sigma_s = 4 m^2 for a plain mass, or a multi-shift offset when refining.
// Sources leave the block when they finish: the device state array and the
// field pointers passed to the kernels hold only the running sources
// (act[k] = original index of block position k), so a source that has
// converged costs no D_eo work while the others continue.
static int block_cg_shifted(int slot, int par, int nsrc, const double *msq4, const mks_invert_arg *arg,
                            CgFields &f, mks_invert_result *res) {
  Context &c = ctx();
  const LinkSlot &sl = c.slots[slot];
  const int prec = arg->prec;
  const bool mixed = prec != MKS_PREC_DOUBLE;
  Solver S;
  MKS_TRY(wsv("cg_state", MAXSRC, &S.st));
  MKS_TRY(wsv("cg_skip", 1, &S.skip));

  bool one_shift = true;            // every source solves the same operator
  for (int s = 1; s < nsrc; s++) one_shift = one_shift && msq4[s] == msq4[0];
  std::vector<CgState> fin(nsrc);   // final state by original index
  std::vector<int> act, xzero;      // running sources; zero initial guess by block position
  // source norms and initial-guess norms (a zero guess needs no D D x)
  {
    OpNorm<double2> op;
    memset(&op, 0, sizeof op);
    for (int s = 0; s < nsrc; s++) { op.v[s] = f.src[s]; op.v[nsrc + s] = f.x[s]; }
    op.Vh = (int)c.Vh;
    double *tot;
    MKS_TRY(wsv("cg_tot1", 2 * MAXSRC, &tot));
    MKS_TRY((launch_site<OpNorm<double2>, 1, FinNone>(MKS_K_BLAS, op, FinNone(), nullptr, 2 * nsrc, tot)));
    std::vector<double> h(2 * nsrc);
    MKS_CUDA(cudaMemcpyAsync(h.data(), tot, 2 * nsrc * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    MKS_CUDA(cudaStreamSynchronize(c.stream));
    for (int s = 0; s < nsrc; s++) {
      CgState &q = fin[s];
      memset(&q, 0, sizeof q);
      q.source_norm = h[s];
      q.rsqmin = arg->resid * arg->resid;
      q.relrsqmin = arg->relresid * arg->relresid;
      q.niter = arg->max > 0 ? arg->max : 1;
      q.max_restarts = arg->nrestart > 0 ? arg->nrestart : 1;
      q.max_cg = q.niter * q.max_restarts;
      q.mixed = mixed;
      q.delta = arg->delta > 0 ? arg->delta : 0.1;
      q.size_relr = 1.0;
      q.converged = 1;
      q.status = ST_HOST;
      if (h[s] == 0.0) {
        q.status = ST_DONE;  // trivial source: zero solution
        MKS_CUDA(cudaMemsetAsync(f.x[s], 0, 3 * c.Vh * sizeof(double2), c.stream));
      } else {
        act.push_back(s);
        xzero.push_back(h[nsrc + s] == 0.0);
      }
    }
  }
  // block view of the running sources
  CgFields g;
  double sig[MAXSRC];
  std::vector<CgState> hs;
  auto compact = [&](const std::vector<int> &keep) {
    std::vector<int> a2;
    std::vector<CgState> h2;
    for (int k : keep) { a2.push_back(act[k]); h2.push_back(hs.empty() ? fin[act[k]] : hs[k]); }
    act.swap(a2);
    hs.swap(h2);
    memset(&g, 0, sizeof g);
    for (int k = 0; k < (int)act.size(); k++) {
      const int s = act[k];
      g.src[k] = f.src[s]; g.x[k] = f.x[s]; g.r[k] = f.r[s]; g.p[k] = f.p[s]; g.ttt[k] = f.ttt[s]; g.t[k] = f.t[s];
      g.x32[k] = f.x32[s]; g.r32[k] = f.r32[s]; g.p32[k] = f.p32[s]; g.ttt32[k] = f.ttt32[s]; g.t32[k] = f.t32[s];
      g.p16[k] = f.p16[s]; g.t16[k] = f.t16[s]; g.p16n[k] = f.p16n[s]; g.t16n[k] = f.t16n[s];
      sig[k] = msq4[s];
    }
  };
  {
    std::vector<int> all(act.size());
    for (int k = 0; k < (int)all.size(); k++) all[k] = k;
    compact(all);
  }
  int nact = (int)act.size();
  if (nact > 0) MKS_TRY(write_states(S, nact, hs.data(), 1));
  if (mixed && nact > 0) {
    OpZero<float2> z;
    for (int k = 0; k < nact; k++) z.v[k] = g.x32[k];
    z.Vh = (int)c.Vh;
    MKS_TRY((launch_site<OpZero<float2>, 0, FinNone>(MKS_K_BLAS, z, FinNone(), nullptr, nact)));
  }
  bool first = true;
  int guard = 0;
  while (nact > 0) {
    MKS_TRY(read_states(S, nact, hs.data()));
    bool any_host = false, any_run = false;
    for (int k = 0; k < nact; k++) {
      any_host |= hs[k].status == ST_HOST;
      any_run |= hs[k].status == ST_RUN;
    }
    if (any_host && mixed && !first && ru_join() > 1.0 && one_shift) {
      // batch the FP64 reliable updates: a running source whose residual is
      // within a factor ru_join() of its own trigger takes its update now,
      // with the sources that asked, in one multi-source FP64 D
      bool joined = false;
      for (int k = 0; k < nact; k++) {
        CgState &q = hs[k];
        if (q.status == ST_RUN && sqrt(q.actual_rsq) < ru_join() * q.delta * q.maxrr) {
          q.status = ST_HOST;
          joined = true;
        }
      }
      if (joined) MKS_TRY(write_states(S, nact, hs.data(), 1));
    }
    if (any_host) {
      // restart (FP64 CG) or reliable update (mixed): recompute the true residual
      if (mixed && !first) {
        OpAccumX ax;
        memset(&ax, 0, sizeof ax);
        for (int k = 0; k < nact; k++) { ax.x64[k] = g.x[k]; ax.x32[k] = g.x32[k]; }
        ax.st = S.st; ax.Vh = (int)c.Vh;
        MKS_TRY((launch_site<OpAccumX, 0, FinNone>(MKS_K_BLAS, ax, FinNone(), nullptr, nact)));
      }
      std::vector<double> relrsq;
      std::vector<int> need(nact);
      for (int k = 0; k < nact; k++) need[k] = hs[k].status == ST_HOST;
      MKS_TRY(true_residual(sl, par, nact, sig, g, S, mixed ? (first ? 1 : 0) : 1, need,
                            first ? xzero : std::vector<int>(nact, 0), arg->relresid > 0 ? &relrsq : nullptr));
      if (mixed) {
        OpDemote dm;
        memset(&dm, 0, sizeof dm);
        for (int k = 0; k < nact; k++) {
          dm.r64[k] = g.r[k]; dm.r32[k] = g.r32[k]; dm.p32[k] = g.p32[k]; dm.p16[k] = g.p16[k]; dm.p16n[k] = g.p16n[k];
        }
        dm.st = S.st; dm.Vh = (int)c.Vh; dm.setp = first ? 1 : 0;
        MKS_TRY((launch_site<OpDemote, 0, FinNone>(MKS_K_BLAS, dm, FinNone(), nullptr, nact)));
      }
      MKS_TRY(read_states(S, nact, hs.data()));
      for (int k = 0; k < nact; k++) {
        CgState &q = hs[k];
        if (q.status != ST_HOST) continue;
        if (!relrsq.empty()) q.final_relrsq = relrsq[k] * relrsq[k];
        bool ok = (q.rsqmin <= 0 || q.rsqmin > q.final_rsq) &&
                  (q.relrsqmin <= 0 || q.relrsqmin > q.final_relrsq);
        if (mixed) {
          if (!first) q.reliable++;
          if (ok || q.iter >= q.max_cg || !std::isfinite(q.final_rsq)) {
            q.status = ST_DONE;
            q.converged = ok ? 1 : 0;
          } else {
            q.status = ST_RUN;
          }
        } else {
          // d_congrad5_fn_milc.c:229-241
          if (q.iter >= q.max_cg || q.nrestart >= q.max_restarts || ok || !std::isfinite(q.final_rsq)) {
            q.status = ST_DONE;
            q.converged = (q.nrestart == q.max_restarts || q.iter >= q.max_cg || !ok) ? 0 : 1;
          } else {
            q.nrestart++;
            q.status = ST_RUN;
          }
        }
      }
      first = false;
      std::vector<int> keep;
      for (int k = 0; k < nact; k++) {
        if (hs[k].status == ST_DONE) fin[act[k]] = hs[k];
        else keep.push_back(k);
      }
      if ((int)keep.size() < nact) {
        compact(keep);
        nact = (int)act.size();
      }
      any_run = nact > 0;
      if (nact > 0) MKS_TRY(write_states(S, nact, hs.data(), 0));
    }
    if (!any_run) break;
    int np = poll_interval();
    MKS_TRY(run_batch(sl, par, nact, prec, sig, g, S, np));
    if (++guard > 10000000) return MKS_ERR_TIMEOUT;
  }
  for (int k = 0; k < nact; k++) fin[act[k]] = hs[k];
  // mixed precision: x64 already holds the accumulated solution (the last
  // reliable update folded x32 in)
  for (int s = 0; s < nsrc; s++) {
    const CgState &q = fin[s];
    mks_invert_result &o = res[s];
    o.final_rsq = q.final_rsq;
    o.final_relrsq = q.final_relrsq;
    o.size_r = q.size_r;
    o.size_relr = q.size_relr;
    o.final_iters = q.iter;
    o.final_restart = q.nrestart;
    o.converged = q.converged;
    o.reliable_updates = q.reliable;
  }
  return MKS_OK;
}

static int block_cg(int slot, int par, int nsrc, double mass, const mks_invert_arg *arg, CgFields &f,
                    mks_invert_result *res) {
  double msq4[MAXSRC];
  for (int s = 0; s < nsrc; s++) msq4[s] = 4.0 * mass * mass;
  return block_cg_shifted(slot, par, nsrc, msq4, arg, f, res);
}

static int check_arg(const mks_invert_arg *arg, bool need_parity) {
  if (!arg) return MKS_ERR_ARG;
  if (arg->prec != MKS_PREC_DOUBLE && arg->prec != MKS_PREC_SINGLE && arg->prec != MKS_PREC_HALF) return MKS_ERR_ARG;
  if (need_parity && arg->parity != MKS_EVEN && arg->parity != MKS_ODD) return MKS_ERR_ARG;
  if (arg->max <= 0 || arg->nrestart <= 0) return MKS_ERR_ARG;
  return MKS_OK;
}

// dev variant core: fields already in device AoS FP64 (MILC layout)
static int congrad_block_dev(int nsrc, const double *const *src_dev, double *const *dst_dev, double mass, int slot,
                             const mks_invert_arg *arg, mks_invert_result *res) {
  int par;
  MKS_TRY(parity_index(arg->parity, &par));
  CgFields f;
  memset(&f, 0, sizeof f);
  MKS_TRY(alloc_cg_fields(f, nsrc, arg->prec));
  for (int s = 0; s < nsrc; s++) {
    MKS_TRY(vec_aos_to_soa64(src_dev[s], f.src[s], par));
    MKS_TRY(vec_aos_to_soa64(dst_dev[s], f.x[s], par));
  }
  int rc = block_cg(slot, par, nsrc, mass, arg, f, res);
  if (rc == MKS_ERR_TIMEOUT && take_tma_retry()) {
    // the staged D_eo kernel gave up and is now off: solve again from the
    // caller's initial guess (dst is written only on success)
    for (int s = 0; s < nsrc; s++) MKS_TRY(vec_aos_to_soa64(dst_dev[s], f.x[s], par));
    rc = block_cg(slot, par, nsrc, mass, arg, f, res);
  }
  MKS_TRY(rc);
  for (int s = 0; s < nsrc; s++) MKS_TRY(vec_soa64_to_aos(f.x[s], dst_dev[s], par));
  MKS_CUDA(cudaStreamSynchronize(ctx().stream));
  return MKS_OK;
}

// The device address of a page-locked host array mapped into the device
// address space (cudaHostAlloc / cudaHostRegister), else nullptr (pageable
// memory, which kernels must not touch).
// MKS_HOST_INPLACE=0 copies page-locked host fields in and out with the
// copy engines (cudaMemcpyAsync) like pageable ones, instead of reading and
// writing them in place from the layout kernels
static bool host_inplace() {
  static int v = -1;
  if (v < 0) {
    const char *e = getenv("MKS_HOST_INPLACE");
    v = e ? atoi(e) : 1;
  }
  return v != 0;
}

static double *mapped_host(const double *p) {
  if (!host_inplace()) return nullptr;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost ? (double *)at.devicePointer : nullptr;
}

// host arrays: solve in batches of MAXSRC.  A parity solve reads and writes
// only the sites of its parity, which are one contiguous half of MILC's
// even-first field: only that half moves.  Page-locked arrays are read and
// written in place by the solver's layout kernels (over the host link, no
// staging copy); pageable ones are copied in and out.
static int congrad_block_host(int nsrc, const double *const *src, double *const *dst, double mass, int slot,
                              const mks_invert_arg *arg, mks_invert_result *res) {
  Context &c = ctx();
  int par;
  MKS_TRY(parity_index(arg->parity, &par));
  const size_t off = (size_t)par * c.Vh * 6, bytes = c.Vh * 6 * sizeof(double);
  for (int b0 = 0; b0 < nsrc; b0 += MAXSRC) {
    int nb = nsrc - b0 < MAXSRC ? nsrc - b0 : MAXSRC;
    double *ds[MAXSRC], *dd[MAXSRC];
    bool staged[MAXSRC];
    for (int s = 0; s < nb; s++) {
      double *ms = mapped_host(src[b0 + s]), *md = mapped_host(dst[b0 + s]);
      staged[s] = !(ms && md);
      if (!staged[s]) {
        ds[s] = ms;
        dd[s] = md;
        continue;
      }
      MKS_TRY(wsv("hsrc" + std::to_string(s), 6 * c.V, &ds[s]));
      MKS_TRY(wsv("hdst" + std::to_string(s), 6 * c.V, &dd[s]));
      MKS_CUDA(cudaMemcpyAsync(ds[s] + off, src[b0 + s] + off, bytes, cudaMemcpyHostToDevice, c.stream));
      MKS_CUDA(cudaMemcpyAsync(dd[s] + off, dst[b0 + s] + off, bytes, cudaMemcpyHostToDevice, c.stream));
    }
    MKS_TRY(congrad_block_dev(nb, ds, dd, mass, slot, arg, res + b0));
    for (int s = 0; s < nb; s++)
      if (staged[s])
        MKS_CUDA(cudaMemcpyAsync(dst[b0 + s] + off, dd[s] + off, bytes, cudaMemcpyDeviceToHost, c.stream));
    MKS_CUDA(cudaStreamSynchronize(c.stream));
  }
  return MKS_OK;
}

static int max_iters(int nsrc, const mks_invert_result *res) {
  int m = 0;
  for (int s = 0; s < nsrc; s++) m = res[s].final_iters > m ? res[s].final_iters : m;
  return m;
}

}  // namespace mks

extern "C" {

int mks_ks_congrad_parity_dev(const double *src_dev, double *dst_dev, double mass, int slot,
                              const mks_invert_arg *arg, mks_invert_result *res) {
  MKS_TRY(check_ready());
  MKS_TRY(slot_ok(slot));
  MKS_TRY(check_arg(arg, true));
  if (!src_dev || !dst_dev || !res) return MKS_ERR_ARG;
  MKS_TRY(congrad_block_dev(1, &src_dev, &dst_dev, mass, slot, arg, res));
  return res[0].final_iters;
}

int mks_ks_congrad_parity(const double *src, double *dst, double mass, int slot, const mks_invert_arg *arg,
                          mks_invert_result *res) {
  MKS_TRY(check_ready());
  MKS_TRY(slot_ok(slot));
  MKS_TRY(check_arg(arg, true));
  if (!src || !dst || !res) return MKS_ERR_ARG;
  MKS_TRY(congrad_block_host(1, &src, &dst, mass, slot, arg, res));
  return res[0].final_iters;
}

int mks_ks_congrad_block_parity_dev(int nsrc, const double *const *src_dev, double *const *dst_dev, double mass,
                                    int slot, const mks_invert_arg *arg, mks_invert_result *res) {
  MKS_TRY(check_ready());
  MKS_TRY(slot_ok(slot));
  MKS_TRY(check_arg(arg, true));
  if (nsrc <= 0 || nsrc > MAXSRC || !src_dev || !dst_dev || !res) return MKS_ERR_ARG;
  MKS_TRY(congrad_block_dev(nsrc, src_dev, dst_dev, mass, slot, arg, res));
  return max_iters(nsrc, res);
}

int mks_ks_congrad_block_parity(int nsrc, const double *const *src, double *const *dst, double mass, int slot,
                                const mks_invert_arg *arg, mks_invert_result *res) {
  MKS_TRY(check_ready());
  MKS_TRY(slot_ok(slot));
  MKS_TRY(check_arg(arg, true));
  if (nsrc <= 0 || !src || !dst || !res) return MKS_ERR_ARG;
  MKS_TRY(congrad_block_host(nsrc, src, dst, mass, slot, arg, res));
  return max_iters(nsrc, res);
}

}  // extern "C"

namespace mks {

// out = alpha*a + beta*b (FP64, one parity, per source)
struct OpLin64 {
  double2 *out[BLAS_MAXSRC], *a[BLAS_MAXSRC], *b[BLAS_MAXSRC];
  double alpha, beta;
  int Vh;
  __device__ void operator()(int h, int s, double *) const {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      size_t i = (size_t)k * Vh + h;
      double2 x = a[s][i], y = b[s][i];
      out[s][i] = make_double2(alpha * x.x + beta * y.x, alpha * x.y + beta * y.y);
    }
  }
};

static int lin64(int nsrc, double2 *const *out, double alpha, double2 *const *a, double beta, double2 *const *b) {
  OpLin64 op;
  memset(&op, 0, sizeof op);
  for (int s = 0; s < nsrc; s++) { op.out[s] = out[s]; op.a[s] = a[s]; op.b[s] = b[s]; }
  op.alpha = alpha; op.beta = beta; op.Vh = (int)ctx().Vh;
  return launch_site<OpLin64, 0, FinNone>(MKS_K_BLAS, op, FinNone(), nullptr, nsrc);
}

// M^{-1} for nsrc sources given device AoS fields (generic_ks/mat_invert.c:328-483):
//   tmp = M^dag src = 2m src - D src; even CG on tmp; dst_o = (src_o - D_oe dst_e)/(2m);
//   odd CG on tmp (polish).
static int mat_invert_dev(int nsrc, const double *const *src_dev, double *const *dst_dev, double mass, int slot,
                          const mks_invert_arg *arg, mks_invert_result *res) {
  Context &c = ctx();
  const LinkSlot &sl = c.slots[slot];
  CgFields f;
  memset(&f, 0, sizeof f);
  MKS_TRY(alloc_cg_fields(f, nsrc, arg->prec));
  double2 *se[MAXSRC], *so[MAXSRC], *te[MAXSRC], *to[MAXSRC], *de[MAXSRC], *dn[MAXSRC];
  size_t n = 3 * c.Vh;
  for (int s = 0; s < nsrc; s++) {
    std::string k = std::to_string(s);
    MKS_TRY(wsv("mi_se" + k, n, &se[s])); MKS_TRY(wsv("mi_so" + k, n, &so[s]));
    MKS_TRY(wsv("mi_te" + k, n, &te[s])); MKS_TRY(wsv("mi_to" + k, n, &to[s]));
    MKS_TRY(wsv("mi_de" + k, n, &de[s])); MKS_TRY(wsv("mi_dn" + k, n, &dn[s]));
    MKS_TRY(vec_aos_to_soa64(src_dev[s], se[s], 0));
    MKS_TRY(vec_aos_to_soa64(src_dev[s], so[s], 1));
    MKS_TRY(vec_aos_to_soa64(dst_dev[s], f.x[s], 0));
  }
  // tmp_e = 2m src_e - D src_o ; tmp_o = 2m src_o - D src_e
  MKS_TRY(dslash64(sl, 0, nsrc, so, de));
  MKS_TRY(dslash64(sl, 1, nsrc, se, dn));
  MKS_TRY(lin64(nsrc, te, 2.0 * mass, se, -1.0, de));
  MKS_TRY(lin64(nsrc, to, 2.0 * mass, so, -1.0, dn));
  // even solve
  mks_invert_arg a = *arg;
  a.parity = MKS_EVEN;
  for (int s = 0; s < nsrc; s++)
    MKS_CUDA(cudaMemcpyAsync(f.src[s], te[s], n * sizeof(double2), cudaMemcpyDeviceToDevice, c.stream));
  std::vector<mks_invert_result> r_even(nsrc);
  MKS_TRY(block_cg(slot, 0, nsrc, mass, &a, f, r_even.data()));
  // odd reconstruction: dst_o = (src_o - D_oe dst_e) / (2m)
  for (int s = 0; s < nsrc; s++)
    MKS_CUDA(cudaMemcpyAsync(de[s], f.x[s], n * sizeof(double2), cudaMemcpyDeviceToDevice, c.stream));
  MKS_TRY(dslash64(sl, 1, nsrc, de, dn));
  MKS_TRY(lin64(nsrc, f.x, 1.0 / (2.0 * mass), so, -1.0 / (2.0 * mass), dn));
  // odd polish
  a.parity = MKS_ODD;
  for (int s = 0; s < nsrc; s++)
    MKS_CUDA(cudaMemcpyAsync(f.src[s], to[s], n * sizeof(double2), cudaMemcpyDeviceToDevice, c.stream));
  MKS_TRY(block_cg(slot, 1, nsrc, mass, &a, f, res));
  for (int s = 0; s < nsrc; s++) {
    res[s].final_iters += r_even[s].final_iters;
    MKS_TRY(vec_soa64_to_aos(de[s], dst_dev[s], 0));
    MKS_TRY(vec_soa64_to_aos(f.x[s], dst_dev[s], 1));
  }
  MKS_CUDA(cudaStreamSynchronize(c.stream));
  return MKS_OK;
}

static int mat_invert_host(int nsrc, const double *const *src, double *const *dst, double mass, int slot,
                           const mks_invert_arg *arg, mks_invert_result *res) {
  Context &c = ctx();
  size_t bytes = c.V * 6 * sizeof(double);
  for (int b0 = 0; b0 < nsrc; b0 += MAXSRC) {
    int nb = nsrc - b0 < MAXSRC ? nsrc - b0 : MAXSRC;
    double *ds[MAXSRC], *dd[MAXSRC];
    for (int s = 0; s < nb; s++) {
      MKS_TRY(wsv("hsrc" + std::to_string(s), 6 * c.V, &ds[s]));
      MKS_TRY(wsv("hdst" + std::to_string(s), 6 * c.V, &dd[s]));
      MKS_CUDA(cudaMemcpyAsync(ds[s], src[b0 + s], bytes, cudaMemcpyHostToDevice, c.stream));
      MKS_CUDA(cudaMemcpyAsync(dd[s], dst[b0 + s], bytes, cudaMemcpyHostToDevice, c.stream));
    }
    MKS_TRY(mat_invert_dev(nb, ds, dd, mass, slot, arg, res + b0));
    for (int s = 0; s < nb; s++) MKS_CUDA(cudaMemcpyAsync(dst[b0 + s], dd[s], bytes, cudaMemcpyDeviceToHost, c.stream));
    MKS_CUDA(cudaStreamSynchronize(c.stream));
  }
  return MKS_OK;
}

}  // namespace mks

extern "C" {

int mks_mat_invert_uml_field(const double *src, double *dst, double mass, int slot, const mks_invert_arg *arg,
                             mks_invert_result *res) {
  MKS_TRY(check_ready());
  MKS_TRY(slot_ok(slot));
  MKS_TRY(check_arg(arg, false));
  if (!src || !dst || !res || mass == 0.0) return MKS_ERR_ARG;
  MKS_TRY(mat_invert_host(1, &src, &dst, mass, slot, arg, res));
  return res[0].final_iters;
}

int mks_mat_invert_block_uml(int nsrc, const double *const *src, double *const *dst, double mass, int slot,
                             const mks_invert_arg *arg, mks_invert_result *res) {
  MKS_TRY(check_ready());
  MKS_TRY(slot_ok(slot));
  MKS_TRY(check_arg(arg, false));
  if (nsrc <= 0 || !src || !dst || !res || mass == 0.0) return MKS_ERR_ARG;
  MKS_TRY(mat_invert_host(nsrc, src, dst, mass, slot, arg, res));
  return max_iters(nsrc, res);
}

}  // extern "C"

namespace mks {

// deterministic pseudo-random fill for benchmark inputs
__global__ void k_fill_bench(float2 *v, size_t n, unsigned seed) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    unsigned a = (unsigned)i * 2654435761u ^ seed, b = a * 1664525u + 1013904223u;
    v[i] = make_float2((a >> 8) * (1.0f / 16777216.0f) - 0.5f, (b >> 8) * (1.0f / 16777216.0f) - 0.5f);
  }
}
__global__ void k_f32_to_f64(const float2 *a, double2 *b, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    b[i] = make_double2(a[i].x, a[i].y);
}
__global__ void k_f32_to_f16(const float2 *a, __half2 *b, float *nrm, int Vh) {
  int h = blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= Vh) return;
  float m = 0.f;
  for (int c = 0; c < 3; c++) m = fmaxf(m, fmaxf(fabsf(a[(size_t)c * Vh + h].x), fabsf(a[(size_t)c * Vh + h].y)));
  float inv = m > 0 ? 1.f / m : 0.f;
  nrm[h] = m;
  for (int c = 0; c < 3; c++) b[(size_t)c * Vh + h] = __floats2half2_rn(a[(size_t)c * Vh + h].x * inv, a[(size_t)c * Vh + h].y * inv);
}
__global__ void k_flush(float4 *buf, size_t n, float v) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    buf[i] = make_float4(v, v, v, v);
}

}  // namespace mks

extern "C" int mks_bench_dslash(int prec, int nsrc, int parity, int slot, int iters, int flush_l2, double *ms) {
  MKS_TRY(check_ready());
  MKS_TRY(slot_ok(slot));
  if (nsrc < 1 || nsrc > MAXSRC || iters < 1 || !ms) return MKS_ERR_ARG;
  int par;
  MKS_TRY(parity_index(parity, &par));
  Context &c = ctx();
  const LinkSlot &sl = c.slots[slot];
  size_t n = 3 * c.Vh;
  float2 *in32[MAXSRC], *out32[MAXSRC];
  double2 *in64[MAXSRC], *out64[MAXSRC];
  __half2 *in16[MAXSRC];
  float *in16n[MAXSRC];
  for (int s = 0; s < nsrc; s++) {
    std::string k = std::to_string(s);
    MKS_TRY(wsv("bd_in32" + k, n, &in32[s]));
    MKS_TRY(wsv("bd_out32" + k, n, &out32[s]));
    k_fill_bench<<<c.sm_count * 4, 256, 0, c.stream>>>(in32[s], n, 1234u + s);
    if (prec == MKS_PREC_DOUBLE) {
      MKS_TRY(wsv("bd_in64" + k, n, &in64[s]));
      MKS_TRY(wsv("bd_out64" + k, n, &out64[s]));
      k_f32_to_f64<<<c.sm_count * 4, 256, 0, c.stream>>>(in32[s], in64[s], n);
    } else if (prec == MKS_PREC_HALF) {
      MKS_TRY(wsv("bd_in16" + k, n, &in16[s]));
      MKS_TRY(wsv("bd_in16n" + k, c.Vh, &in16n[s]));
      k_f32_to_f16<<<grid_for(c.Vh, 256), 256, 0, c.stream>>>(in32[s], in16[s], in16n[s], (int)c.Vh);
    }
  }
  float4 *flush = nullptr;
  size_t nflush = (size_t)256 << 20;  // bytes
  if (flush_l2) MKS_TRY(wsv("bd_flush", nflush / sizeof(float4), &flush));
  MKS_CUDA(cudaGetLastError());
  cudaEvent_t e0, e1;
  MKS_CUDA(cudaEventCreate(&e0));
  MKS_CUDA(cudaEventCreate(&e1));
  double total = 0;
  for (int it = 0; it < iters + 1; it++) {  // first launch is a warm-up
    if (flush) k_flush<<<c.sm_count * 4, 256, 0, c.stream>>>(flush, nflush / sizeof(float4), (float)it);
    MKS_CUDA(cudaEventRecord(e0, c.stream));
    if (prec == MKS_PREC_DOUBLE) {
      MKS_TRY(dslash64(sl, par, nsrc, in64, out64));
    } else if (prec == MKS_PREC_SINGLE) {
      DslashArgs<VecF32, VecF32, VecF32> a;
      memset(&a, 0, sizeof a);
      a.out_par = par; a.nsrc = nsrc;
      for (int s = 0; s < nsrc; s++) { a.in[s].p = in32[s]; a.out[s].p = out32[s]; }
      LinkSet32 L = links32(sl);
      MKS_TRY((launch_dslash<float, LinkF32, VecF32, VecF32, EPI_PLAIN, 0>(MKS_K_DSLASH_F32, L.fat, L.lng, a, FinNone())));
    } else {
      DslashArgs<VecF16, VecF32, VecF32> a;
      memset(&a, 0, sizeof a);
      a.out_par = par; a.nsrc = nsrc;
      for (int s = 0; s < nsrc; s++) { a.in[s].p = in16[s]; a.in[s].norm = in16n[s]; a.out[s].p = out32[s]; }
      LinkSet16 L = links16(sl);
      MKS_TRY((launch_dslash<float, LinkF16, VecF16, VecF32, EPI_PLAIN, 0>(MKS_K_DSLASH_F16, L.fat, L.lng, a, FinNone())));
    }
    MKS_CUDA(cudaEventRecord(e1, c.stream));
    MKS_CUDA(cudaEventSynchronize(e1));
    float t = 0;
    MKS_CUDA(cudaEventElapsedTime(&t, e0, e1));
    if (it > 0) total += t;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = total / iters;
  return MKS_OK;
}

// ====================================================================
// Multi-shift CG (generic_ks/ks_multicg_offset.c:63-505).
// Per iteration: K1 t = D_oe p; K2 ttt = D_eo t + shift0 p with
// pkp, <ttt,r>, |ttt|^2 and, in its last block, every shift's zeta/beta/
// alpha recurrence; K3 one pass over all shifts: psim_j += beta_j pm_j,
// r += beta ttt, pm_j = zeta_j r + alpha_j pm_j, p = pm_low, and the true
// |r|^2 that decides convergence.  alpha uses |r_new|^2 expanded from the
// K2 sums (the FEWSUMS device of d_congrad5_fn_milc.c:296-312), so the
// shift updates need only the one pass.
namespace mks {

constexpr int MAXSH = 32;

struct MsState {
  double rsq, pkp, source_norm, rsqstop, shift0;
  double shifts[MAXSH], zeta_i[MAXSH], zeta_im1[MAXSH], zeta_ip1[MAXSH];
  double beta_i[MAXSH], beta_im1[MAXSH], alpha[MAXSH];
  double maxrr, delta;   // reliable updates of the sloppy solve: max |r| since the last one, threshold
  double rsqretire;      // sloppy solve: a shift whose |zeta_j r|^2 fell below this is no longer updated
  int iter, niter, status, j_low, num_now, num_offsets, need_scroll, want_reliable;
  int n_reliable;
  int check_true;        // sloppy solve: stop only when the lowest shift's FP64 residual meets the target
  int retired[MAXSH];
  long long shift_updates;  // sum over iterations of the shifts the update kernel advanced
};

// the zeta / beta / alpha recurrences of one field after K2 (t: its three sums)
__device__ __forceinline__ void ms_alpha(MsState &m, const double *t) {
    if (m.status != ST_RUN) return;
    if (m.need_scroll) {
      for (int j = 0; j < m.num_now; j++) {
        m.beta_im1[j] = m.beta_i[j];
        m.zeta_im1[j] = m.zeta_i[j];
        m.zeta_i[j] = m.zeta_ip1[j];
      }
      m.need_scroll = 0;
    }
    const int jl = m.j_low;
    double pkp = t[0], c_tr = t[1], c_tt = t[2];
    m.pkp = pkp;
    m.iter++;
    m.beta_i[jl] = -m.rsq / pkp;
    m.zeta_ip1[jl] = 1.0;
    for (int j = 0; j < m.num_now; j++) {
      if (j == jl) continue;
      m.zeta_ip1[j] = m.zeta_i[j] * m.zeta_im1[j] * m.beta_im1[jl];
      double c1 = m.beta_i[jl] * m.alpha[jl] * (m.zeta_im1[j] - m.zeta_i[j]);
      double c2 = m.zeta_im1[j] * m.beta_im1[jl] * (1.0 + m.shifts[j] * m.beta_i[jl]);
      if (c1 + c2 != 0.0) m.zeta_ip1[j] /= c1 + c2;
      else m.zeta_ip1[j] = 0.0;
      if (m.zeta_i[j] != 0.0) {
        m.beta_i[j] = m.beta_i[jl] * m.zeta_ip1[j] / m.zeta_i[j];
      } else {
        m.zeta_ip1[j] = 0.0;
        m.beta_i[j] = 0.0;
        if (j == m.num_now - 1 && j > jl) m.num_now--;
      }
    }
    // |r + beta ttt|^2 from the K2 sums
    double b = m.beta_i[jl];
    double rsq_new = m.rsq + 2.0 * b * c_tr + b * b * c_tt;
    m.alpha[jl] = rsq_new / m.rsq;
    for (int j = 0; j < m.num_now; j++) {
      if (j == jl) continue;
      if (m.zeta_i[j] * m.beta_i[jl] != 0.0)
        m.alpha[j] = m.alpha[jl] * m.zeta_ip1[j] * m.beta_i[j] / (m.zeta_i[j] * m.beta_i[jl]);
      else
        m.alpha[j] = 0.0;
    }
    if (!isfinite(m.beta_i[jl])) m.status = ST_HOST;
    // the update kernel of this iteration advances every shift not retired
    for (int j = 0; j < m.num_now; j++) m.shift_updates += m.retired[j] ? 0 : 1;
}

struct FinMsAlpha {
  MsState *st;
  __device__ void operator()(const double *t, int) const {
    if (threadIdx.x != 0) return;
    ms_alpha(*st, t);
  }
};

// the state of one field after K3 (rsq: the new |r|^2): retirement of
// converged shifts, stop, reliable-update request
__device__ __forceinline__ void ms_update(MsState &m, double rsq) {
    if (m.status == ST_RUN) {
      m.rsq = rsq;
      m.need_scroll = 1;
      if (m.rsqretire > 0)
        for (int j = 0; j < m.num_now; j++)
          if (j != m.j_low && m.zeta_ip1[j] * m.zeta_ip1[j] * m.rsq < m.rsqretire) m.retired[j] = 1;
      if ((m.rsqstop > 0 && m.rsq <= m.rsqstop) || m.iter >= m.niter || !isfinite(m.rsq)) {
        m.status = ST_HOST;
        // the sloppy recursion met the target: the host recomputes the
        // lowest shift's residual in FP64 and goes on unless that meets it
        if (m.check_true && m.delta > 0 && m.iter < m.niter && isfinite(m.rsq)) m.want_reliable = 1;
      } else if (m.delta > 0) {
        // sloppy solve: ask for a reliable update when |r| fell below
        // delta * max|r| since the last one
        double rn = sqrt(m.rsq);
        if (rn > m.maxrr) m.maxrr = rn;
        if (rn < m.delta * m.maxrr) { m.status = ST_HOST; m.want_reliable = 1; }
      }
    }
}

struct FinMsUpdate {
  MsState *st;
  int *skip;
  __device__ void operator()(const double *t, int) const {
    if (threadIdx.x != 0) return;
    ms_update(*st, t[0]);
    *skip = (st->status != ST_RUN);
  }
};

// several fields in one multi-shift (one per row k, field map[k])
constexpr int MSF = 4;
struct FinMsAlphaM {
  MsState *st;
  int map[MSF];
  __device__ void operator()(const double *t, int n) const {
    const int k = threadIdx.x;
    if (k < n) ms_alpha(st[map[k]], t + 3 * k);
  }
};
struct FinMsUpdateM {
  MsState *st;
  int *skip;
  int map[MSF];
  __device__ void operator()(const double *t, int n) const {
    const int k = threadIdx.x;
    if (k < n) ms_update(st[map[k]], t[k]);
    __syncthreads();
    if (threadIdx.x == 0) {
      int any = 0;
      for (int i = 0; i < n; i++) any |= (st[map[i]].status != ST_RUN);
      *skip = any;
    }
  }
};

// K3 at one site for one field: r += beta ttt, every shift's psim and pm,
// the lowest shift's p (and its FP16 shadow); out[0] = |r|^2 at the site
template <typename R, typename RS = R>
__device__ __forceinline__ void ms_site_update(const MsState &m, typename VT<RS>::v2 *const *psim,
                                               typename VT<RS>::v2 *const *pm, typename VT<R>::v2 *r,
                                               const typename VT<R>::v2 *ttt, typename VT<R>::v2 *cgp,
                                               __half2 *p16, float *p16n, int h, int Vh, double *out) {
    typedef typename VT<R>::v2 T2;
    typedef typename VT<RS>::v2 S2;
    const int n = m.num_now, jl = m.j_low;
    const R bl = (R)m.beta_i[jl];
    T2 rn[3];
    R rr = 0;  // per-site sum in the storage precision
#pragma unroll
    for (int k = 0; k < 3; k++) {
      size_t i = (size_t)k * Vh + h;
      T2 rv = r[i], tv = ttt[i];
      rv.x = rv.x + bl * tv.x; rv.y = rv.y + bl * tv.y;
      rn[k] = rv;
      r[i] = rv;
      rr += rv.x * rv.x + rv.y * rv.y;
    }
    for (int j = 0; j < n; j++) {
      if (m.retired[j]) continue;
      const RS bj = (RS)m.beta_i[j], zj = (RS)m.zeta_ip1[j], aj = (RS)m.alpha[j];
#pragma unroll
      for (int k = 0; k < 3; k++) {
        size_t i = (size_t)k * Vh + h;
        S2 pv = pm[j][i], xv = psim[j][i];
        xv.x = xv.x + bj * pv.x; xv.y = xv.y + bj * pv.y;
        pv.x = zj * (RS)rn[k].x + aj * pv.x; pv.y = zj * (RS)rn[k].y + aj * pv.y;
        psim[j][i] = xv;
        pm[j][i] = pv;
        if (j == jl) { T2 cv; cv.x = (R)pv.x; cv.y = (R)pv.y; cgp[i] = cv; }
      }
      if (j == jl && p16) {
        float mx = 0.f;
#pragma unroll
        for (int k = 0; k < 3; k++) {
          S2 pv = pm[j][(size_t)k * Vh + h];
          mx = fmaxf(mx, fmaxf(fabsf((float)pv.x), fabsf((float)pv.y)));
        }
        float inv = mx > 0.f ? 1.f / mx : 0.f;
        p16n[h] = mx;
#pragma unroll
        for (int k = 0; k < 3; k++) {
          S2 pv = pm[j][(size_t)k * Vh + h];
          p16[(size_t)k * Vh + h] = __floats2half2_rn((float)pv.x * inv, (float)pv.y * inv);
        }
      }
    }
    out[0] = rr;
}

template <typename R, typename RS = R> struct OpShiftUpdate {
  typedef typename VT<R>::v2 T2;
  typedef typename VT<RS>::v2 S2;
  S2 *psim[MAXSH], *pm[MAXSH];
  T2 *r, *ttt, *cgp;
  __half2 *p16;
  float *p16n;
  const MsState *st;
  int Vh;
  __device__ void operator()(int h, int, double *out) const {
    ms_site_update<R, RS>(*st, psim, pm, r, ttt, cgp, p16, p16n, h, Vh, out);
  }
};

// the same for several fields, one per row k (field map[k])
template <typename R, typename RS = R> struct OpShiftUpdateM {
  typedef typename VT<R>::v2 T2;
  typedef typename VT<RS>::v2 S2;
  S2 *psim[MSF][MAXSH], *pm[MSF][MAXSH];
  T2 *r[MSF], *ttt[MSF], *cgp[MSF];
  const MsState *st;
  int map[MSF];
  int Vh;
  __device__ void operator()(int h, int k, double *out) const {
    const int f = map[k];
    ms_site_update<R, RS>(st[f], psim[f], pm[f], r[f], ttt[f], cgp[f], nullptr, nullptr, h, Vh, out);
  }
};

// initial fields: r = p = pm_j = src (converted), psim_j = 0
template <typename R, typename RS = R> struct OpShiftInit {
  typedef typename VT<R>::v2 T2;
  typedef typename VT<RS>::v2 S2;
  S2 *psim[MAXSH], *pm[MAXSH];
  T2 *r, *cgp;
  const double2 *src;
  __half2 *p16;
  float *p16n;
  int Vh, n;
  __device__ void operator()(int h, int, double *out) const {
    double a = 0;
    float mx = 0.f;
    T2 v[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      size_t i = (size_t)k * Vh + h;
      double2 sv = src[i];
      v[k].x = (R)sv.x; v[k].y = (R)sv.y;
      r[i] = v[k]; cgp[i] = v[k];
      a += sv.x * sv.x + sv.y * sv.y;
      mx = fmaxf(mx, fmaxf(fabsf((float)sv.x), fabsf((float)sv.y)));
      for (int j = 0; j < n; j++) {
        S2 pv; pv.x = (RS)sv.x; pv.y = (RS)sv.y;
        pm[j][i] = pv;
        S2 z; z.x = 0; z.y = 0;
        psim[j][i] = z;
      }
    }
    if (p16) {
      float inv = mx > 0.f ? 1.f / mx : 0.f;
      p16n[h] = mx;
#pragma unroll
      for (int k = 0; k < 3; k++) p16[(size_t)k * Vh + h] = __floats2half2_rn((float)v[k].x * inv, (float)v[k].y * inv);
    }
    out[0] = a;
  }
};

// reliable update of the sloppy multi-shift solve, per shift:
// x64_j += x32_j ; x32_j = 0
struct OpMsFold {
  double2 *x64[BLAS_MAXSRC];
  float2 *x32[BLAS_MAXSRC];
  int Vh;
  __device__ void operator()(int h, int s, double *) const {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      size_t i = (size_t)k * Vh + h;
      double2 a = x64[s][i];
      float2 b = x32[s][i];
      x64[s][i] = make_double2(a.x + (double)b.x, a.y + (double)b.y);
      x32[s][i] = make_float2(0.f, 0.f);
    }
  }
};

// FP64 residual of the lowest shift, r = src - (sigma - D D) x with
// ddx = D D x, stored into the sloppy r; |r|^2 in FP64
struct OpMsResid {
  const double2 *src, *ddx, *x;
  float2 *r32;
  double sigma;
  int Vh;
  __device__ void operator()(int h, int, double *out) const {
    double a = 0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      size_t i = (size_t)k * Vh + h;
      double2 sv = src[i], dv = ddx[i], xv = x[i];
      double2 rv = make_double2(sv.x + (dv.x - sigma * xv.x), sv.y + (dv.y - sigma * xv.y));
      r32[i] = make_float2((float)rv.x, (float)rv.y);
      a += rv.x * rv.x + rv.y * rv.y;
    }
    out[0] = a;
  }
};

// x64_j += x32_j for every shift (FP32 sloppy solutions folded into FP64)
static int ms_fold(int nsh, double2 *const *x64, void *const *x32) {
  for (int b0 = 0; b0 < nsh; b0 += BLAS_MAXSRC) {
    int nb = nsh - b0 < BLAS_MAXSRC ? nsh - b0 : BLAS_MAXSRC;
    OpMsFold op;
    memset(&op, 0, sizeof op);
    for (int s = 0; s < nb; s++) { op.x64[s] = x64[b0 + s]; op.x32[s] = (float2 *)x32[b0 + s]; }
    op.Vh = (int)ctx().Vh;
    MKS_TRY((launch_site<OpMsFold, 0, FinNone>(MKS_K_BLAS, op, FinNone(), nullptr, nb)));
  }
  return MKS_OK;
}

// sloppy (or FP64) multi-shift iterations; R selects vector storage precision.
// With x64 given (sloppy storage only), the solve makes reliable updates:
// when |r| fell below delta times its maximum since the last update, every
// shift's FP32 solution is folded into its FP64 accumulator x64_j and the
// residual of the lowest shift is recomputed in FP64 from x64_low and
// replaces the sloppy one (the shifted residuals stay zeta_j r); on exit
// x64_j holds the whole solution.
// RS: storage of the shifts' solutions and search directions.  RS = double
// with R = float keeps p_j and x_j in FP64 (the solutions are then the x64
// accumulators themselves, no fold): the shifted residuals zeta_j r stay
// consistent with the shifts' solutions, which FP32 p_j and x_j lose to
// rounding that the lowest shift's reliable updates do not repair.
template <typename R, typename RS = R>
static int multishift_core(const LinkSlot &sl, int par, int prec, const double2 *src64, int nsh,
                           const double *offsets, double resid, int niter, void **psim_out, MsState *hstate,
                           double2 *const *x64 = nullptr, double delta = 0.0) {
  typedef typename VT<R>::v2 T2;
  typedef typename VT<RS>::v2 S2;
  constexpr bool wide = !std::is_same<R, RS>::value;
  Context &c = ctx();
  const int Vh = (int)c.Vh;
  size_t n = 3 * c.Vh;
  T2 *r, *cgp, *ttt, *t;
  S2 *pm[MAXSH], *psim[MAXSH];
  const char *tag = sizeof(R) == 8 ? "64" : "32";
  const char *stag = sizeof(RS) == 8 ? "64" : "32";
  MKS_TRY(wsv(std::string("ms_r") + tag, n, &r));
  MKS_TRY(wsv(std::string("ms_p") + tag, n, &cgp));
  MKS_TRY(wsv(std::string("ms_ttt") + tag, n, &ttt));
  MKS_TRY(wsv(std::string("ms_t") + tag, n, &t));
  for (int j = 0; j < nsh; j++) {
    MKS_TRY(wsv(std::string("ms_pm") + stag + "_" + std::to_string(j), n, &pm[j]));
    if (wide && x64) psim[j] = (S2 *)x64[j];
    else MKS_TRY(wsv(std::string("ms_x") + stag + "_" + std::to_string(j), n, &psim[j]));
    psim_out[j] = psim[j];
  }
  __half2 *p16 = nullptr, *t16 = nullptr;
  float *p16n = nullptr, *t16n = nullptr;
  if (prec == MKS_PREC_HALF) {
    MKS_TRY(wsv("ms_p16", n, &p16)); MKS_TRY(wsv("ms_t16", n, &t16));
    MKS_TRY(wsv("ms_p16n", c.Vh, &p16n)); MKS_TRY(wsv("ms_t16n", c.Vh, &t16n));
  }
  MsState *st;
  int *skip;
  MKS_TRY(wsv("ms_state", 1, &st));
  MKS_TRY(wsv("ms_skip", 1, &skip));
  // initial state (ks_multicg_offset.c:180-262)
  MsState h;
  memset(&h, 0, sizeof h);
  double offset_low = 1.0e20;
  int j_low = -1;
  for (int j = 0; j < nsh; j++) {
    h.shifts[j] = offsets[j];
    if (offsets[j] < offset_low) { offset_low = offsets[j]; j_low = j; }
  }
  for (int j = 0; j < nsh; j++)
    if (j != j_low) h.shifts[j] -= h.shifts[j_low];
  h.shift0 = -h.shifts[j_low];
  h.j_low = j_low; h.num_now = nsh; h.num_offsets = nsh; h.niter = niter;
  for (int j = 0; j < nsh; j++) { h.zeta_im1[j] = h.zeta_i[j] = 1.0; h.beta_im1[j] = -1.0; h.alpha[j] = 0.0; }
  {
    OpShiftInit<R, RS> op;
    memset(&op, 0, sizeof op);
    for (int j = 0; j < nsh; j++) { op.psim[j] = psim[j]; op.pm[j] = pm[j]; }
    op.r = r; op.cgp = cgp; op.src = src64; op.p16 = p16; op.p16n = p16n; op.Vh = Vh; op.n = nsh;
    double *tot;
    MKS_TRY(wsv("ms_tot", 4, &tot));
    MKS_TRY((launch_site<OpShiftInit<R, RS>, 1, FinNone>(MKS_K_BLAS, op, FinNone(), nullptr, 1, tot)));
    double sn = 0;
    MKS_CUDA(cudaMemcpyAsync(&sn, tot, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    MKS_CUDA(cudaStreamSynchronize(c.stream));
    h.source_norm = sn;
    h.rsq = sn;
    h.rsqstop = resid * resid * sn;
    h.iter = 1;
    h.status = sn == 0.0 ? ST_DONE : ST_RUN;
    h.maxrr = sqrt(sn);
    h.delta = (x64 && sizeof(R) == 4) ? delta : 0.0;
    // sloppy solve: stop updating a shift once its iterated residual is a
    // decade below the target (its true residual is checked afterwards)
    h.rsqretire = h.delta > 0 ? 0.01 * h.rsqstop : 0.0;
    h.check_true = h.delta > 0 && ms_true_stop();
  }
  if (h.delta > 0 && !wide)
    for (int j = 0; j < nsh; j++) MKS_CUDA(cudaMemsetAsync(x64[j], 0, n * sizeof(double2), c.stream));
  MKS_CUDA(cudaMemcpyAsync(st, &h, sizeof h, cudaMemcpyHostToDevice, c.stream));
  int zero = 0;
  MKS_CUDA(cudaMemcpyAsync(skip, &zero, sizeof zero, cudaMemcpyHostToDevice, c.stream));
  double *tot;
  MKS_TRY(wsv("ms_tot3", 4, &tot));
  int guard = 0;
  const int np = poll_interval();
  // one batch of np iterations (3 launches each), replayed as a CUDA graph
  auto issue = [&]() -> int {
    for (int k = 0; k < np; k++) {
      if (prec == MKS_PREC_DOUBLE) {
        LinkSet64 L = links64(sl);
        DslashArgs<VecF64, VecF64, VecF64> a1;
        memset(&a1, 0, sizeof a1);
        a1.out_par = 1 - par; a1.nsrc = 1; a1.skip = skip;
        a1.in[0].p = (double2 *)cgp; a1.out[0].p = (double2 *)t;
        MKS_TRY((launch_dslash<double, LinkF64, VecF64, VecF64, EPI_PLAIN, 0>(MKS_K_DSLASH_F64, L.fat, L.lng, a1, FinNone())));
        DslashArgs<VecF64, VecF64, VecF64> a2;
        memset(&a2, 0, sizeof a2);
        a2.out_par = par; a2.nsrc = 1; a2.skip = skip; a2.totals = tot;
        a2.in[0].p = (double2 *)t; a2.out[0].p = (double2 *)ttt; a2.p[0].p = (double2 *)cgp; a2.r[0].p = (double2 *)r;
        a2.coef[0] = h.shift0;
        MKS_TRY((launch_dslash<double, LinkF64, VecF64, VecF64, EPI_AXPY, 3>(MKS_K_DSLASH_F64, L.fat, L.lng, a2, FinMsAlpha{st})));
      } else if (prec == MKS_PREC_SINGLE) {
        LinkSet32 L = links32(sl);
        DslashArgs<VecF32, VecF32, VecF32> a1;
        memset(&a1, 0, sizeof a1);
        a1.out_par = 1 - par; a1.nsrc = 1; a1.skip = skip;
        a1.in[0].p = (float2 *)cgp; a1.out[0].p = (float2 *)t;
        MKS_TRY((launch_dslash<float, LinkF32, VecF32, VecF32, EPI_PLAIN, 0>(MKS_K_DSLASH_F32, L.fat, L.lng, a1, FinNone())));
        DslashArgs<VecF32, VecF32, VecF32> a2;
        memset(&a2, 0, sizeof a2);
        a2.out_par = par; a2.nsrc = 1; a2.skip = skip; a2.totals = tot;
        a2.in[0].p = (float2 *)t; a2.out[0].p = (float2 *)ttt; a2.p[0].p = (float2 *)cgp; a2.r[0].p = (float2 *)r;
        a2.coef[0] = h.shift0;
        MKS_TRY((launch_dslash<float, LinkF32, VecF32, VecF32, EPI_AXPY, 3>(MKS_K_DSLASH_F32, L.fat, L.lng, a2, FinMsAlpha{st})));
      } else {
        LinkSet16 L = links16(sl);
        DslashArgs<VecF16, VecF16, VecF32> a1;
        memset(&a1, 0, sizeof a1);
        a1.out_par = 1 - par; a1.nsrc = 1; a1.skip = skip;
        a1.in[0].p = p16; a1.in[0].norm = p16n; a1.out[0].p = t16; a1.out[0].norm = t16n;
        MKS_TRY((launch_dslash<float, LinkF16, VecF16, VecF16, EPI_PLAIN, 0>(MKS_K_DSLASH_F16, L.fat, L.lng, a1, FinNone())));
        DslashArgs<VecF16, VecF32, VecF32> a2;
        memset(&a2, 0, sizeof a2);
        a2.out_par = par; a2.nsrc = 1; a2.skip = skip; a2.totals = tot;
        a2.in[0].p = t16; a2.in[0].norm = t16n; a2.out[0].p = (float2 *)ttt; a2.p[0].p = (float2 *)cgp;
        a2.r[0].p = (float2 *)r; a2.coef[0] = h.shift0;
        MKS_TRY((launch_dslash<float, LinkF16, VecF16, VecF32, EPI_AXPY, 3>(MKS_K_DSLASH_F16, L.fat, L.lng, a2, FinMsAlpha{st})));
      }
      OpShiftUpdate<R, RS> up;
      memset(&up, 0, sizeof up);
      for (int j = 0; j < nsh; j++) { up.psim[j] = psim[j]; up.pm[j] = pm[j]; }
      up.r = r; up.ttt = ttt; up.cgp = cgp; up.p16 = p16; up.p16n = p16n; up.st = st; up.Vh = Vh;
      MKS_TRY((launch_site<OpShiftUpdate<R, RS>, 1, FinMsUpdate>(MKS_K_SHIFT, up, FinMsUpdate{st, skip}, skip, 1)));
    }
    return MKS_OK;
  };
  std::vector<uint64_t> key;
  key_push(key, -1); key_push(key, sizeof(R)); key_push(key, prec); key_push(key, par); key_push(key, np);
  key_push(key, (int)c.timing); key_push(key, c.geom.Vh); key_push(key, c.geom.nx); key_push(key, c.geom.ny);
  key_push(key, c.geom.nz); key_push(key, c.geom.nt);
  key_push(key, sl.fat64); key_push(key, sl.lng64); key_push(key, sl.fat32a); key_push(key, sl.lng32a);
  key_push(key, sl.fat32b); key_push(key, sl.lng32b); key_push(key, sl.fat16a); key_push(key, sl.lng16a);
  key_push(key, sl.fat16b); key_push(key, sl.lng16b); key_push(key, sl.fat16scale); key_push(key, sl.lng16scale);
  key_push(key, st); key_push(key, skip); key_push(key, tot); key_push(key, c.red.partials); key_push(key, c.red.count);
  key_push(key, h.shift0); key_push(key, nsh); key_push(key, r); key_push(key, cgp); key_push(key, ttt);
  key_push(key, t); key_push(key, p16); key_push(key, t16); key_push(key, p16n); key_push(key, t16n);
  for (int j = 0; j < nsh; j++) { key_push(key, psim[j]); key_push(key, pm[j]); }
  while (h.status == ST_RUN) {
    MKS_TRY(graph_batch(key, issue));
    MKS_CUDA(cudaMemcpyAsync(&h, st, sizeof h, cudaMemcpyDeviceToHost, c.stream));
    MKS_CUDA(cudaStreamSynchronize(c.stream));
    if (++guard > 10000000) return MKS_ERR_TIMEOUT;
    if (h.status == ST_HOST && h.want_reliable) {
      // reliable update: fold, FP64 residual of the lowest shift, continue
      if (!wide) MKS_TRY(ms_fold(nsh, x64, psim_out));
      double2 *t64, *dd64;
      MKS_TRY(wsv("ms_rel_t64", n, &t64));
      MKS_TRY(wsv("ms_rel_dd64", n, &dd64));
      double2 *xl = x64[h.j_low];
      MKS_TRY(apply_DD64(sl, par, 1, &xl, &t64, &dd64));
      OpMsResid op;
      op.src = src64; op.ddx = dd64; op.x = xl; op.r32 = (float2 *)r; op.sigma = offsets[h.j_low]; op.Vh = Vh;
      MKS_TRY((launch_site<OpMsResid, 1, FinNone>(MKS_K_BLAS, op, FinNone(), nullptr, 1, tot)));
      double rr = 0;
      MKS_CUDA(cudaMemcpyAsync(&rr, tot, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
      MKS_CUDA(cudaStreamSynchronize(c.stream));
      h.rsq = rr;
      h.maxrr = sqrt(rr);
      h.want_reliable = 0;
      h.n_reliable++;
      h.status = (h.rsq <= h.rsqstop || !std::isfinite(h.rsq)) ? ST_HOST : ST_RUN;
      MKS_CUDA(cudaMemcpyAsync(st, &h, sizeof h, cudaMemcpyHostToDevice, c.stream));
      MKS_CUDA(cudaMemcpyAsync(skip, &zero, sizeof zero, cudaMemcpyHostToDevice, c.stream));
    }
  }
  if (h.delta > 0 && !wide) MKS_TRY(ms_fold(nsh, x64, psim_out));
  *hstate = h;
  return MKS_OK;
}

// Several fields (sources), each with its own offsets, advanced together
// on the same links: one multi-source D_eo pair per iteration reads the
// links once for all running fields, and one update launch advances every
// field's shifts.  FP32 sloppy vectors with FP64 reliable updates of each
// field's lowest shift, exactly as multishift_core does for one field; a
// field that stops leaves the launches (the kernels are rebuilt for the
// remaining fields).  On exit x64[f][j] holds every field's solutions.
template <typename RS = float>
static int multishift_multi_core(const LinkSlot &sl, int par, int nf, const double2 *const *src64, const int *nsh,
                                 const double *const *offsets, double resid, int niter, double2 *const *const *x64,
                                 double delta, MsState *hs) {
  typedef float2 T2;
  typedef typename VT<RS>::v2 S2;
  constexpr bool wide = sizeof(RS) == 8;
  Context &c = ctx();
  const int Vh = (int)c.Vh;
  const size_t n = 3 * c.Vh;
  T2 *r[MSF], *cgp[MSF], *ttt[MSF], *t[MSF];
  S2 *pm[MSF][MAXSH], *psim[MSF][MAXSH];
  for (int f = 0; f < nf; f++) {
    const std::string k = std::to_string(f);
    MKS_TRY(wsv("msm_r_" + k, n, &r[f]));
    MKS_TRY(wsv("msm_p_" + k, n, &cgp[f]));
    MKS_TRY(wsv("msm_ttt_" + k, n, &ttt[f]));
    MKS_TRY(wsv("msm_t_" + k, n, &t[f]));
    for (int j = 0; j < nsh[f]; j++) {
      MKS_TRY(wsv((wide ? "msm_pm64_" : "msm_pm_") + k + "_" + std::to_string(j), n, &pm[f][j]));
      if (wide) psim[f][j] = (S2 *)x64[f][j];
      else MKS_TRY(wsv("msm_x_" + k + "_" + std::to_string(j), n, &psim[f][j]));
    }
  }
  MsState *st;
  int *skip;
  double *tot, *tot1;
  MKS_TRY(wsv("msm_state", MSF, &st));
  MKS_TRY(wsv("msm_skip", 1, &skip));
  MKS_TRY(wsv("msm_tot", 3 * MSF, &tot));
  MKS_TRY(wsv("msm_tot1", 4, &tot1));
  // initial state of every field (ks_multicg_offset.c:180-262)
  for (int f = 0; f < nf; f++) {
    MsState &h = hs[f];
    memset(&h, 0, sizeof h);
    double offset_low = 1.0e20;
    int j_low = 0;
    for (int j = 0; j < nsh[f]; j++) {
      h.shifts[j] = offsets[f][j];
      if (offsets[f][j] < offset_low) { offset_low = offsets[f][j]; j_low = j; }
    }
    for (int j = 0; j < nsh[f]; j++)
      if (j != j_low) h.shifts[j] -= h.shifts[j_low];
    h.shift0 = -h.shifts[j_low];
    h.j_low = j_low; h.num_now = nsh[f]; h.num_offsets = nsh[f]; h.niter = niter;
    for (int j = 0; j < nsh[f]; j++) { h.zeta_im1[j] = h.zeta_i[j] = 1.0; h.beta_im1[j] = -1.0; h.alpha[j] = 0.0; }
    OpShiftInit<float, RS> op;
    memset(&op, 0, sizeof op);
    for (int j = 0; j < nsh[f]; j++) { op.psim[j] = psim[f][j]; op.pm[j] = pm[f][j]; }
    op.r = r[f]; op.cgp = cgp[f]; op.src = src64[f]; op.Vh = Vh; op.n = nsh[f];
    MKS_TRY((launch_site<OpShiftInit<float, RS>, 1, FinNone>(MKS_K_BLAS, op, FinNone(), nullptr, 1, tot1)));
    double sn = 0;
    MKS_CUDA(cudaMemcpyAsync(&sn, tot1, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    MKS_CUDA(cudaStreamSynchronize(c.stream));
    h.source_norm = sn;
    h.rsq = sn;
    h.rsqstop = resid * resid * sn;
    h.iter = 1;
    h.status = sn == 0.0 ? ST_DONE : ST_RUN;
    h.maxrr = sqrt(sn);
    h.delta = delta;
    h.rsqretire = 0.01 * h.rsqstop;
    h.check_true = ms_true_stop();
    if (!wide)
      for (int j = 0; j < nsh[f]; j++) MKS_CUDA(cudaMemsetAsync(x64[f][j], 0, n * sizeof(double2), c.stream));
  }
  MKS_CUDA(cudaMemcpyAsync(st, hs, nf * sizeof(MsState), cudaMemcpyHostToDevice, c.stream));
  const int zero = 0;
  MKS_CUDA(cudaMemcpyAsync(skip, &zero, sizeof zero, cudaMemcpyHostToDevice, c.stream));
  const int np = poll_interval();
  LinkSet32 L = links32(sl);
  int guard = 0;
  while (true) {
    int act[MSF], nact = 0;
    for (int f = 0; f < nf; f++)
      if (hs[f].status == ST_RUN) act[nact++] = f;
    if (nact == 0) break;
    auto issue = [&]() -> int {
      for (int k = 0; k < np; k++) {
        DslashArgs<VecF32, VecF32, VecF32> a1;
        memset(&a1, 0, sizeof a1);
        a1.out_par = 1 - par; a1.nsrc = nact; a1.skip = skip;
        for (int q = 0; q < nact; q++) { a1.in[q].p = cgp[act[q]]; a1.out[q].p = t[act[q]]; }
        MKS_TRY((launch_dslash<float, LinkF32, VecF32, VecF32, EPI_PLAIN, 0>(MKS_K_DSLASH_F32, L.fat, L.lng, a1,
                                                                           FinNone())));
        DslashArgs<VecF32, VecF32, VecF32> a2;
        memset(&a2, 0, sizeof a2);
        a2.out_par = par; a2.nsrc = nact; a2.skip = skip; a2.totals = tot;
        FinMsAlphaM fa;
        fa.st = st;
        for (int q = 0; q < nact; q++) {
          const int f = act[q];
          a2.in[q].p = t[f]; a2.out[q].p = ttt[f]; a2.p[q].p = cgp[f]; a2.r[q].p = r[f]; a2.coef[q] = hs[f].shift0;
          fa.map[q] = f;
        }
        MKS_TRY((launch_dslash<float, LinkF32, VecF32, VecF32, EPI_AXPY, 3>(MKS_K_DSLASH_F32, L.fat, L.lng, a2, fa)));
        OpShiftUpdateM<float, RS> up;
        memset(&up, 0, sizeof up);
        FinMsUpdateM fu;
        fu.st = st; fu.skip = skip;
        for (int f = 0; f < nf; f++) {
          for (int j = 0; j < nsh[f]; j++) { up.psim[f][j] = psim[f][j]; up.pm[f][j] = pm[f][j]; }
          up.r[f] = r[f]; up.ttt[f] = ttt[f]; up.cgp[f] = cgp[f];
        }
        for (int q = 0; q < nact; q++) { up.map[q] = act[q]; fu.map[q] = act[q]; }
        up.st = st; up.Vh = Vh;
        MKS_TRY((launch_site<OpShiftUpdateM<float, RS>, 1, FinMsUpdateM>(MKS_K_SHIFT, up, fu, skip, nact)));
      }
      return MKS_OK;
    };
    std::vector<uint64_t> key;
    key_push(key, -2); key_push(key, par); key_push(key, np); key_push(key, (int)c.timing);
    key_push(key, c.geom.Vh); key_push(key, c.geom.nx); key_push(key, c.geom.ny); key_push(key, c.geom.nz);
    key_push(key, c.geom.nt); key_push(key, sl.fat32a); key_push(key, sl.lng32a); key_push(key, sl.fat32b);
    key_push(key, sl.lng32b); key_push(key, st); key_push(key, skip); key_push(key, tot);
    key_push(key, c.red.partials); key_push(key, c.red.count); key_push(key, nact);
    for (int q = 0; q < nact; q++) {
      const int f = act[q];
      key_push(key, f); key_push(key, hs[f].shift0); key_push(key, nsh[f]); key_push(key, r[f]);
      key_push(key, cgp[f]); key_push(key, ttt[f]); key_push(key, t[f]);
    }
    for (int f = 0; f < nf; f++)
      for (int j = 0; j < nsh[f]; j++) { key_push(key, psim[f][j]); key_push(key, pm[f][j]); }
    // poll until a field needs the host, then serve it
    bool host = false;
    while (!host) {
      MKS_TRY(graph_batch(key, issue));
      MKS_CUDA(cudaMemcpyAsync(hs, st, nf * sizeof(MsState), cudaMemcpyDeviceToHost, c.stream));
      MKS_CUDA(cudaStreamSynchronize(c.stream));
      MKS_TRY(red_check());
      if (++guard > 10000000) return MKS_ERR_TIMEOUT;
      for (int q = 0; q < nact; q++) host |= hs[act[q]].status != ST_RUN;
    }
    for (int q = 0; q < nact; q++) {
      const int f = act[q];
      MsState &h = hs[f];
      if (h.status != ST_HOST || !h.want_reliable) continue;   // stopped fields leave the launches
      // reliable update of field f: fold, FP64 residual of its lowest shift
      if (!wide) MKS_TRY(ms_fold(nsh[f], x64[f], (void *const *)psim[f]));
      double2 *t64, *dd64;
      MKS_TRY(wsv("ms_rel_t64", n, &t64));
      MKS_TRY(wsv("ms_rel_dd64", n, &dd64));
      double2 *xl = x64[f][h.j_low];
      MKS_TRY(apply_DD64(sl, par, 1, &xl, &t64, &dd64));
      OpMsResid op;
      op.src = src64[f]; op.ddx = dd64; op.x = xl; op.r32 = r[f]; op.sigma = offsets[f][h.j_low]; op.Vh = Vh;
      MKS_TRY((launch_site<OpMsResid, 1, FinNone>(MKS_K_BLAS, op, FinNone(), nullptr, 1, tot1)));
      double rr = 0;
      MKS_CUDA(cudaMemcpyAsync(&rr, tot1, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
      MKS_CUDA(cudaStreamSynchronize(c.stream));
      h.rsq = rr;
      h.maxrr = sqrt(rr);
      h.want_reliable = 0;
      h.n_reliable++;
      h.status = (h.rsq <= h.rsqstop || !std::isfinite(h.rsq)) ? ST_HOST : ST_RUN;
    }
    MKS_CUDA(cudaMemcpyAsync(st, hs, nf * sizeof(MsState), cudaMemcpyHostToDevice, c.stream));
    MKS_CUDA(cudaMemcpyAsync(skip, &zero, sizeof zero, cudaMemcpyHostToDevice, c.stream));
  }
  if (!wide)
    for (int f = 0; f < nf; f++) MKS_TRY(ms_fold(nsh[f], x64[f], (void *const *)psim[f]));
  MKS_CUDA(cudaStreamSynchronize(c.stream));
  return MKS_OK;
}

// nf fields on one slot: offsets, psim_dev and res are the fields' lists one
// after the other (num_offsets[f] entries each)
// iterations and shift updates (shifts advanced, summed over iterations) of
// the last multi-shift iteration phase, for the update kernel's byte count
static long long g_ms_iters = 0, g_ms_shift_updates = 0;

// The block-CG refinement after a sloppy multi-shift runs its inner solve
// in FP32 when the multi-shift ran in FP16: the multi-source FP16 D_eo is
// slower than the FP32 one (its half-to-float conversions make it
// issue-bound), and the refinement solves several shifts at once.
static mks_invert_arg refine_arg(const mks_invert_arg *arg) {
  mks_invert_arg a = *arg;
  if (a.prec == MKS_PREC_HALF) a.prec = MKS_PREC_SINGLE;
  return a;
}

static int multishift_multi_dev_once(int nf, const double *const *src_dev, const int *num_offsets,
                                     const double *offsets, double *const *psim_dev, int slot,
                                     const mks_invert_arg *arg, mks_invert_result *res) {
  Context &c = ctx();
  const LinkSlot &sl = c.slots[slot];
  int par;
  MKS_TRY(parity_index(arg->parity, &par));
  const double2 *src64[MSF];
  const double *offs[MSF];
  double2 *x64s[MSF][MAXSH];
  double2 *const *x64p[MSF];
  int base[MSF + 1];
  base[0] = 0;
  for (int f = 0; f < nf; f++) {
    base[f + 1] = base[f] + num_offsets[f];
    offs[f] = offsets + base[f];
    for (int j = 0; j < num_offsets[f]; j++)
      if (!(offs[f][j] > 0)) return MKS_ERR_ARG;
    double2 *s64;
    MKS_TRY(wsv("msm_src64_" + std::to_string(f), 3 * c.Vh, &s64));
    MKS_TRY(vec_aos_to_soa64(src_dev[f], s64, par));
    src64[f] = s64;
    for (int j = 0; j < num_offsets[f]; j++)
      MKS_TRY(wsv("msm_x64_" + std::to_string(f) + "_" + std::to_string(j), 3 * c.Vh, &x64s[f][j]));
    x64p[f] = x64s[f];
  }
  MsState hs[MSF];
  if (ms_shift64(arg->resid, true))
    MKS_TRY(multishift_multi_core<double>(sl, par, nf, src64, num_offsets, offs, arg->resid, arg->max * arg->nrestart,
                                          x64p, arg->delta > 0 ? arg->delta : 0.1, hs));
  else
    MKS_TRY(multishift_multi_core<float>(sl, par, nf, src64, num_offsets, offs, arg->resid, arg->max * arg->nrestart,
                                         x64p, arg->delta > 0 ? arg->delta : 0.1, hs));
  g_ms_iters = 0;
  g_ms_shift_updates = 0;
  for (int f = 0; f < nf; f++) {
    g_ms_iters = hs[f].iter > g_ms_iters ? hs[f].iter : g_ms_iters;
    g_ms_shift_updates += hs[f].shift_updates;
  }
  // FP64 check of every shift of every field, refinement of those that miss
  // (ks_multicg.c:170-228), blocks of up to MAXSRC shifts across the fields
  const int total = base[nf];
  std::vector<int> fld(total), shf(total);
  for (int f = 0; f < nf; f++)
    for (int j = 0; j < num_offsets[f]; j++) { fld[base[f] + j] = f; shf[base[f] + j] = j; }
  for (int b0 = 0; b0 < total; b0 += MAXSRC) {
    const int nb = total - b0 < MAXSRC ? total - b0 : MAXSRC;
    CgFields cf;
    memset(&cf, 0, sizeof cf);
    const mks_invert_arg ra = refine_arg(arg);
    MKS_TRY(alloc_cg_fields(cf, nb, ra.prec));
    double sig[MAXSRC];
    for (int q = 0; q < nb; q++) {
      const int f = fld[b0 + q], j = shf[b0 + q];
      cf.src[q] = (double2 *)src64[f];
      cf.x[q] = x64s[f][j];
      sig[q] = offs[f][j];
    }
    MKS_TRY(block_cg_shifted(slot, par, nb, sig, &ra, cf, res + b0));
    for (int q = 0; q < nb; q++) {
      const int f = fld[b0 + q];
      MKS_TRY(vec_soa64_to_aos(cf.x[q], psim_dev[b0 + q], par));
      res[b0 + q].final_iters += hs[f].iter;
      res[b0 + q].reliable_updates += hs[f].n_reliable;
    }
  }
  MKS_CUDA(cudaStreamSynchronize(c.stream));
  int mx = 0;
  for (int q = 0; q < total; q++) mx = res[q].final_iters > mx ? res[q].final_iters : mx;
  return mx;
}

static int multishift_dev_once(const double *src_dev, double *const *psim_dev, const double *offsets, int nsh,
                               int slot, const mks_invert_arg *arg, mks_invert_result *res) {
  Context &c = ctx();
  const LinkSlot &sl = c.slots[slot];
  int par;
  MKS_TRY(parity_index(arg->parity, &par));
  for (int j = 0; j < nsh; j++)
    if (!(offsets[j] > 0)) return MKS_ERR_ARG;  // ks_multicg_offset.c:152-158
  double2 *src64;
  MKS_TRY(wsv("ms_src64", 3 * c.Vh, &src64));
  MKS_TRY(vec_aos_to_soa64(src_dev, src64, par));
  const int niter = arg->max * arg->nrestart;
  MsState h;
  void *psim[MAXSH];
  if (arg->prec == MKS_PREC_DOUBLE) {
    MKS_TRY(multishift_core<double>(sl, par, MKS_PREC_DOUBLE, src64, nsh, offsets, arg->resid, niter, psim, &h));
    g_ms_iters = h.iter;
    g_ms_shift_updates = h.shift_updates;
    for (int j = 0; j < nsh; j++) {
      MKS_TRY(vec_soa64_to_aos((double2 *)psim[j], psim_dev[j], par));
      res[j] = mks_invert_result();
      res[j].final_rsq = h.rsq / (h.source_norm > 0 ? h.source_norm : 1.0);
      res[j].size_r = res[j].final_rsq;
      res[j].final_iters = h.iter;
      res[j].converged = (h.source_norm == 0 || h.rsq <= h.rsqstop) ? 1 : 0;
    }
    if (h.source_norm == 0)
      for (int j = 0; j < nsh; j++) MKS_TRY(vec_soa64_to_aos(src64, psim_dev[j], par));  // zero source -> zero
    MKS_CUDA(cudaStreamSynchronize(c.stream));
    return h.iter;
  }
  // sloppy multi-shift (FP32 / FP16 vectors) with FP64 reliable updates of the
  // lowest shift to the requested residual, the shifts' solutions accumulated
  // in FP64; then each shift's true residual is checked in FP64 and the shifts
  // that miss it are refined by the mixed-precision block CG
  // (generic_ks/ks_multicg.c:170-228)
  double2 *x64[MAXSH];
  for (int j = 0; j < nsh; j++) MKS_TRY(wsv("ms_x64_" + std::to_string(j), 3 * c.Vh, &x64[j]));
  if (ms_shift64(arg->resid, false))
    MKS_TRY((multishift_core<float, double>(sl, par, arg->prec, src64, nsh, offsets, arg->resid, niter, psim, &h,
                                            x64, arg->delta > 0 ? arg->delta : 0.1)));
  else
    MKS_TRY(multishift_core<float>(sl, par, arg->prec, src64, nsh, offsets, arg->resid, niter, psim, &h, x64,
                                   arg->delta > 0 ? arg->delta : 0.1));
  int total_iters = h.iter;
  g_ms_iters = h.iter;
  g_ms_shift_updates = h.shift_updates;
  for (int b0 = 0; b0 < nsh; b0 += MAXSRC) {
    int nb = nsh - b0 < MAXSRC ? nsh - b0 : MAXSRC;
    CgFields f;
    memset(&f, 0, sizeof f);
    const mks_invert_arg ra = refine_arg(arg);
    MKS_TRY(alloc_cg_fields(f, nb, ra.prec));
    for (int s = 0; s < nb; s++) {
      f.src[s] = src64;       // read only in the block CG
      f.x[s] = x64[b0 + s];   // the sloppy solve's FP64 solution is the initial guess
    }
    double sig[MAXSRC];
    for (int s = 0; s < nb; s++) sig[s] = offsets[b0 + s];
    MKS_TRY(block_cg_shifted(slot, par, nb, sig, &ra, f, res + b0));
    for (int s = 0; s < nb; s++) {
      MKS_TRY(vec_soa64_to_aos(f.x[s], psim_dev[b0 + s], par));
      res[b0 + s].final_iters += total_iters;
      res[b0 + s].reliable_updates += h.n_reliable;
    }
  }
  MKS_CUDA(cudaStreamSynchronize(c.stream));
  int mx = 0;
  for (int j = 0; j < nsh; j++) mx = res[j].final_iters > mx ? res[j].final_iters : mx;
  return mx;
}

// The multi-shift entry cores, repeated once when the staged D_eo kernel gave
// up during the call (it is off afterwards; the solutions are outputs only).
static int multishift_dev(const double *src_dev, double *const *psim_dev, const double *offsets, int nsh, int slot,
                          const mks_invert_arg *arg, mks_invert_result *res) {
  int rc = multishift_dev_once(src_dev, psim_dev, offsets, nsh, slot, arg, res);
  if (rc == MKS_ERR_TIMEOUT && take_tma_retry()) rc = multishift_dev_once(src_dev, psim_dev, offsets, nsh, slot, arg, res);
  return rc;
}
static int multishift_multi_dev(int nf, const double *const *src_dev, const int *num_offsets, const double *offsets,
                                double *const *psim_dev, int slot, const mks_invert_arg *arg, mks_invert_result *res) {
  int rc = multishift_multi_dev_once(nf, src_dev, num_offsets, offsets, psim_dev, slot, arg, res);
  if (rc == MKS_ERR_TIMEOUT && take_tma_retry())
    rc = multishift_multi_dev_once(nf, src_dev, num_offsets, offsets, psim_dev, slot, arg, res);
  return rc;
}

}  // namespace mks

extern "C" {

int mks_ks_multicg_offset_field_dev(const double *src_dev, double *const *psim_dev, const double *offsets,
                                    int num_offsets, int slot, const mks_invert_arg *arg, mks_invert_result *res) {
  MKS_TRY(check_ready());
  MKS_TRY(slot_ok(slot));
  MKS_TRY(check_arg(arg, true));
  if (num_offsets == 0) return 0;
  if (num_offsets < 0 || num_offsets > MAXSH || !src_dev || !psim_dev || !offsets || !res) return MKS_ERR_ARG;
  return multishift_dev(src_dev, psim_dev, offsets, num_offsets, slot, arg, res);
}

int mks_ks_multicg_offset_multi_dev(int nf, const double *const *src_dev, const int *num_offsets,
                                    const double *offsets, double *const *psim_dev, int slot,
                                    const mks_invert_arg *arg, mks_invert_result *res) {
  MKS_TRY(check_ready());
  MKS_TRY(slot_ok(slot));
  MKS_TRY(check_arg(arg, true));
  if (nf < 1 || nf > MSF || !src_dev || !num_offsets || !offsets || !psim_dev || !res) return MKS_ERR_ARG;
  int total = 0;
  for (int f = 0; f < nf; f++) {
    if (num_offsets[f] < 1 || num_offsets[f] > MAXSH || !src_dev[f]) return MKS_ERR_ARG;
    total += num_offsets[f];
  }
  if (arg->prec != MKS_PREC_SINGLE || nf == 1) {
    // one field at a time (FP64 keeps MILC's single-field semantics)
    int mx = 0, off = 0;
    for (int f = 0; f < nf; f++) {
      const int it = multishift_dev(src_dev[f], psim_dev + off, offsets + off, num_offsets[f], slot, arg, res + off);
      if (it < 0) return it;
      mx = it > mx ? it : mx;
      off += num_offsets[f];
    }
    return mx;
  }
  (void)total;
  return multishift_multi_dev(nf, src_dev, num_offsets, offsets, psim_dev, slot, arg, res);
}

int mks_ks_multicg_offset_field(const double *src, double *const *psim, const double *offsets, int num_offsets,
                                int slot, const mks_invert_arg *arg, mks_invert_result *res) {
  MKS_TRY(check_ready());
  MKS_TRY(slot_ok(slot));
  MKS_TRY(check_arg(arg, true));
  if (num_offsets == 0) return 0;
  if (num_offsets < 0 || num_offsets > MAXSH || !src || !psim || !offsets || !res) return MKS_ERR_ARG;
  Context &c = ctx();
  // the solve reads the source and writes the solutions on arg->parity only
  // (one contiguous half of MILC's even-first fields); psim is output only
  int par;
  MKS_TRY(parity_index(arg->parity, &par));
  const size_t off = (size_t)par * c.Vh * 6, bytes = c.Vh * 6 * sizeof(double);
  double *ds;
  double *dp[MAXSH];
  // page-locked, mapped arrays are read and written in place by the layout
  // kernels; otherwise the source and solutions are staged by copies
  bool mapped = (ds = mapped_host(src)) != nullptr;
  for (int j = 0; j < num_offsets && mapped; j++) mapped = (dp[j] = mapped_host(psim[j])) != nullptr;
  if (mapped) {
    int it = multishift_dev(ds, dp, offsets, num_offsets, slot, arg, res);
    MKS_CUDA(cudaStreamSynchronize(c.stream));
    return it;
  }
  MKS_TRY(wsv("hsrc0", 6 * c.V, &ds));
  MKS_CUDA(cudaMemcpyAsync(ds + off, src + off, bytes, cudaMemcpyHostToDevice, c.stream));
  for (int j = 0; j < num_offsets; j++) MKS_TRY(wsv("hpsim" + std::to_string(j), 6 * c.V, &dp[j]));
  int it = multishift_dev(ds, dp, offsets, num_offsets, slot, arg, res);
  if (it < 0) return it;
  for (int j = 0; j < num_offsets; j++)
    MKS_CUDA(cudaMemcpyAsync(psim[j] + off, dp[j] + off, bytes, cudaMemcpyDeviceToHost, c.stream));
  MKS_CUDA(cudaStreamSynchronize(c.stream));
  return it;
}

}  // extern "C"

extern "C" int mks_tuned_shape(int prec, int nsrc, int *G, int *nb, int *block) {
  if (prec < 0 || prec > 2 || nsrc < 1 || nsrc > MAXSRC) return MKS_ERR_ARG;
  const Shape &s = g_shape[prec][nsrc];
  if (s.G == 0) return MKS_ERR_STATE;
  if (G) *G = s.G;
  if (nb) *nb = s.NB;
  if (block) *block = s.block;
  return MKS_OK;
}

extern "C" int mks_tuned_shape_epi(int prec, int nsrc, int *G, int *nb, int *block, int *tma) {
  if (prec < 0 || prec > 2 || nsrc < 1 || nsrc > MAXSRC) return MKS_ERR_ARG;
  const Shape &s = g_shape_epi[prec][nsrc];
  if (s.G == 0) return MKS_ERR_STATE;
  if (G) *G = s.G;
  if (nb) *nb = s.NB;
  if (block) *block = s.block;
  if (tma) *tma = s.tma;
  return MKS_OK;
}

extern "C" int mks_multishift_counts(long long *iters, long long *shift_updates) {
  if (iters) *iters = g_ms_iters;
  if (shift_updates) *shift_updates = g_ms_shift_updates;
  return MKS_OK;
}

extern "C" int mks_tuned_variant(int prec, int nsrc, int epi) {
  if (prec < 0 || prec > 2 || nsrc < 1 || nsrc > MAXSRC) return MKS_ERR_ARG;
  const Shape &s = (epi ? g_shape_epi : g_shape)[prec][nsrc];
  if (s.G == 0) return MKS_ERR_STATE;
  return (s.tma ? 1 : (s.pipe ? 2 : (s.as ? 3 : 0))) + (s.persist ? 4 : 0) + 8 * s.as;
}
