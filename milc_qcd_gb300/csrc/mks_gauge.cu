// mks_gauge.cu -- gauge-field side of the RHMC molecular dynamics on the GPU.
//
// Replaces, for a GPU-resident trajectory:
//   imp_gauge_force_cpu / _gpu   generic/gauge_force_imp.c:37-223 (USE_GF_GPU)
//   imp_gauge_action             generic/gauge_stuff.c:277-330
//   make_loop_table              generic/gauge_stuff.c:87-197 with
//                                generic/imp_actions/symanzik_1loop_hisq_action.h
//   update_u                     ks_imp_rhmc/update_u.c:49-108 (8th-order Taylor)
//   hmom_action                  ks_imp_rhmc/d_action_rhmc.c:89-122
//   reunitarize_ks               generic_ks/reunitarize_ks.c, generic/reunitarize2.c:112-216
//   ranmom, site generators      generic/ranmom.c, generic/ranstuff.c:60-130,
//                                libraries/gaussrand.c:78-100, libraries/rand_ahmat.c:36-52
//   d_plaquette                  generic/d_plaq4.c
//
// State held in the context: the thin links (auxU, phases in, FP64 SoA),
// the momentum field (MILC's anti_hermitmat[V][4] layout, device) and one
// MILC site random generator per site.  Every kernel works on one link or
// one site per thread; the loop/staple paths are tables in constant memory
// generated on the host exactly as MILC generates its loop table.  The
// force and action walk each path link by link (recomputation instead of
// stored intermediate staple fields), in FP64.
#include <cmath>
#include <cstring>
#include <vector>
#include "mks_internal.cuh"
#include "mks_su3.cuh"
#include "mks_blas.cuh"

namespace mks {

// ------------------------------------------------------------------ phases
// MILC's staggered phases and antiperiodic time boundary
// (generic_ks/rephase.c:61-95): eta_x = (-1)^t, eta_y = (-1)^(t+x),
// eta_z = (-1)^(t+x+y), eta_t = 1, times -1 on the t links of t = nt-1.
__device__ __forceinline__ double stag_phase(const Geom &g, const int c[4], int dir) {
  const int t = c[3], x = c[0], y = c[1];
  switch (dir) {
  case 0: return (t & 1) ? -1.0 : 1.0;
  case 1: return ((t + x) & 1) ? -1.0 : 1.0;
  case 2: return ((t + x + y) & 1) ? -1.0 : 1.0;
  default: return (t == g.nt - 1) ? -1.0 : 1.0;
  }
}

__device__ __forceinline__ M3<double> load_link(const Geom &g, const double2 *U, const int c[4], int dir,
                                                bool unphase) {
  const int par = (c[0] + c[1] + c[2] + c[3]) & 1;
  const int h = cb_index(g, c[0], c[1], c[2], c[3]);
  M3<double> m = link_dir(const_cast<double2 *>(U), dir, g.Vh).ld(par, h, g.Vh);
  if (unphase && stag_phase(g, c, dir) < 0) {
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) { m.e[i][j].re = -m.e[i][j].re; m.e[i][j].im = -m.e[i][j].im; }
  }
  return m;
}

// unphased FP32 copy of the thin links, same [2][4][9][Vh] layout: the FP32
// gauge force walks ~230 links per output link through L1/L2, so halving
// the bytes of every link fetched matters more than the conversion pass
__global__ void __launch_bounds__(128) k_thin_to_f32(Geom g, const double2 *U, float2 *U32) {
  const int h = blockIdx.x * blockDim.x + threadIdx.x, par = blockIdx.y, mu = blockIdx.z;
  if (h >= g.Vh) return;
  int c[4];
  site_coords(g, par, h, c[0], c[1], c[2], c[3]);
  const float ph = (float)stag_phase(g, c, mu);
  const size_t base = ((size_t)par * 4 + mu) * 9 * g.Vh + h;
#pragma unroll
  for (int k = 0; k < 9; k++) {
    const double2 a = U[base + (size_t)k * g.Vh];
    U32[base + (size_t)k * g.Vh] = make_float2(ph * (float)a.x, ph * (float)a.y);
  }
}

__device__ __forceinline__ M3<float> load_link32(const Geom &g, const float2 *U32, const int c[4], int dir) {
  const int par = (c[0] + c[1] + c[2] + c[3]) & 1;
  const int h = cb_index(g, c[0], c[1], c[2], c[3]);
  const float2 *b = U32 + ((size_t)par * 4 + dir) * 9 * g.Vh + h;
  M3<float> m;
#pragma unroll
  for (int k = 0; k < 9; k++) {
    const float2 a = __ldg(b + (size_t)k * g.Vh);
    m.e[k / 3][k % 3] = {a.x, a.y};
  }
  return m;
}

// ------------------------------------------------------------------ paths
constexpr int GPATH_MAX = 64;
struct LoopPaths {       // every loop orientation of the action (34 for Symanzik 1-loop)
  int n;
  int len[GPATH_MAX];
  signed char dir[GPATH_MAX][6];
  double c[GPATH_MAX];
};
struct StaplePaths {     // per link direction: the rest of each loop through the link
  int n[4];
  int len[4][GPATH_MAX];
  signed char dir[4][GPATH_MAX][5];
  double c[4][GPATH_MAX];
};
__constant__ LoopPaths c_loops;
__constant__ StaplePaths c_staples;

struct LoopTable {
  int nloop, length[3], num[3], dirs[3][16][6];
  double coeff[3];
};

// smallest label of a path over cyclic shifts and reversal
// (gauge_stuff.c:237-275): equal labels are the same loop
static int loop_label(const int *dig, int length) {
  int tenl = 1, chr, old, newv, bdig[8] = {0};
  for (int j = 0; j < length - 1; j++) tenl *= 10;
  chr = dig[length - 1];
  for (int j = length - 2; j >= 0; j--) chr = chr * 10 + dig[j];
  old = chr;
  for (int j = length - 1; j >= 1; j--) {
    newv = (old - tenl * dig[j]) * 10 + dig[j];
    if (newv < chr) chr = newv;
    old = newv;
  }
  for (int j = 0; j < length; j++) bdig[j] = 7 - dig[length - j - 1];
  old = bdig[length - 1];
  for (int j = length - 2; j >= 0; j--) old = old * 10 + bdig[j];
  if (old < chr) chr = old;
  for (int j = length - 1; j >= 1; j--) {
    newv = (old - tenl * bdig[j]) * 10 + bdig[j];
    if (newv < chr) chr = newv;
    old = newv;
  }
  return chr;
}

// plaquette, 1x2 rectangle and 1x1x1 bent loop, all rotations and
// reflections; coefficients of the HISQ-improved Symanzik action
static void make_loop_table(int nflavors, double u0, LoopTable &T) {
  static const int base[3][6] = {{0, 1, 7, 6, 0, 0}, {0, 0, 1, 7, 7, 6}, {0, 1, 2, 7, 6, 5}};
  static const int blen[3] = {4, 6, 6};
  memset(&T, 0, sizeof T);
  T.nloop = 3;
  const double lu = std::log(u0);
  T.coeff[0] = 1.0;
  T.coeff[1] = -1.0 / (20.0 * u0 * u0) * (1.0 - (0.6264 - 1.1746 * nflavors) * lu);
  T.coeff[2] = 1.0 / (u0 * u0) * (0.0433 - 0.0156 * nflavors) * lu;
  for (int il = 0; il < 3; il++) {
    int count = 0, labels[16];
    T.length[il] = blen[il];
    int perm[4], ir[4], pp[8], vec[6];
    for (perm[0] = 0; perm[0] < 4; perm[0]++)
      for (perm[1] = 0; perm[1] < 4; perm[1]++)
        for (perm[2] = 0; perm[2] < 4; perm[2]++)
          for (perm[3] = 0; perm[3] < 4; perm[3]++) {
            if (perm[0] == perm[1] || perm[0] == perm[2] || perm[0] == perm[3] || perm[1] == perm[2] ||
                perm[1] == perm[3] || perm[2] == perm[3])
              continue;
            for (ir[0] = 0; ir[0] < 2; ir[0]++)
              for (ir[1] = 0; ir[1] < 2; ir[1]++)
                for (ir[2] = 0; ir[2] < 2; ir[2]++)
                  for (ir[3] = 0; ir[3] < 2; ir[3]++) {
                    for (int j = 0; j < 4; j++) {
                      pp[j] = ir[j] ? 7 - perm[j] : perm[j];
                      pp[7 - j] = 7 - pp[j];
                    }
                    for (int j = 0; j < blen[il]; j++) vec[j] = pp[base[il][j]];
                    const int chr = loop_label(vec, blen[il]);
                    bool seen = false;
                    for (int j = 0; j < count; j++) seen |= labels[j] == chr;
                    if (!seen && count < 16) {
                      labels[count] = chr;
                      for (int j = 0; j < blen[il]; j++) T.dirs[il][count][j] = vec[j];
                      count++;
                    }
                  }
          }
    T.num[il] = count;
  }
}

static int upload_paths(int nflavors, double u0) {
  static int last_nf = -1;
  static double last_u0 = 0.0;
  static int last_dev = -1;
  Context &c = ctx();
  if (nflavors == last_nf && u0 == last_u0 && c.device == last_dev) return MKS_OK;
  if (!(u0 > 0)) return MKS_ERR_ARG;
  LoopTable T;
  make_loop_table(nflavors, u0, T);
  LoopPaths lp;
  memset(&lp, 0, sizeof lp);
  StaplePaths sp;
  memset(&sp, 0, sizeof sp);
  for (int il = 0; il < T.nloop; il++)
    for (int ln = 0; ln < T.num[il]; ln++) {
      if (lp.n >= GPATH_MAX) return MKS_ERR_ARG;
      lp.len[lp.n] = T.length[il];
      for (int k = 0; k < T.length[il]; k++) lp.dir[lp.n][k] = (signed char)T.dirs[il][ln][k];
      lp.c[lp.n] = T.coeff[il];
      lp.n++;
    }
  // the staples of gauge_force_imp.c:121-155: each loop rotated to start
  // along `dir`, and for each of its links along +-dir the rest of the loop
  // from the link's far end back to its start (reversed loop for -dir)
  for (int dir = 0; dir < 4; dir++)
    for (int il = 0; il < T.nloop; il++)
      for (int ln = 0; ln < T.num[il]; ln++) {
        const int len = T.length[il];
        int dirs[6];
        for (int k = 0; k < len; k++) {
          const int d = T.dirs[il][ln][k];
          dirs[k] = d < 4 ? (dir + d) % 4 : 7 - ((dir + 7 - d) % 4);
        }
        for (int k = 0; k < len; k++) {
          if (dirs[k] != dir && dirs[k] != 7 - dir) continue;
          const int n = sp.n[dir];
          if (n >= GPATH_MAX) return MKS_ERR_ARG;
          for (int j = 0; j < len - 1; j++) {
            if (dirs[k] < 4)
              sp.dir[dir][n][j] = (signed char)dirs[(k + j + 1) % len];
            else
              sp.dir[dir][n][len - 2 - j] = (signed char)(7 - dirs[(k + j + 1) % len]);
          }
          sp.len[dir][n] = len - 1;
          sp.c[dir][n] = T.coeff[il];
          sp.n[dir]++;
        }
      }
  MKS_CUDA(cudaMemcpyToSymbolAsync(c_loops, &lp, sizeof lp, 0, cudaMemcpyHostToDevice, c.stream));
  MKS_CUDA(cudaMemcpyToSymbolAsync(c_staples, &sp, sizeof sp, 0, cudaMemcpyHostToDevice, c.stream));
  MKS_CUDA(cudaStreamSynchronize(c.stream));
  last_nf = nflavors;
  last_u0 = u0;
  last_dev = c.device;
  return MKS_OK;
}

template <typename R>
__device__ __forceinline__ M3<R> to_r(const M3<double> &m) {
  M3<R> o;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) o.e[i][j] = {(R)m.e[i][j].re, (R)m.e[i][j].im};
  return o;
}
template <typename R>
__device__ __forceinline__ M3<R> mul_nn(const M3<R> &a, const M3<R> &b) {
  M3<R> c;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      R re = 0, im = 0;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        re = fma(a.e[i][k].re, b.e[k][j].re, re); re = fma(-a.e[i][k].im, b.e[k][j].im, re);
        im = fma(a.e[i][k].re, b.e[k][j].im, im); im = fma(a.e[i][k].im, b.e[k][j].re, im);
      }
      c.e[i][j] = {re, im};
    }
  return c;
}
template <typename R>
__device__ __forceinline__ M3<R> mul_na(const M3<R> &a, const M3<R> &b) {  // a b^dag
  M3<R> c;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      R re = 0, im = 0;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        re = fma(a.e[i][k].re, b.e[j][k].re, re); re = fma(a.e[i][k].im, b.e[j][k].im, re);
        im = fma(a.e[i][k].im, b.e[j][k].re, im); im = fma(-a.e[i][k].re, b.e[j][k].im, im);
      }
      c.e[i][j] = {re, im};
    }
  return c;
}

// product of the links along `path` from site c (modified: ends at the
// path's end), in arithmetic R (links stored FP64)
template <typename R>
__device__ __forceinline__ M3<R> walk_r(const Geom &g, const double2 *U, int c[4], const signed char *path, int len) {
  const int L[4] = {g.nx, g.ny, g.nz, g.nt};
  // the product starts from the first link itself (the identity product it
  // replaces is exact, so the result is the same to the last bit)
  M3<R> P;
  for (int k = 0; k < len; k++) {
    const int d = path[k];
    if (d < 4) {
      const M3<R> Lk = to_r<R>(load_link(g, U, c, d, true));
      P = k ? mul_nn<R>(P, Lk) : Lk;
      c[d] = wrap_add(c[d], 1, L[d]);
    } else {
      const int dd = 7 - d;
      c[dd] = wrap_add(c[dd], -1, L[dd]);
      const M3<R> Lk = to_r<R>(load_link(g, U, c, dd, true));
      P = k ? mul_na<R>(P, Lk) : tadj<R>(Lk);
    }
  }
  return P;
}
__device__ __forceinline__ M3<double> walk(const Geom &g, const double2 *U, int c[4], const signed char *path,
                                           int len) {
  return walk_r<double>(g, U, c, path, len);
}

// the same walk on the unphased FP32 copy
__device__ __forceinline__ M3<float> walk32(const Geom &g, const float2 *U32, int c[4], const signed char *path,
                                            int len) {
  const int L[4] = {g.nx, g.ny, g.nz, g.nt};
  M3<float> P;
  for (int k = 0; k < len; k++) {
    const int d = path[k];
    if (d < 4) {
      const M3<float> Lk = load_link32(g, U32, c, d);
      P = k ? mul_nn<float>(P, Lk) : Lk;
      c[d] = wrap_add(c[d], 1, L[d]);
    } else {
      const int dd = 7 - d;
      c[dd] = wrap_add(c[dd], -1, L[dd]);
      const M3<float> Lk = load_link32(g, U32, c, dd);
      P = k ? mul_na<float>(P, Lk) : tadj<float>(Lk);
    }
  }
  return P;
}

// mom_mu(x) <- TA(mom_mu(x) - eb3 U_mu(x) sum_p c_p Q_p), Q_p the staple
// paths from x+mu back to x (links without phases)
// staple sum and product in arithmetic R (FP64 reproduces MILC's double
// build; FP32 runs at the FP32 rate for large-lattice molecular dynamics);
// the momentum update is FP64 either way
template <typename R>
__global__ void __launch_bounds__(128) k_gauge_force(Geom g, const double2 *U, const float2 *U32, double *mom,
                                                     double eb3) {
  const int h = blockIdx.x * blockDim.x + threadIdx.x, par = blockIdx.y, mu = blockIdx.z;
  if (h >= g.Vh) return;
  int x0[4];
  site_coords(g, par, h, x0[0], x0[1], x0[2], x0[3]);
  const int L[4] = {g.nx, g.ny, g.nz, g.nt};
  M3<R> S;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) S.e[i][j] = {(R)0, (R)0};
  const int np = c_staples.n[mu];
  for (int p = 0; p < np; p++) {
    int c[4] = {x0[0], x0[1], x0[2], x0[3]};
    c[mu] = wrap_add(c[mu], 1, L[mu]);
    M3<R> Q;
    if constexpr (sizeof(R) == 4) Q = walk32(g, U32, c, c_staples.dir[mu][p], c_staples.len[mu][p]);
    else Q = walk_r<R>(g, U, c, c_staples.dir[mu][p], c_staples.len[mu][p]);
    const R cf = (R)c_staples.c[mu][p];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        S.e[i][j].re = fma(cf, Q.e[i][j].re, S.e[i][j].re);
        S.e[i][j].im = fma(cf, Q.e[i][j].im, S.e[i][j].im);
      }
  }
  M3<R> Ux;
  if constexpr (sizeof(R) == 4) Ux = load_link32(g, U32, x0, mu);
  else Ux = to_r<R>(load_link(g, U, x0, mu, true));
  const M3<R> Gr = mul_nn<R>(Ux, S);
  M3<double> G;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) G.e[i][j] = {(double)Gr.e[i][j].re, (double)Gr.e[i][j].im};
  double *m = mom + (((size_t)par * g.Vh + h) * 4 + mu) * 10;
  // A = uncompressed mom - eb3 G, then its traceless anti-Hermitian part
  // (libraries/uncmp_ahmat.c, make_ahmat.c)
  const double d0 = m[6] - eb3 * G.e[0][0].im, d1 = m[7] - eb3 * G.e[1][1].im, d2 = m[8] - eb3 * G.e[2][2].im;
  const double t = (d0 + d1 + d2) * 0.33333333333333333;
  const double a01r = m[0], a01i = m[1], a02r = m[2], a02i = m[3], a12r = m[4], a12i = m[5];
  m[0] = ((a01r - eb3 * G.e[0][1].re) - (-a01r - eb3 * G.e[1][0].re)) * 0.5;
  m[1] = ((a01i - eb3 * G.e[0][1].im) + (a01i - eb3 * G.e[1][0].im)) * 0.5;
  m[2] = ((a02r - eb3 * G.e[0][2].re) - (-a02r - eb3 * G.e[2][0].re)) * 0.5;
  m[3] = ((a02i - eb3 * G.e[0][2].im) + (a02i - eb3 * G.e[2][0].im)) * 0.5;
  m[4] = ((a12r - eb3 * G.e[1][2].re) - (-a12r - eb3 * G.e[2][1].re)) * 0.5;
  m[5] = ((a12i - eb3 * G.e[1][2].im) + (a12i - eb3 * G.e[2][1].im)) * 0.5;
  m[6] = d0 - t;
  m[7] = d1 - t;
  m[8] = d2 - t;
}

// sum over sites of one parity (row = parity) of c (3 - Re tr W) over every
// loop orientation W starting at the site
struct OpGaugeAction {
  Geom g;
  const double2 *U;
  __device__ void operator()(int h, int par, double *out) const {
    int x0[4];
    site_coords(g, par, h, x0[0], x0[1], x0[2], x0[3]);
    double acc = 0.0;
    for (int p = 0; p < c_loops.n; p++) {
      int c[4] = {x0[0], x0[1], x0[2], x0[3]};
      const M3<double> W = walk(g, U, c, c_loops.dir[p], c_loops.len[p]);
      acc += c_loops.c[p] * (3.0 - (W.e[0][0].re + W.e[1][1].re + W.e[2][2].re));
    }
    out[0] = acc;
  }
};

// plaquettes: out[0] space-space, out[1] space-time sums of Re tr
struct OpPlaquette {
  Geom g;
  const double2 *U;
  __device__ void operator()(int h, int par, double *out) const {
    int x0[4];
    site_coords(g, par, h, x0[0], x0[1], x0[2], x0[3]);
    double ss = 0.0, st = 0.0;
    for (int mu = 0; mu < 4; mu++)
      for (int nu = mu + 1; nu < 4; nu++) {
        const signed char path[4] = {(signed char)mu, (signed char)nu, (signed char)(7 - mu), (signed char)(7 - nu)};
        int c[4] = {x0[0], x0[1], x0[2], x0[3]};
        const M3<double> W = walk(g, U, c, path, 4);
        const double tr = W.e[0][0].re + W.e[1][1].re + W.e[2][2].re;
        if (nu == 3) st += tr; else ss += tr;
      }
    out[0] = ss;
    out[1] = st;
  }
};

// sum over the four directions of |mom|^2 - 4 (ahmat_mag_sq, d_action_rhmc.c:110-122)
struct OpMomAction {
  int Vh;
  const double *mom;
  __device__ void operator()(int h, int par, double *out) const {
    const double *m = mom + ((size_t)par * Vh + h) * 40;
    double acc = 0.0;
#pragma unroll
    for (int d = 0; d < 4; d++) {
      const double *q = m + 10 * d;
      double s = 0.5 * (q[6] * q[6] + q[7] * q[7] + q[8] * q[8]);
#pragma unroll
      for (int k = 0; k < 6; k++) s += q[k] * q[k];
      acc += s - 4.0;
    }
    out[0] = acc;
  }
};

// |v|^2 over the sites of one parity of an AoS FP64 field [V][6]
struct OpNormAos {
  int Vh, par;
  const double *v;
  __device__ void operator()(int h, int, double *out) const {
    const double *q = v + ((size_t)par * Vh + h) * 6;
    double a = 0.0;
#pragma unroll
    for (int k = 0; k < 6; k++) a += q[k] * q[k];
    out[0] = a;
  }
};

struct FinKeep {
  __device__ void operator()(const double *, int) const {}
};

template <class Op, int NS>
static int site_sum(const Op &op, int rows, double *host_out) {
  Context &c = ctx();
  const int Vh = (int)c.Vh;
  int gx = grid_for(Vh, 256);
  if (gx > c.sm_count * 4) gx = c.sm_count * 4;
  MKS_TRY(ensure_red(NS * rows, gx * rows));
  double *tot = nullptr;
  MKS_TRY(dev_alloc((void **)&tot, (size_t)NS * rows * sizeof(double)));
  timing_begin(MKS_K_GAUGE);
  k_site<Op, NS, FinKeep><<<dim3(gx, rows), 256, 0, c.stream>>>(op, FinKeep(), nullptr, Vh, c.red, tot);
  timing_end(MKS_K_GAUGE);
  int rc = cudaGetLastError() == cudaSuccess ? MKS_OK : MKS_ERR_CUDA;
  if (rc >= 0 && cudaMemcpyAsync(host_out, tot, (size_t)NS * rows * sizeof(double), cudaMemcpyDeviceToHost,
                                 c.stream) != cudaSuccess)
    rc = MKS_ERR_CUDA;
  if (rc >= 0 && cudaStreamSynchronize(c.stream) != cudaSuccess) rc = MKS_ERR_CUDA;
  dev_free(tot);
  if (rc >= 0) rc = red_check();
  return rc;
}

// ------------------------------------------------------------------ link update
__device__ __forceinline__ M3<double> uncompress_ah(const double *m) {
  M3<double> A;
  A.e[0][1] = {m[0], m[1]};
  A.e[0][2] = {m[2], m[3]};
  A.e[1][2] = {m[4], m[5]};
  A.e[1][0] = {-m[0], m[1]};
  A.e[2][0] = {-m[2], m[3]};
  A.e[2][1] = {-m[4], m[5]};
  A.e[0][0] = {0.0, m[6]};
  A.e[1][1] = {0.0, m[7]};
  A.e[2][2] = {0.0, m[8]};
  return A;
}

// U <- exp(eps H) U to eighth order: U + eps H (U + eps/2 H (U + ...))
__global__ void __launch_bounds__(128) k_update_u(Geom g, double2 *U, const double *mom, double eps) {
  const int h = blockIdx.x * blockDim.x + threadIdx.x, par = blockIdx.y, mu = blockIdx.z;
  if (h >= g.Vh) return;
  const MatF Um = link_dir(U, mu, g.Vh);
  const M3<double> link = Um.ld(par, h, g.Vh);
  const M3<double> H = uncompress_ah(mom + (((size_t)par * g.Vh + h) * 4 + mu) * 10);
  M3<double> T = link;
  for (int o = 8; o >= 1; o--) {
    const M3<double> HT = mm_nn(H, T);
    const double f = eps / (double)o;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        T.e[i][j].re = link.e[i][j].re + f * HT.e[i][j].re;
        T.e[i][j].im = link.e[i][j].im + f * HT.e[i][j].im;
      }
  }
  Um.st(par, h, g.Vh, T);
}

// reunit_su3 with the phases taken out and put back (reunitarize_ks)
__global__ void __launch_bounds__(128) k_reunit(Geom g, double2 *U) {
  const int h = blockIdx.x * blockDim.x + threadIdx.x, par = blockIdx.y, mu = blockIdx.z;
  if (h >= g.Vh) return;
  int c[4];
  site_coords(g, par, h, c[0], c[1], c[2], c[3]);
  const double ph = stag_phase(g, c, mu);
  const MatF Um = link_dir(U, mu, g.Vh);
  M3<double> m = Um.ld(par, h, g.Vh);
  double n0 = 0;
#pragma unroll
  for (int j = 0; j < 3; j++) {
    m.e[0][j].re *= ph; m.e[0][j].im *= ph; m.e[1][j].re *= ph; m.e[1][j].im *= ph;
    n0 += m.e[0][j].re * m.e[0][j].re + m.e[0][j].im * m.e[0][j].im;
  }
  n0 = 1.0 / sqrt(n0);
  double ar = 0, ai = 0;
#pragma unroll
  for (int j = 0; j < 3; j++) {
    m.e[0][j].re *= n0; m.e[0][j].im *= n0;
    ar += m.e[0][j].re * m.e[1][j].re + m.e[0][j].im * m.e[1][j].im;
    ai += m.e[0][j].re * m.e[1][j].im - m.e[0][j].im * m.e[1][j].re;
  }
  double n1 = 0;
#pragma unroll
  for (int j = 0; j < 3; j++) {
    m.e[1][j].re -= ar * m.e[0][j].re - ai * m.e[0][j].im;
    m.e[1][j].im -= ar * m.e[0][j].im + ai * m.e[0][j].re;
    n1 += m.e[1][j].re * m.e[1][j].re + m.e[1][j].im * m.e[1][j].im;
  }
  n1 = 1.0 / sqrt(n1);
#pragma unroll
  for (int j = 0; j < 3; j++) { m.e[1][j].re *= n1; m.e[1][j].im *= n1; }
#pragma unroll
  for (int j = 0; j < 3; j++) {
    const int a = (j + 1) % 3, b = (j + 2) % 3;
    const double re = m.e[0][a].re * m.e[1][b].re - m.e[0][a].im * m.e[1][b].im -
                      (m.e[0][b].re * m.e[1][a].re - m.e[0][b].im * m.e[1][a].im);
    const double im = m.e[0][a].re * m.e[1][b].im + m.e[0][a].im * m.e[1][b].re -
                      (m.e[0][b].re * m.e[1][a].im + m.e[0][b].im * m.e[1][a].re);
    m.e[2][j] = {re, -im};
  }
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) { m.e[i][j].re *= ph; m.e[i][j].im *= ph; }
  Um.st(par, h, g.Vh, m);
}

// ------------------------------------------------------------------ RNG
// MILC's site generator (ranstuff.c, 64-bit congruence variant): a 7-word
// feedback shift register XOR a 64-bit linear congruential generator
struct SitePrn {
  uint32_t r[7];
  uint32_t pad;
  unsigned long long mult, add, ic;
};

__device__ __forceinline__ double prn_rand(SitePrn &p) {
  const uint32_t t = (((p.r[5] >> 7) | (p.r[6] << 17)) ^ ((p.r[4] >> 1) | (p.r[5] << 23))) & 0xffffffu;
#pragma unroll
  for (int k = 6; k > 0; k--) p.r[k] = p.r[k - 1];
  p.r[0] = t;
  const unsigned long long s = p.ic * p.mult + p.add;
  p.ic = s;
  return (double)(t ^ (uint32_t)((s >> 40) & 0xffffffull)) * (1.0 / 16777216.0);
}

// polar Box-Muller pair, (v2 fac, v1 fac) (gaussrand.c:90-100)
__device__ __forceinline__ void prn_cgauss(SitePrn &p, double &re, double &im) {
  double v1, v2, r;
  do {
    v1 = 2.0 * prn_rand(p) - 1.0;
    v2 = 2.0 * prn_rand(p) - 1.0;
    r = v1 * v1 + v2 * v2;
  } while (r >= 1.0);
  const double fac = sqrt(-log(r) / r);
  re = v2 * fac;
  im = v1 * fac;
}

__global__ void k_prn_init(Geom g, SitePrn *prn, int seed) {
  const int h = blockIdx.x * blockDim.x + threadIdx.x, par = blockIdx.y;
  if (h >= g.Vh) return;
  int x, y, z, t;
  site_coords(g, par, h, x, y, z, t);
  const int index = x + g.nx * (y + g.ny * (z + g.nz * t));
  uint32_t s = (uint32_t)seed;
  const uint32_t a = (uint32_t)(69607 + 8 * index);
  SitePrn p;
#pragma unroll
  for (int k = 0; k < 7; k++) {
    s = a * s + 12345u;
    p.r[k] = ((uint32_t)((int32_t)s >> 8)) & 0xffffffu;
  }
  s = a * s + 12345u;
  p.pad = 0;
  p.ic = (unsigned long long)(long long)(int32_t)s;
  p.mult = 100000005ull + 8ull * (unsigned long long)index;
  p.add = 12345ull;
  prn[(size_t)par * g.Vh + h] = p;
}

// random_anti_hermitian per direction (rand_ahmat.c:38-52)
__global__ void k_ranmom(Geom g, SitePrn *prn, double *mom) {
  const int h = blockIdx.x * blockDim.x + threadIdx.x, par = blockIdx.y;
  if (h >= g.Vh) return;
  const size_t i = (size_t)par * g.Vh + h;
  SitePrn p = prn[i];
  const double sqrt_third = sqrt(1.0 / 3.0);
  for (int d = 0; d < 4; d++) {
    double *m = mom + (i * 4 + d) * 10;
    double r, s;
    prn_cgauss(p, r, s);
    m[6] = r + sqrt_third * s;
    m[7] = -r + sqrt_third * s;
    m[8] = -2.0 * sqrt_third * s;
    prn_cgauss(p, m[0], m[1]);
    prn_cgauss(p, m[2], m[3]);
    prn_cgauss(p, m[4], m[5]);
    m[9] = 0.0;
  }
  prn[i] = p;
}

// three complex Gaussians per site of the parities in `mask` (AoS [V][6])
__global__ void k_gauss_vec(Geom g, SitePrn *prn, int mask, double *v) {
  const int h = blockIdx.x * blockDim.x + threadIdx.x, par = blockIdx.y;
  if (h >= g.Vh) return;
  if (!(mask & (par == 0 ? MKS_EVEN : MKS_ODD))) return;
  const size_t i = (size_t)par * g.Vh + h;
  SitePrn p = prn[i];
  double *q = v + i * 6;
  prn_cgauss(p, q[0], q[1]);
  prn_cgauss(p, q[2], q[3]);
  prn_cgauss(p, q[4], q[5]);
  prn[i] = p;
}

// out = a[0] src + sum_j a[j+1] x_j on the sites of `par` (AoS [V][6])
constexpr int LINCOMB_MAX = 32;
struct LinComb {
  const double *src;
  const double *x[LINCOMB_MAX];
  double a[LINCOMB_MAX + 1];
  int n;
};
__global__ void k_lincomb(Geom g, int par, LinComb lc, double *out) {
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= g.Vh) return;
  const size_t i = ((size_t)par * g.Vh + h) * 6;
  double acc[6];
#pragma unroll
  for (int k = 0; k < 6; k++) acc[k] = lc.a[0] * lc.src[i + k];
  for (int j = 0; j < lc.n; j++)
#pragma unroll
    for (int k = 0; k < 6; k++) acc[k] = fma(lc.a[j + 1], lc.x[j][i + k], acc[k]);
#pragma unroll
  for (int k = 0; k < 6; k++) out[i + k] = acc[k];
}

// ------------------------------------------------------------------ host side
static SitePrn *g_prn = nullptr;
static size_t g_prn_sites = 0;
static float2 *g_u32 = nullptr;  // unphased FP32 thin links for the FP32 gauge force
static size_t g_u32_sites = 0;

static int ensure_mom() {
  Context &c = ctx();
  if (!c.mom) {
    MKS_TRY(dev_alloc((void **)&c.mom, c.V * 40 * sizeof(double)));
    MKS_CUDA(cudaMemsetAsync(c.mom, 0, c.V * 40 * sizeof(double), c.stream));
  }
  return MKS_OK;
}

static int ensure_thin() {
  Context &c = ctx();
  if (!c.auxU) {
    const size_t nall = 8 * 9 * c.Vh;
    MKS_TRY(dev_alloc((void **)&c.auxU, nall * sizeof(double2)));
    MKS_TRY(dev_alloc((void **)&c.auxV, nall * sizeof(double2)));
    MKS_TRY(dev_alloc((void **)&c.auxW, nall * sizeof(double2)));
  }
  return MKS_OK;
}

// the resident thin links changed: fermion links built from them are stale
static void thin_changed() {
  Context &c = ctx();
  for (int i = 0; i < MKS_MAX_SLOTS; i++) c.slots[i].valid = false;
  c.aux_action = 0;
}

static dim3 link_grid() { return dim3(grid_for(ctx().Vh, 128), 2, 4); }

int gauge_force_dev(double eps, double beta, double u0, int nflavors, int prec) {
  Context &c = ctx();
  MKS_TRY(upload_paths(nflavors, u0));
  timing_begin(MKS_K_GAUGE);
  if (prec == MKS_PREC_DOUBLE) {
    k_gauge_force<double><<<link_grid(), 128, 0, c.stream>>>(c.geom, c.auxU, nullptr, c.mom, eps * beta / 3.0);
  } else {
    if (g_u32_sites != c.V) {
      dev_free(g_u32);
      g_u32 = nullptr;
      g_u32_sites = 0;
      MKS_TRY(dev_alloc((void **)&g_u32, c.V * 36 * sizeof(float2)));
      g_u32_sites = c.V;
    }
    k_thin_to_f32<<<link_grid(), 128, 0, c.stream>>>(c.geom, c.auxU, g_u32);
    k_gauge_force<float><<<link_grid(), 128, 0, c.stream>>>(c.geom, c.auxU, g_u32, c.mom, eps * beta / 3.0);
  }
  timing_end(MKS_K_GAUGE);
  MKS_CUDA(cudaGetLastError());
  return MKS_OK;
}

int gauge_action_dev(double beta, double u0, int nflavors, double *action) {
  Context &c = ctx();
  MKS_TRY(upload_paths(nflavors, u0));
  double tot[2];
  MKS_TRY((site_sum<OpGaugeAction, 1>(OpGaugeAction{c.geom, c.auxU}, 2, tot)));
  *action = beta / 3.0 * (tot[0] + tot[1]);
  return MKS_OK;
}

int mom_action_dev(double *h) {
  Context &c = ctx();
  double tot[2];
  MKS_TRY((site_sum<OpMomAction, 1>(OpMomAction{(int)c.Vh, c.mom}, 2, tot)));
  *h = tot[0] + tot[1];
  return MKS_OK;
}

int plaquette_dev(double *ss, double *st) {
  Context &c = ctx();
  double tot[4];
  MKS_TRY((site_sum<OpPlaquette, 2>(OpPlaquette{c.geom, c.auxU}, 2, tot)));
  *ss = (tot[0] + tot[2]) / (3.0 * (double)c.V);
  *st = (tot[1] + tot[3]) / (3.0 * (double)c.V);
  return MKS_OK;
}

int update_u_dev(double eps) {
  Context &c = ctx();
  timing_begin(MKS_K_GAUGE);
  k_update_u<<<link_grid(), 128, 0, c.stream>>>(c.geom, c.auxU, c.mom, eps);
  timing_end(MKS_K_GAUGE);
  MKS_CUDA(cudaGetLastError());
  thin_changed();
  return MKS_OK;
}

int reunitarize_dev() {
  Context &c = ctx();
  timing_begin(MKS_K_GAUGE);
  k_reunit<<<link_grid(), 128, 0, c.stream>>>(c.geom, c.auxU);
  timing_end(MKS_K_GAUGE);
  MKS_CUDA(cudaGetLastError());
  thin_changed();
  return MKS_OK;
}

int ranmom_dev() {
  Context &c = ctx();
  if (!g_prn || g_prn_sites != c.V) return MKS_ERR_STATE;
  MKS_TRY(ensure_mom());
  timing_begin(MKS_K_GAUGE);
  k_ranmom<<<dim3(grid_for(c.Vh, 128), 2), 128, 0, c.stream>>>(c.geom, g_prn, c.mom);
  timing_end(MKS_K_GAUGE);
  MKS_CUDA(cudaGetLastError());
  return MKS_OK;
}

int gauss_vec_dev(int parity, double *v_dev) {
  Context &c = ctx();
  if (!g_prn || g_prn_sites != c.V) return MKS_ERR_STATE;
  timing_begin(MKS_K_GAUGE);
  k_gauss_vec<<<dim3(grid_for(c.Vh, 128), 2), 128, 0, c.stream>>>(c.geom, g_prn, parity, v_dev);
  timing_end(MKS_K_GAUGE);
  MKS_CUDA(cudaGetLastError());
  return MKS_OK;
}

int norm2_aos_dev(const double *v_dev, int par, double *out) {
  Context &c = ctx();
  double tot;
  MKS_TRY((site_sum<OpNormAos, 1>(OpNormAos{(int)c.Vh, par, v_dev}, 1, &tot)));
  *out = tot;
  return MKS_OK;
}

int lincomb_aos_dev(int par, const double *src, const double *const *x, const double *a, int n, double *out) {
  Context &c = ctx();
  if (n < 0 || n > LINCOMB_MAX) return MKS_ERR_ARG;
  LinComb lc;
  memset(&lc, 0, sizeof lc);
  lc.src = src;
  lc.n = n;
  lc.a[0] = a[0];
  for (int j = 0; j < n; j++) { lc.x[j] = x[j]; lc.a[j + 1] = a[j + 1]; }
  timing_begin(MKS_K_GAUGE);
  k_lincomb<<<grid_for(c.Vh, 128), 128, 0, c.stream>>>(c.geom, par, lc, out);
  timing_end(MKS_K_GAUGE);
  MKS_CUDA(cudaGetLastError());
  return MKS_OK;
}

int prn_seed_dev(int seed) {
  Context &c = ctx();
  if (g_prn_sites != c.V) {
    dev_free(g_prn);
    g_prn = nullptr;
    g_prn_sites = 0;
    MKS_TRY(dev_alloc((void **)&g_prn, c.V * sizeof(SitePrn)));
    g_prn_sites = c.V;
  }
  k_prn_init<<<dim3(grid_for(c.Vh, 128), 2), 128, 0, c.stream>>>(c.geom, g_prn, seed);
  c.launches++;
  MKS_CUDA(cudaGetLastError());
  return MKS_OK;
}

void gauge_free() {
  dev_free(g_prn);
  g_prn = nullptr;
  g_prn_sites = 0;
  dev_free(g_u32);
  g_u32 = nullptr;
  g_u32_sites = 0;
}

static int host_io(double *host, double *dev, size_t bytes, bool up) {
  Context &c = ctx();
  MKS_CUDA(cudaMemcpyAsync(up ? dev : host, up ? host : dev, bytes,
                           up ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost, c.stream));
  MKS_CUDA(cudaStreamSynchronize(c.stream));
  return MKS_OK;
}

// thin links in MILC's host layout without phases <-> resident (phased SoA)
int gauge_load_host(const double *thin_unphased) {
  Context &c = ctx();
  MKS_TRY(ensure_thin());
  const size_t bytes = c.V * 72 * sizeof(double);
  std::vector<double> tmp(thin_unphased, thin_unphased + c.V * 72);
  MKS_TRY(mks_apply_phases(c.dims, tmp.data(), 1));
  double *stage = nullptr;
  MKS_TRY(dev_alloc((void **)&stage, bytes));
  int rc = host_io(tmp.data(), stage, bytes, true);
  if (rc >= 0) rc = links_aos_to_soa64(stage, c.auxU);
  if (rc >= 0 && cudaStreamSynchronize(c.stream) != cudaSuccess) rc = MKS_ERR_CUDA;
  dev_free(stage);
  thin_changed();
  return rc;
}

int gauge_get_host(double *thin_unphased) {
  Context &c = ctx();
  if (!c.auxU) return MKS_ERR_STATE;
  const size_t bytes = c.V * 72 * sizeof(double);
  double *stage = nullptr;
  MKS_TRY(dev_alloc((void **)&stage, bytes));
  int rc = links_soa64_to_aos(c.auxU, stage);
  if (rc >= 0) rc = host_io(thin_unphased, stage, bytes, false);
  dev_free(stage);
  if (rc >= 0) rc = mks_apply_phases(c.dims, thin_unphased, 1);
  return rc;
}

}  // namespace mks

using namespace mks;

extern "C" {

int mks_gauge_load(const double *thin) {
  MKS_TRY(check_ready());
  if (!thin) return MKS_ERR_ARG;
  return gauge_load_host(thin);
}

int mks_gauge_get(double *thin) {
  MKS_TRY(check_ready());
  if (!thin) return MKS_ERR_ARG;
  return gauge_get_host(thin);
}

int mks_mom_load(const double *mom) {
  MKS_TRY(check_ready());
  if (!mom) return MKS_ERR_ARG;
  MKS_TRY(ensure_mom());
  return host_io(const_cast<double *>(mom), ctx().mom, ctx().V * 40 * sizeof(double), true);
}

int mks_mom_get(double *mom) {
  MKS_TRY(check_ready());
  if (!mom) return MKS_ERR_ARG;
  if (!ctx().mom) return MKS_ERR_STATE;
  return host_io(mom, ctx().mom, ctx().V * 40 * sizeof(double), false);
}

int mks_rng_seed(int iseed) {
  MKS_TRY(check_ready());
  return prn_seed_dev(iseed);
}

int mks_ranmom(void) {
  MKS_TRY(check_ready());
  return ranmom_dev();
}

int mks_gaussian_vector(int parity, double *v) {
  MKS_TRY(check_ready());
  if (!v || parity < MKS_ODD || parity > MKS_EVENANDODD) return MKS_ERR_ARG;
  Context &c = ctx();
  const size_t bytes = c.V * 6 * sizeof(double);
  double *dv = nullptr;
  MKS_TRY(dev_alloc((void **)&dv, bytes));
  int rc = host_io(v, dv, bytes, true);
  if (rc >= 0) rc = gauss_vec_dev(parity, dv);
  if (rc >= 0) rc = host_io(v, dv, bytes, false);
  dev_free(dv);
  return rc;
}

int mks_gauge_force(double eps, double beta, double u0, int nflavors) {
  return mks_gauge_force_prec(eps, beta, u0, nflavors, MKS_PREC_DOUBLE);
}

int mks_gauge_force_prec(double eps, double beta, double u0, int nflavors, int prec) {
  MKS_TRY(check_ready());
  if (prec != MKS_PREC_DOUBLE && prec != MKS_PREC_SINGLE) return MKS_ERR_ARG;
  if (!ctx().auxU) return MKS_ERR_STATE;
  MKS_TRY(ensure_mom());
  return gauge_force_dev(eps, beta, u0, nflavors, prec);
}

int mks_gauge_action(double beta, double u0, int nflavors, double *action) {
  MKS_TRY(check_ready());
  if (!action) return MKS_ERR_ARG;
  if (!ctx().auxU) return MKS_ERR_STATE;
  return gauge_action_dev(beta, u0, nflavors, action);
}

int mks_update_u(double eps) {
  MKS_TRY(check_ready());
  if (!ctx().auxU) return MKS_ERR_STATE;
  MKS_TRY(ensure_mom());
  return update_u_dev(eps);
}

int mks_mom_action(double *h) {
  MKS_TRY(check_ready());
  if (!h) return MKS_ERR_ARG;
  if (!ctx().mom) return MKS_ERR_STATE;
  return mom_action_dev(h);
}

int mks_reunitarize(void) {
  MKS_TRY(check_ready());
  if (!ctx().auxU) return MKS_ERR_STATE;
  return reunitarize_dev();
}

int mks_md_precision(int prec) {
  MKS_TRY(check_ready());
  if (prec != MKS_PREC_DOUBLE && prec != MKS_PREC_SINGLE) return MKS_ERR_ARG;
  ctx().md_prec = prec;
  return MKS_OK;
}

int mks_plaquette(double *ss, double *st) {
  MKS_TRY(check_ready());
  if (!ss || !st) return MKS_ERR_ARG;
  if (!ctx().auxU) return MKS_ERR_STATE;
  return plaquette_dev(ss, st);
}

}  // extern "C"
