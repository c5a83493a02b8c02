// mks_links.cu -- HISQ and asqtad fermion-link construction on the GPU.
//
// Replaces load_hisq_aux_links / load_hisq_fn_links
// (generic_ks/fermion_links_hisq_load_milc.c:547-640) and the asqtad
// fattening (generic_ks/fermion_links_fn_load_milc.c:52-271):
//   V = fat7(U)                            staple recursion, level-1 table
//   W = V (V^dag V)^(-1/2)                 analytic U(3) projection
//                                          (generic_ks/su3_mat_op.c:828,
//                                          Hasenfratz-Hoffmann-Schaefer 2007)
//   X = asqtad+2xLepage(W), L = c_naik W W W   level-2 table
//   X_i = X + eps_i (1/8 W), L_i = L + eps_i (-1/24) W W W   (Naik groups)
// The fattening follows the optimised staple recursion of
// load_fatlinks_cpu (ASQ_OPTIMIZED_FATTENING): one generalised staple
//   S(x) = U_nu(x) A(x+nu) U_nu(x+mu)^dag + U_nu(x-nu)^dag A(x-nu) U_nu(x-nu+mu)
// per launch (generic/general_staple.c:42-140).  FP64 fields and
// arithmetic, except in the molecular-dynamics FP32 setting
// (mks_md_precision): there the thin links are copied to FP32 and every
// smearing stage, the U(3) projection included, is stored and computed in
// FP32, while the resident V, W and the slots' fat / long links stay FP64
// fields (holding the FP32 results).
//
// All link fields use the SoA layout of mks_internal.cuh: [par][dir][9][Vh].
#include <cmath>
#include <cstring>
#include <vector>
#include "mks_internal.cuh"
#include "mks_su3.cuh"

namespace mks {


// out = a * in (all four directions, both parities)
template <typename T2>
__global__ void k_scale_links(const T2 *in, T2 *out, double a, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    typedef decltype(T2::x) E;
    const E ae = (E)a;
    T2 v = in[i];
    out[i] = {ae * v.x, ae * v.y};
  }
}
// out = x + a * y, into an FP64 field
template <typename T2>
__global__ void k_axpy_links(const T2 *x, const T2 *y, double2 *out, double a, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    T2 u = x[i], v = y[i];
    out[i] = make_double2((double)u.x + a * (double)v.x, (double)u.y + a * (double)v.y);
  }
}

// L_mu(x) = coef * W_mu(x) W_mu(x+mu) W_mu(x+2mu)   (load_lnglinks: the Naik path)
template <typename R>
__global__ void __launch_bounds__(128) k_naik(Geom g, const typename Stor<R>::t *W, typename Stor<R>::t *lng,
                                              double coef) {
  typedef typename Stor<R>::t T2;
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  const int par = blockIdx.y, mu = blockIdx.z;
  const int Vh = g.Vh;
  if (h >= Vh) return;
  MatT<R> Wm = link_dir((T2 *)W, mu, Vh), Lm = link_dir(lng, mu, Vh);
  const int x1 = nbr(g, par, h, mu, 1), x2 = nbr(g, par, h, mu, 2);
  M3<R> p = tnn<R>(Wm.ld(par, h, Vh), tnn<R>(Wm.ld(1 - par, x1, Vh), Wm.ld(par, x2, Vh)));
  const R c = (R)coef;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) { p.e[i][j].re *= c; p.e[i][j].im *= c; }
  Lm.st(par, h, Vh, p);
}

// W = V (V^dag V)^(-1/2), analytic (u3_unitarize_analytic, generic_ks/su3_mat_op.c:828-1200).
// Counts the links where MILC's HISQ_REUNIT_ALLOW_SVD criteria (1e-8) would
// switch to its SVD branch (in FP64 arithmetic).
template <typename A>
__device__ void u3_unitarize(const M3<A> &V, M3<A> &W, unsigned int *nsvd) {
  M3<A> Q = tan_<A>(V, V), Q2 = tnn<A>(Q, Q);
  A gv[3];
  herm3_eigvals<A>(Q, Q2, gv);
  const A g0 = gv[0], g1 = gv[1], g2 = gv[2];
  // det V for the SVD criterion (FP64 constructions only: the 1e-8 relative
  // test is below FP32 resolution)
  if (sizeof(A) == 8) {
    const cplx<A>(*e)[3] = V.e;
    cplx<A> a1 = {e[1][1].re * e[2][2].re - e[1][1].im * e[2][2].im - e[1][2].re * e[2][1].re + e[1][2].im * e[2][1].im,
                       e[1][1].re * e[2][2].im + e[1][1].im * e[2][2].re - e[1][2].re * e[2][1].im - e[1][2].im * e[2][1].re};
    cplx<A> a2 = {e[1][0].re * e[2][2].re - e[1][0].im * e[2][2].im - e[1][2].re * e[2][0].re + e[1][2].im * e[2][0].im,
                       e[1][0].re * e[2][2].im + e[1][0].im * e[2][2].re - e[1][2].re * e[2][0].im - e[1][2].im * e[2][0].re};
    cplx<A> a3 = {e[1][0].re * e[2][1].re - e[1][0].im * e[2][1].im - e[1][1].re * e[2][0].re + e[1][1].im * e[2][0].im,
                       e[1][0].re * e[2][1].im + e[1][0].im * e[2][1].re - e[1][1].re * e[2][0].im - e[1][1].im * e[2][0].re};
    A dre = e[0][0].re * a1.re - e[0][0].im * a1.im - e[0][1].re * a2.re + e[0][1].im * a2.im + e[0][2].re * a3.re - e[0][2].im * a3.im;
    A dim = e[0][0].im * a1.re + e[0][0].re * a1.im - e[0][1].im * a2.re - e[0][1].re * a2.im + e[0][2].im * a3.re + e[0][2].re * a3.im;
    A det = dre * dre + dim * dim;
    bool svd = (det != 0 && fabs(det - g0 * g1 * g2) / fabs(det) > (A)1e-8) || det < (A)1e-8;
    if (svd && nsvd) atomicAdd(nsvd, 1u);
  }
  A g0sq = sqrt(g0), g1sq = sqrt(g1), g2sq = sqrt(g2);
  A us = g1sq + g2sq, ws = g1sq * g2sq;
  A vs = g0sq * us + ws;
  us += g0sq;
  ws *= g0sq;
  A denom = ws * (us * vs - ws);
  A f0 = (us * vs * vs - ws * (us * us + vs)) / denom;
  A f1 = (2 * us * vs - ws - us * us * us) / denom;
  A f2 = us / denom;
  M3<A> S2;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      S2.e[i][j].re = f1 * Q.e[i][j].re + f2 * Q2.e[i][j].re + (i == j ? f0 : (A)0);
      S2.e[i][j].im = f1 * Q.e[i][j].im + f2 * Q2.e[i][j].im;
    }
  W = tnn<A>(V, S2);
}

// W = V (V^dag V)^(-1/2) for V stored in precision R, arithmetic in R (MILC's
// single-precision build projects in float too); W stored into W64 and
// (when given) Wr, V copied to V64 (when given)
template <typename R>
__global__ void __launch_bounds__(128) k_unitarize(Geom g, const typename Stor<R>::t *Vl, double2 *V64, double2 *W,
                                                   typename Stor<R>::t *Wr, unsigned int *nsvd) {
  typedef typename Stor<R>::t T2;
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  const int par = blockIdx.y, mu = blockIdx.z;
  if (h >= g.Vh) return;
  MatT<R> Vm = link_dir((T2 *)Vl, mu, g.Vh);
  MatF Wm = link_dir(W, mu, g.Vh);
  const M3<R> v = Vm.ld(par, h, g.Vh);
  M3<R> w;
  u3_unitarize<R>(v, w, nsvd);
  M3<double> w64, v64;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      w64.e[i][j] = {(double)w.e[i][j].re, (double)w.e[i][j].im};
      v64.e[i][j] = {(double)v.e[i][j].re, (double)v.e[i][j].im};
    }
  Wm.st(par, h, g.Vh, w64);
  if (V64) link_dir(V64, mu, g.Vh).st(par, h, g.Vh, v64);
  if (Wr) link_dir(Wr, mu, g.Vh).st(par, h, g.Vh, w);
}

struct FatCoeffs { double one_link, naik, three_staple, five_staple, seven_staple, lepage; };

// the smearing stages with fields stored and multiplied in precision R
template <typename R>
struct Smear {
  typedef typename Stor<R>::t T2;

  static int launch_staple(int mu, int nu, MatT<R> Unu, MatT<R> A, MatT<R> fat, double coef, MatT<R> sout) {
    Context &c = ctx();
    timing_begin(MKS_K_LINKS);
    k_staple<R><<<dim3(grid_for(c.Vh, 128), 2), 128, 0, c.stream>>>(c.geom, mu, nu, Unu, A, fat, coef, sout);
    timing_end(MKS_K_LINKS);
    MKS_CUDA(cudaGetLastError());
    return MKS_OK;
  }

  // load_fatlinks_cpu, ASQ_OPTIMIZED_FATTENING (fermion_links_fn_load_milc.c:207-253)
  static int fatten(T2 *links, const FatCoeffs &cf, T2 *fat, T2 *staple, T2 *tmp) {
    Context &c = ctx();
    size_t Vh = c.Vh, nall = 8 * 9 * Vh;
    double one_link = cf.one_link - 6.0 * cf.lepage;
    timing_begin(MKS_K_LINKS);
    k_scale_links<T2><<<c.sm_count * 8, 256, 0, c.stream>>>(links, fat, one_link, nall);
    timing_end(MKS_K_LINKS);
    MKS_CUDA(cudaGetLastError());
    if (cf.three_staple == 0.0 && cf.lepage == 0.0 && cf.five_staple == 0.0) return MKS_OK;
    MatT<R> none = {nullptr, 0};
    for (int mu = 0; mu < 4; mu++) {
      MatT<R> Fm = link_dir(fat, mu, Vh), Um = link_dir(links, mu, Vh);
      for (int nu = 0; nu < 4; nu++) {
        if (nu == mu) continue;
        MatT<R> Un = link_dir(links, nu, Vh);
        MatT<R> S = mat_field(staple, Vh), T = mat_field(tmp, Vh);
        MKS_TRY(launch_staple(mu, nu, Un, Um, Fm, cf.three_staple, S));
        if (cf.lepage != 0.0) MKS_TRY(launch_staple(mu, nu, Un, S, Fm, cf.lepage, none));
        for (int rho = 0; rho < 4; rho++) {
          if (rho == mu || rho == nu) continue;
          MatT<R> Ur = link_dir(links, rho, Vh);
          MKS_TRY(launch_staple(mu, rho, Ur, S, Fm, cf.five_staple, T));
          for (int sig = 0; sig < 4; sig++) {
            if (sig == mu || sig == nu || sig == rho) continue;
            MatT<R> Us = link_dir(links, sig, Vh);
            MKS_TRY(launch_staple(mu, sig, Us, T, Fm, cf.seven_staple, none));
          }
        }
      }
    }
    return MKS_OK;
  }

  static int naik(T2 *W, T2 *lng, double coef) {
    Context &c = ctx();
    timing_begin(MKS_K_LINKS);
    k_naik<R><<<dim3(grid_for(c.Vh, 128), 2, 4), 128, 0, c.stream>>>(c.geom, W, lng, coef);
    timing_end(MKS_K_LINKS);
    MKS_CUDA(cudaGetLastError());
    return MKS_OK;
  }

  static int unitarize(T2 *Vl, double2 *V64, double2 *W, T2 *Wr, unsigned int *nsvd) {
    Context &c = ctx();
    timing_begin(MKS_K_LINKS);
    k_unitarize<R><<<dim3(grid_for(c.Vh, 128), 2, 4), 128, 0, c.stream>>>(c.geom, Vl, V64, W, Wr, nsvd);
    timing_end(MKS_K_LINKS);
    MKS_CUDA(cudaGetLastError());
    return MKS_OK;
  }

  static int to_f64(const T2 *x, double2 *y, size_t n) {
    Context &c = ctx();
    timing_begin(MKS_K_LINKS);
    k_convert<double2, T2><<<c.sm_count * 8, 256, 0, c.stream>>>(x, y, n);
    timing_end(MKS_K_LINKS);
    MKS_CUDA(cudaGetLastError());
    return MKS_OK;
  }
};

// the FP64 entry points of the MILC-facing loaders
static int fatten(double2 *links, const FatCoeffs &cf, double2 *fat, double2 *staple, double2 *tmp) {
  return Smear<double>::fatten(links, cf, fat, staple, tmp);
}
static int naik(double2 *W, double2 *lng, double coef) { return Smear<double>::naik(W, lng, coef); }

static unsigned int g_nsvd = 0;

int links_from_thin(int action, const double *thin_dev_aos, int n_naiks, const double *eps_naik, double u0) {
  Context &c = ctx();
  size_t nall = 8 * 9 * c.Vh;
  if (!c.auxU) {
    MKS_TRY(dev_alloc((void **)&c.auxU, nall * sizeof(double2)));
    MKS_TRY(dev_alloc((void **)&c.auxV, nall * sizeof(double2)));
    MKS_TRY(dev_alloc((void **)&c.auxW, nall * sizeof(double2)));
  }
  MKS_TRY(links_aos_to_soa64(thin_dev_aos, c.auxU));
  return links_from_aux(action, n_naiks, eps_naik, u0);
}

// fat/long links of slots 0..n_naiks-1 built from the resident thin links
// auxU, smearing in precision R (the field pointers of the stages are the
// resident FP64 fields for FP64, FP32 scratch copies otherwise)
template <typename R>
static int build_links(int action, int n_naiks, const double *eps_naik, double u0) {
  typedef typename Stor<R>::t T2;
  constexpr bool low = sizeof(R) < 8;
  Context &c = ctx();
  size_t Vh = c.Vh, nall = 8 * 9 * Vh;
  for (int i = 0; i < n_naiks; i++) {
    LinkSlot &s = c.slots[i];
    if (!s.fat64) {
      MKS_TRY(dev_alloc((void **)&s.fat64, nall * sizeof(double2)));
      MKS_TRY(dev_alloc((void **)&s.lng64, nall * sizeof(double2)));
    }
  }
  // staple, tmp; FP32: U, V, W, fat, long copies; Naik groups: f3, l3
  const size_t nscr = 2 * 2 * 9 * Vh + (low ? 5 * nall : 0) + (n_naiks > 1 ? 2 * nall : 0);
  T2 *scr = nullptr;
  MKS_TRY(dev_alloc((void **)&scr, nscr * sizeof(T2)));
  T2 *staple = scr, *tmp = staple + 2 * 9 * Vh, *p = tmp + 2 * 9 * Vh;
  T2 *Ucp = nullptr, *Vcp = nullptr, *Wcp = nullptr, *Fcp = nullptr, *Lcp = nullptr, *f3 = nullptr, *l3 = nullptr;
  if (low) { Ucp = p; Vcp = p + nall; Wcp = p + 2 * nall; Fcp = p + 3 * nall; Lcp = p + 4 * nall; p += 5 * nall; }
  if (n_naiks > 1) { f3 = p; l3 = p + nall; }
  unsigned int *nsvd = nullptr;
  int rc = dev_alloc((void **)&nsvd, sizeof(unsigned int));
  LinkSlot &s0 = c.slots[0];
  typedef Smear<R> Sm;
  do {
    if (rc < 0) break;
    if (cudaMemsetAsync(nsvd, 0, sizeof(unsigned int), c.stream) != cudaSuccess) { rc = MKS_ERR_CUDA; break; }
    T2 *U = (T2 *)c.auxU;
    if constexpr (low) {
      timing_begin(MKS_K_LINKS);
      k_convert<T2, double2><<<c.sm_count * 8, 256, 0, c.stream>>>(c.auxU, Ucp, nall);
      timing_end(MKS_K_LINKS);
      U = Ucp;
    }
    T2 *F = low ? Fcp : (T2 *)s0.fat64, *L = low ? Lcp : (T2 *)s0.lng64;
    if (action == MKS_ACTION_HISQ) {
      // generic_ks/imp_actions/hisq/hisq_u3_action.h: path_coeff_1 / _2 / _3 (no tadpole factors)
      const FatCoeffs c1 = {1.0 / 8.0, 0.0, -1.0 / 16.0, 1.0 / 64.0, -1.0 / 384.0, 0.0};
      const FatCoeffs c2 = {1.0 / 8.0 + 2.0 * 6.0 / 16.0 + 1.0 / 8.0, -1.0 / 24.0, -1.0 / 16.0, 1.0 / 64.0,
                            -1.0 / 384.0, -2.0 / 16.0};
      const FatCoeffs c3 = {1.0 / 8.0, -1.0 / 24.0, 0, 0, 0, 0};
      T2 *Vf = low ? Vcp : (T2 *)c.auxV, *W = low ? Wcp : (T2 *)c.auxW;
      if ((rc = Sm::fatten(U, c1, Vf, staple, tmp)) < 0) break;
      if ((rc = Sm::unitarize(Vf, low ? c.auxV : nullptr, c.auxW, low ? Wcp : nullptr, nsvd)) < 0) break;
      if ((rc = Sm::fatten(W, c2, F, staple, tmp)) < 0) break;
      if ((rc = Sm::naik(W, L, c2.naik)) < 0) break;
      if (n_naiks > 1) {
        if ((rc = Sm::fatten(W, c3, f3, staple, tmp)) < 0) break;
        if ((rc = Sm::naik(W, l3, c3.naik)) < 0) break;
        for (int i = 1; i < n_naiks; i++) {
          LinkSlot &s = c.slots[i];
          k_axpy_links<T2><<<c.sm_count * 8, 256, 0, c.stream>>>(F, f3, s.fat64, eps_naik[i], nall);
          k_axpy_links<T2><<<c.sm_count * 8, 256, 0, c.stream>>>(L, l3, s.lng64, eps_naik[i], nall);
          c.launches += 2;
        }
      }
    } else {
      // asqtad_action.h with the tadpole division of ks_action_paths.c
      const double u2 = u0 * u0, u4 = u2 * u2, u6 = u4 * u2;
      const FatCoeffs ca = {1.0 / 8.0 + 6.0 / 16.0 + 1.0 / 8.0, -1.0 / 24.0 / u2, -1.0 / 16.0 / u2, 1.0 / 64.0 / u4,
                            -1.0 / 384.0 / u6, -1.0 / 16.0 / u4};
      if ((rc = Sm::fatten(U, ca, F, staple, tmp)) < 0) break;
      if ((rc = Sm::naik(U, L, ca.naik)) < 0) break;
      n_naiks = 1;
    }
    if constexpr (low) {
      if ((rc = Sm::to_f64(F, s0.fat64, nall)) < 0) break;
      if ((rc = Sm::to_f64(L, s0.lng64, nall)) < 0) break;
    }
    for (int i = 0; i < n_naiks && rc >= 0; i++) {
      LinkSlot &s = c.slots[i];
      rc = links_make_lowprec(s);
      s.eps_naik = eps_naik ? eps_naik[i] : 0.0;
      s.valid = true;
    }
    if (rc < 0) break;
    c.aux_action = action;
    c.aux_u0 = u0;
    c.links_prec = low ? MKS_PREC_SINGLE : MKS_PREC_DOUBLE;
    if (cudaMemcpyAsync(&g_nsvd, nsvd, sizeof(unsigned int), cudaMemcpyDeviceToHost, c.stream) != cudaSuccess)
      rc = MKS_ERR_CUDA;
    if (rc >= 0 && cudaStreamSynchronize(c.stream) != cudaSuccess) rc = MKS_ERR_CUDA;
  } while (0);
  cudaStreamSynchronize(c.stream);
  dev_free(nsvd);
  dev_free(scr);
  return rc;
}

int links_from_aux(int action, int n_naiks, const double *eps_naik, double u0) {
  if (!ctx().auxU) return MKS_ERR_STATE;
  if (ctx().md_prec == MKS_PREC_SINGLE) return build_links<float>(action, n_naiks, eps_naik, u0);
  return build_links<double>(action, n_naiks, eps_naik, u0);
}

}  // namespace mks

using namespace mks;

extern "C" {

int mks_load_links_from_thin(int action, const double *thin, int n_naiks, const double *eps_naik, double u0) {
  MKS_TRY(check_ready());
  if (!thin || (action != MKS_ACTION_HISQ && action != MKS_ACTION_ASQTAD)) return MKS_ERR_ARG;
  if (n_naiks < 1 || n_naiks > MKS_MAX_SLOTS || (n_naiks > 1 && !eps_naik) || !(u0 > 0)) return MKS_ERR_ARG;
  Context &c = ctx();
  size_t bytes = c.V * 4 * 18 * sizeof(double);
  double *tmp;
  MKS_TRY(dev_alloc((void **)&tmp, bytes));
  MKS_CUDA(cudaMemcpyAsync(tmp, thin, bytes, cudaMemcpyHostToDevice, c.stream));
  int rc = links_from_thin(action, tmp, n_naiks, eps_naik, u0);
  cudaStreamSynchronize(c.stream);
  dev_free(tmp);
  return rc;
}

int mks_rebuild_links(int action, int n_naiks, const double *eps_naik, double u0) {
  MKS_TRY(check_ready());
  if (action != MKS_ACTION_HISQ && action != MKS_ACTION_ASQTAD) return MKS_ERR_ARG;
  if (n_naiks < 1 || n_naiks > MKS_MAX_SLOTS || (n_naiks > 1 && !eps_naik) || !(u0 > 0)) return MKS_ERR_ARG;
  if (!ctx().auxU) return MKS_ERR_STATE;
  return links_from_aux(action, n_naiks, eps_naik, u0);
}

int mks_hisq_reunit_svd_count(void) { return (int)g_nsvd; }

int mks_get_hisq_aux(double *V, double *W) {
  MKS_TRY(check_ready());
  Context &c = ctx();
  if (!c.auxW) return MKS_ERR_STATE;
  size_t bytes = c.V * 4 * 18 * sizeof(double);
  double *tmp;
  MKS_TRY(dev_alloc((void **)&tmp, bytes));
  if (V) {
    MKS_TRY(links_soa64_to_aos(c.auxV, tmp));
    MKS_CUDA(cudaMemcpyAsync(V, tmp, bytes, cudaMemcpyDeviceToHost, c.stream));
    MKS_CUDA(cudaStreamSynchronize(c.stream));
  }
  if (W) {
    MKS_TRY(links_soa64_to_aos(c.auxW, tmp));
    MKS_CUDA(cudaMemcpyAsync(W, tmp, bytes, cudaMemcpyDeviceToHost, c.stream));
    MKS_CUDA(cudaStreamSynchronize(c.stream));
  }
  dev_free(tmp);
  return MKS_OK;
}

}  // extern "C"

// --------------------------------------------------------------------
// Generic-coefficient entry points, one per MILC loader the drop-in
// replaces (generic_ks/fermion_links_fn_load_gpu.c:19-110).
namespace mks {

static int ensure_aux() {
  Context &c = ctx();
  size_t nall = 8 * 9 * c.Vh;
  if (!c.auxU) {
    MKS_TRY(dev_alloc((void **)&c.auxU, nall * sizeof(double2)));
    MKS_TRY(dev_alloc((void **)&c.auxV, nall * sizeof(double2)));
    MKS_TRY(dev_alloc((void **)&c.auxW, nall * sizeof(double2)));
  }
  return MKS_OK;
}

static int to_host(const double2 *soa, double *host, double *stage) {
  Context &c = ctx();
  MKS_TRY(links_soa64_to_aos(soa, stage));
  MKS_CUDA(cudaMemcpyAsync(host, stage, c.V * 72 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  MKS_CUDA(cudaStreamSynchronize(c.stream));
  return MKS_OK;
}

}  // namespace mks

extern "C" {

int mks_fatlong_links(const double coeffs[6], const double *links, double *fat, double *lng) {
  MKS_TRY(check_ready());
  if (!coeffs || !links || (!fat && !lng)) return MKS_ERR_ARG;
  Context &c = ctx();
  const size_t Vh = c.Vh, nall = 8 * 9 * Vh, bytes = c.V * 72 * sizeof(double);
  const FatCoeffs cf = {coeffs[0], coeffs[1], coeffs[2], coeffs[3], coeffs[4], coeffs[5]};
  double *stage = nullptr;
  double2 *L = nullptr, *F = nullptr, *S = nullptr, *T = nullptr;
  int rc = dev_alloc((void **)&stage, bytes);
  if (rc >= 0) rc = dev_alloc((void **)&L, nall * sizeof(double2));
  if (rc >= 0) rc = dev_alloc((void **)&F, nall * sizeof(double2));
  if (rc >= 0) rc = dev_alloc((void **)&S, 2 * 9 * Vh * sizeof(double2));
  if (rc >= 0) rc = dev_alloc((void **)&T, 2 * 9 * Vh * sizeof(double2));
  if (rc >= 0 && cudaMemcpyAsync(stage, links, bytes, cudaMemcpyHostToDevice, c.stream) != cudaSuccess)
    rc = MKS_ERR_CUDA;
  if (rc >= 0) rc = links_aos_to_soa64(stage, L);
  if (rc >= 0 && fat) rc = fatten(L, cf, F, S, T);
  if (rc >= 0 && fat) rc = to_host(F, fat, stage);
  if (rc >= 0 && lng) rc = naik(L, F, cf.naik);
  if (rc >= 0 && lng) rc = to_host(F, lng, stage);
  cudaStreamSynchronize(c.stream);
  dev_free(stage); dev_free(L); dev_free(F); dev_free(S); dev_free(T);
  return rc;
}

int mks_hisq_aux_links(const double coeffs1[6], const double *U, double *V, double *W) {
  MKS_TRY(check_ready());
  if (!coeffs1 || !U) return MKS_ERR_ARG;
  Context &c = ctx();
  const size_t Vh = c.Vh, bytes = c.V * 72 * sizeof(double);
  const FatCoeffs cf = {coeffs1[0], coeffs1[1], coeffs1[2], coeffs1[3], coeffs1[4], coeffs1[5]};
  MKS_TRY(ensure_aux());
  double *stage = nullptr;
  double2 *S = nullptr, *T = nullptr;
  unsigned int *nsvd = nullptr;
  int rc = dev_alloc((void **)&stage, bytes);
  if (rc >= 0) rc = dev_alloc((void **)&S, 2 * 9 * Vh * sizeof(double2));
  if (rc >= 0) rc = dev_alloc((void **)&T, 2 * 9 * Vh * sizeof(double2));
  if (rc >= 0) rc = dev_alloc((void **)&nsvd, sizeof(unsigned int));
  if (rc >= 0 && cudaMemsetAsync(nsvd, 0, sizeof(unsigned int), c.stream) != cudaSuccess) rc = MKS_ERR_CUDA;
  if (rc >= 0 && cudaMemcpyAsync(stage, U, bytes, cudaMemcpyHostToDevice, c.stream) != cudaSuccess)
    rc = MKS_ERR_CUDA;
  if (rc >= 0) rc = links_aos_to_soa64(stage, c.auxU);
  c.aux_action = MKS_ACTION_HISQ;
  c.aux_u0 = 1.0;
  if (rc >= 0) rc = fatten(c.auxU, cf, c.auxV, S, T);
  if (rc >= 0) rc = Smear<double>::unitarize(c.auxV, nullptr, c.auxW, nullptr, nsvd);
  if (rc >= 0 && cudaMemcpyAsync(&g_nsvd, nsvd, sizeof(unsigned int), cudaMemcpyDeviceToHost, c.stream) != cudaSuccess)
    rc = MKS_ERR_CUDA;
  if (rc >= 0 && V) rc = to_host(c.auxV, V, stage);
  if (rc >= 0 && W) rc = to_host(c.auxW, W, stage);
  cudaStreamSynchronize(c.stream);
  dev_free(stage); dev_free(S); dev_free(T); dev_free(nsvd);
  return rc;
}

int mks_load_hisq_aux(const double *U, const double *V, const double *W) {
  MKS_TRY(check_ready());
  if (!U || !V || !W) return MKS_ERR_ARG;
  Context &c = ctx();
  const size_t bytes = c.V * 72 * sizeof(double);
  MKS_TRY(ensure_aux());
  double *stage = nullptr;
  MKS_TRY(dev_alloc((void **)&stage, bytes));
  const double *src[3] = {U, V, W};
  double2 *dst[3] = {c.auxU, c.auxV, c.auxW};
  c.aux_action = MKS_ACTION_HISQ;
  c.aux_u0 = 1.0;
  int rc = MKS_OK;
  for (int k = 0; k < 3 && rc >= 0; k++) {
    if (cudaMemcpyAsync(stage, src[k], bytes, cudaMemcpyHostToDevice, c.stream) != cudaSuccess) rc = MKS_ERR_CUDA;
    if (rc >= 0) rc = links_aos_to_soa64(stage, dst[k]);
    if (rc >= 0 && cudaStreamSynchronize(c.stream) != cudaSuccess) rc = MKS_ERR_CUDA;
  }
  dev_free(stage);
  return rc;
}

}  // extern "C"
