// mks_force.cu -- the HISQ fermion force as a hand-written adjoint kernel set.
//
// Replaces eo_fermion_force_multi / fn_fermion_force_multi_hisq_wrapper_mx
// (generic_ks/fermion_force_hisq_multi.c:170-219, :1182-1475).  For
//   S = sum_j res_j phi^dag (sigma_j - D_eo D_oe)^-1 phi
// and a link-like field Z, write dS = 2 Re sum tr(K_Z dZ).  The kernels
// run the link construction of mks_links.cu backwards:
//   1. K_fat, K_lng from the outer products of the rational-function
//      solutions (level 0; generic_ks/fermion_force_hisq_multi.c:1478-1635):
//      K(z) = s(z) res_j xxx_j(z+mu) xxx_j(z)^dag (z+3mu for Naik),
//      s = +1 on even and -1 on odd z
//   2. K_W: reverse of the level-2 staple recursion and the Naik product
//      (every term), plus eps_i times the reverse of (1-link + Naik) for the
//      terms of Naik group i
//   3. K_V: reverse of the analytic U(3) projection W = V (V^dag V)^-1/2,
//      with MILC's eigenvalue filter (generic_ks/su3_mat_op.c:1680-1734)
//   4. K_U: reverse of the fat7 staple recursion
//   5. mom_mu(x) <- TA(mom_mu(x) + 2 eps U_mu(x) K_U(x))
// The staple intermediates (S1 = staple of U_mu, S2 = staple of S1) are
// recomputed inside the reverse sweep instead of being stored for all
// (mu, nu, rho).  Every adjoint kernel is a gather: a thread owns one site
// of the accumulated field and pulls the contributions of its neighbours,
// so nothing is written by two threads.
#include <cmath>
#include <cstring>
#include <vector>
#include "mks_internal.cuh"
#include "mks_su3.cuh"

namespace mks {

// d += f s in precision R
template <typename R>
__device__ __forceinline__ void macc(M3<R> &d, const M3<R> &s, R f) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) { d.e[i][j].re += f * s.e[i][j].re; d.e[i][j].im += f * s.e[i][j].im; }
}
template <typename R>
__device__ __forceinline__ M3<double> to64(const M3<R> &a) {
  M3<double> c;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) c.e[i][j] = {(double)a.e[i][j].re, (double)a.e[i][j].im};
  return c;
}
template <typename R>
__device__ __forceinline__ M3<R> from64(const M3<double> &a) {
  M3<R> c;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) c.e[i][j] = {(R)a.e[i][j].re, (R)a.e[i][j].im};
  return c;
}

// 1. level-0 outer products for terms [j0, j1), scaled by `scale`
template <typename R>
struct OuterArgs {
  const typename Stor<R>::t *x[64];   // full-lattice SoA [2][3][Vh] per term
  double res[64];
  int j0, j1;
  double scale;
};
template <typename R>
__global__ void __launch_bounds__(128) k_outer(Geom g, OuterArgs<R> a, typename Stor<R>::t *Kf,
                                               typename Stor<R>::t *Kl) {
  typedef typename Stor<R>::t T2;
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  const int par = blockIdx.y, mu = blockIdx.z;
  const int Vh = g.Vh;
  if (h >= Vh) return;
  const int y1 = nbr(g, par, h, mu, 1), y3 = nbr(g, par, h, mu, 3);
  const double s = par == 0 ? a.scale : -a.scale;
  MatT<R> F = link_dir(Kf, mu, Vh), L = link_dir(Kl, mu, Vh);
  M3<R> kf = F.ld(par, h, Vh), kl = L.ld(par, h, Vh);
  for (int j = a.j0; j < a.j1; j++) {
    const T2 *x = a.x[j];
    const R r = (R)(s * a.res[j]);
    cplx<R> b[3], u1[3], u3[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      T2 q = x[((size_t)par * 3 + c) * Vh + h];
      b[c] = {q.x, q.y};
      q = x[((size_t)(1 - par) * 3 + c) * Vh + y1];
      u1[c] = {q.x, q.y};
      q = x[((size_t)(1 - par) * 3 + c) * Vh + y3];
      u3[c] = {q.x, q.y};
    }
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int k = 0; k < 3; k++) {
        // (u b^dag)_ik = u_i conj(b_k)
        kf.e[i][k].re += r * (u1[i].re * b[k].re + u1[i].im * b[k].im);
        kf.e[i][k].im += r * (u1[i].im * b[k].re - u1[i].re * b[k].im);
        kl.e[i][k].re += r * (u3[i].re * b[k].re + u3[i].im * b[k].im);
        kl.e[i][k].im += r * (u3[i].im * b[k].re - u3[i].re * b[k].im);
      }
  }
  F.st(par, h, Vh, kf);
  L.st(par, h, Vh, kl);
}

// 2/4. reverse of one staple S(x) = U_nu(x) A(x+nu) U_nu(x+mu)^dag + U_nu(x-nu)^dag A(x-nu) U_nu(x-nu+mu)
// given its adjoint K (scaled by f):
//   KA(y)    += U_nu(y-nu+mu)^dag K(y-nu) U_nu(y-nu) + U_nu(y+mu) K(y+nu) U_nu(y)^dag
//   KUnu(y)  += A(y+nu) U_nu(y+mu)^dag K(y) + A(y-mu+nu)^dag U_nu(y-mu)^dag K(y-mu)^dag
//             + K(y+nu)^dag U_nu(y+mu)^dag A(y)^dag + K(y+nu-mu) U_nu(y-mu)^dag A(y-mu)
// Fields stored and products computed in precision R.
template <typename R>
__global__ void __launch_bounds__(128) k_staple_adj(Geom g, int mu, int nu, MatT<R> Unu, MatT<R> A, MatT<R> K,
                                                    double f, MatT<R> KA, MatT<R> KU) {
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  const int par = blockIdx.y, op = 1 - par;
  const int Vh = g.Vh;
  if (h >= Vh) return;
  const int ymnu = nbr(g, par, h, nu, -1), ypnu = nbr(g, par, h, nu, 1), ypmu = nbr(g, par, h, mu, 1);
  const int ymmu = nbr(g, par, h, mu, -1);
  const int ymnupmu = nbr2(g, par, h, nu, -1, mu, 1), ypnummu = nbr2(g, par, h, nu, 1, mu, -1);
  const M3<R> Uy = Unu.ld(par, h, Vh);
  const M3<R> Uypmu = Unu.ld(op, ypmu, Vh);
  const M3<R> Uymmu = Unu.ld(op, ymmu, Vh);
  const R fr = (R)f;
  // KA
  {
    const M3<R> Uymnu = Unu.ld(op, ymnu, Vh);
    const M3<R> Uymnupmu = Unu.ld(par, ymnupmu, Vh);
    M3<R> acc = tnn<R>(tan_<R>(Uymnupmu, K.ld(op, ymnu, Vh)), Uymnu);
    const M3<R> t = tna<R>(tnn<R>(Uypmu, K.ld(op, ypnu, Vh)), Uy);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) { acc.e[i][j].re += t.e[i][j].re; acc.e[i][j].im += t.e[i][j].im; }
    M3<R> out = KA.ld(par, h, Vh);
    macc<R>(out, acc, fr);
    KA.st(par, h, Vh, out);
  }
  // KU_nu
  {
    const M3<R> Ky = K.ld(par, h, Vh), Ay = A.ld(par, h, Vh);
    M3<R> acc = tnn<R>(tna<R>(A.ld(op, ypnu, Vh), Uypmu), Ky);                                       // T1
    tacc<R>(acc, tadj<R>(tnn<R>(K.ld(op, ymmu, Vh), tnn<R>(Uymmu, A.ld(par, ypnummu, Vh)))), (R)1);  // T2 = (K U A)^dag
    tacc<R>(acc, tadj<R>(tnn<R>(Ay, tnn<R>(Uypmu, K.ld(op, ypnu, Vh)))), (R)1);                      // T3 = (A U K)^dag
    tacc<R>(acc, tnn<R>(tna<R>(K.ld(par, ypnummu, Vh), Uymmu), A.ld(op, ymmu, Vh)), (R)1);           // T4
    M3<R> out = KU.ld(par, h, Vh);
    macc<R>(out, acc, fr);
    KU.st(par, h, Vh, out);
  }
}

// reverse of L_mu(x) = c W_mu(x) W_mu(x+mu) W_mu(x+2mu):
//   KW(y) += c [W(y+mu) W(y+2mu) K(y) + W(y+mu) K(y-mu) W(y-mu) + K(y-2mu) W(y-2mu) W(y-mu)]
template <typename R>
__global__ void __launch_bounds__(128) k_naik_adj(Geom g, const typename Stor<R>::t *W, const typename Stor<R>::t *Kl,
                                                  typename Stor<R>::t *KW, double c) {
  typedef typename Stor<R>::t T2;
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  const int par = blockIdx.y, mu = blockIdx.z, op = 1 - par;
  const int Vh = g.Vh;
  if (h >= Vh) return;
  MatT<R> Wm = link_dir((T2 *)W, mu, Vh), Km = link_dir((T2 *)Kl, mu, Vh), Om = link_dir(KW, mu, Vh);
  const int p1 = nbr(g, par, h, mu, 1), p2 = nbr(g, par, h, mu, 2), m1 = nbr(g, par, h, mu, -1), m2 = nbr(g, par, h, mu, -2);
  const M3<R> Wp1 = Wm.ld(op, p1, Vh), Wm1 = Wm.ld(op, m1, Vh);
  const R cr = (R)c;
  M3<R> acc = Om.ld(par, h, Vh);
  macc<R>(acc, tnn<R>(tnn<R>(Wp1, Wm.ld(par, p2, Vh)), Km.ld(par, h, Vh)), cr);
  macc<R>(acc, tnn<R>(tnn<R>(Wp1, Km.ld(op, m1, Vh)), Wm1), cr);
  macc<R>(acc, tnn<R>(tnn<R>(Km.ld(par, m2, Vh), Wm.ld(par, m2, Vh)), Wm1), cr);
  Om.st(par, h, Vh, acc);
}

// 3. reverse of W = V (V^dag V)^-1/2.  With Q = V^dag V, R = Q^-1/2 =
// f0 + f1 Q + f2 Q^2 (f_i rational in u = sum s_a, v = sum_{a<b} s_a s_b,
// w = s0 s1 s2, s_a^2 the eigenvalues of Q) and du = tr(R dQ)/2,
// dv = tr((u R - 1) dQ)/2, dw = (w/2) tr(R^2 dQ):
//   K_V = R K_W + (N + N^dag) V^dag,  M = K_W V,
//   N = sum_i tr(M Q^i) Psi_i + f1 M + f2 (Q M + M Q),
//   Psi_i = df_i/du R/2 + df_i/dv (u R - 1)/2 + df_i/dw (w/2) R^2.
// Arithmetic and the storage of K_W, K_V in precision S (MILC's own
// single-precision build runs this derivative in float too); V is the
// resident FP64 field.
template <typename S>
__global__ void __launch_bounds__(128) k_unit_adj(Geom g, const double2 *Vl, const typename Stor<S>::t *KW,
                                                  typename Stor<S>::t *KV, unsigned int *nfilter) {
  typedef typename Stor<S>::t T2;
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  const int par = blockIdx.y, mu = blockIdx.z;
  const int Vh = g.Vh;
  if (h >= Vh) return;
  MatF Vm = link_dir((double2 *)Vl, mu, Vh);
  MatT<S> Kw = link_dir((T2 *)KW, mu, Vh), Kv = link_dir(KV, mu, Vh);
  const M3<S> V = from64<S>(Vm.ld(par, h, Vh));
  M3<S> Q = tan_<S>(V, V), Q2 = tnn<S>(Q, Q);
  S gv[3];
  herm3_eigvals<S>(Q, Q2, gv);
  S gmin = fmin(gv[0], fmin(gv[1], gv[2]));
  if (gmin < (S)5.0e-5) {  // HISQ_FORCE_FILTER
    if (nfilter) atomicAdd(nfilter, 1u);
    for (int a = 0; a < 3; a++) gv[a] += (S)5.0e-5;
    for (int i = 0; i < 3; i++) Q.e[i][i].re += (S)5.0e-5;
    Q2 = tnn<S>(Q, Q);
  }
  const S s0 = sqrt(gv[0]), s1 = sqrt(gv[1]), s2 = sqrt(gv[2]);
  const S u = s0 + s1 + s2, v = s0 * s1 + s0 * s2 + s1 * s2, w = s0 * s1 * s2;
  const S D = w * (u * v - w);
  const S f0 = (u * v * v - w * (u * u + v)) / D, f1 = (2 * u * v - w - u * u * u) / D, f2 = u / D;
  const S Du = v * w, Dv = u * w, Dw = u * v - 2 * w;
  S fu[3], fv[3], fw[3];
  fu[0] = (v * v - 2 * u * w) / D - f0 * Du / D;
  fv[0] = (2 * u * v - w) / D - f0 * Dv / D;
  fw[0] = (-u * u - v) / D - f0 * Dw / D;
  fu[1] = (2 * v - 3 * u * u) / D - f1 * Du / D;
  fv[1] = (2 * u) / D - f1 * Dv / D;
  fw[1] = (S)-1 / D - f1 * Dw / D;
  fu[2] = (S)1 / D - f2 * Du / D;
  fv[2] = -f2 * Dv / D;
  fw[2] = -f2 * Dw / D;
  M3<S> R;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      R.e[i][j].re = f1 * Q.e[i][j].re + f2 * Q2.e[i][j].re + (i == j ? f0 : (S)0);
      R.e[i][j].im = f1 * Q.e[i][j].im + f2 * Q2.e[i][j].im;
    }
  const M3<S> R2 = tnn<S>(R, R);
  const M3<S> Kwv = Kw.ld(par, h, Vh);
  const M3<S> M = tnn<S>(Kwv, V);
  const M3<S> QM = tnn<S>(Q, M), MQ = tnn<S>(M, Q), MQ2 = tnn<S>(M, Q2);
  cplx<S> tr[3] = {{0, 0}, {0, 0}, {0, 0}};
#pragma unroll
  for (int a = 0; a < 3; a++) {
    tr[0].re += M.e[a][a].re; tr[0].im += M.e[a][a].im;
    tr[1].re += MQ.e[a][a].re; tr[1].im += MQ.e[a][a].im;
    tr[2].re += MQ2.e[a][a].re; tr[2].im += MQ2.e[a][a].im;
  }
  M3<S> N;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      N.e[i][j].re = f1 * M.e[i][j].re + f2 * (QM.e[i][j].re + MQ.e[i][j].re);
      N.e[i][j].im = f1 * M.e[i][j].im + f2 * (QM.e[i][j].im + MQ.e[i][j].im);
    }
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const S cu = (S)0.5 * fu[k] + (S)0.5 * fv[k] * u, cw = (S)0.5 * fw[k] * w, cd = (S)-0.5 * fv[k];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        S pr = cu * R.e[i][j].re + cw * R2.e[i][j].re + (i == j ? cd : (S)0);
        S pi = cu * R.e[i][j].im + cw * R2.e[i][j].im;
        N.e[i][j].re += tr[k].re * pr - tr[k].im * pi;
        N.e[i][j].im += tr[k].re * pi + tr[k].im * pr;
      }
  }
  M3<S> Nh;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      Nh.e[i][j].re = N.e[i][j].re + N.e[j][i].re;
      Nh.e[i][j].im = N.e[i][j].im - N.e[j][i].im;
    }
  M3<S> out = tnn<S>(R, Kwv);
  macc<S>(out, tna<S>(Nh, V), (S)1);
  Kv.st(par, h, Vh, out);
}

// 5. mom <- TA(mom + fac U K_U) in MILC's anti_hermitmat layout, device AoS [V][4][10]
template <typename S>
__global__ void __launch_bounds__(128) k_force_mom(Geom g, const double2 *U, const typename Stor<S>::t *KU,
                                                   double *mom, double fac) {
  typedef typename Stor<S>::t T2;
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  const int par = blockIdx.y, mu = blockIdx.z;
  const int Vh = g.Vh;
  if (h >= Vh) return;
  MatF Um = link_dir((double2 *)U, mu, Vh);
  MatT<S> Km = link_dir((T2 *)KU, mu, Vh);
  const M3<double> G = mm_nn(Um.ld(par, h, Vh), to64<S>(Km.ld(par, h, Vh)));
  double *m = mom + (((size_t)par * Vh + h) * 4 + mu) * 10;
  // uncompress, add, compress (libraries/uncmp_ahmat.c, make_ahmat.c)
  double a01r = m[0], a01i = m[1], a02r = m[2], a02i = m[3], a12r = m[4], a12i = m[5];
  double d0 = m[6] + fac * G.e[0][0].im, d1 = m[7] + fac * G.e[1][1].im, d2 = m[8] + fac * G.e[2][2].im;
  double t = (d0 + d1 + d2) * 0.33333333333333333;
  m[6] = d0 - t; m[7] = d1 - t; m[8] = d2 - t;
  m[0] = ((a01r + fac * G.e[0][1].re) - (-a01r + fac * G.e[1][0].re)) * 0.5;
  m[1] = ((a01i + fac * G.e[0][1].im) + (a01i + fac * G.e[1][0].im)) * 0.5;
  m[2] = ((a02r + fac * G.e[0][2].re) - (-a02r + fac * G.e[2][0].re)) * 0.5;
  m[3] = ((a02i + fac * G.e[0][2].im) + (a02i + fac * G.e[2][0].im)) * 0.5;
  m[4] = ((a12r + fac * G.e[1][2].re) - (-a12r + fac * G.e[2][1].re)) * 0.5;
  m[5] = ((a12i + fac * G.e[1][2].im) + (a12i + fac * G.e[2][1].im)) * 0.5;
}

struct ForceCoeffs { double one_link, naik, three_staple, five_staple, seven_staple, lepage; };

static double g_force_flops = 0.0;
static unsigned int g_nfilter = 0;

// The force runs in the molecular-dynamics precision: FP64 fields and
// arithmetic, or (MKS_PREC_SINGLE) every intermediate field -- the thin and
// W links, the staples and all adjoints -- stored and multiplied in FP32.
// The U(3)-projection adjoint keeps FP64 arithmetic and the momentum update
// FP64 fields.
template <typename R>
struct ForceRun {
  typedef typename Stor<R>::t T2;

  static int staple_fwd(int mu, int nu, MatT<R> Unu, MatT<R> A, MatT<R> S) {
    Context &c = ctx();
    MatT<R> none = {nullptr, 0};
    timing_begin(MKS_K_FORCE);
    k_staple<R><<<dim3(grid_for(c.Vh, 128), 2), 128, 0, c.stream>>>(c.geom, mu, nu, Unu, A, none, 0.0, S);
    timing_end(MKS_K_FORCE);
    g_force_flops += 4.0 * 198 * c.V;
    MKS_CUDA(cudaGetLastError());
    return MKS_OK;
  }

  static int staple_adj(int mu, int nu, MatT<R> Unu, MatT<R> A, MatT<R> K, double f, MatT<R> KA, MatT<R> KU) {
    Context &c = ctx();
    timing_begin(MKS_K_FORCE);
    k_staple_adj<R><<<dim3(grid_for(c.Vh, 128), 2), 128, 0, c.stream>>>(c.geom, mu, nu, Unu, A, K, f, KA, KU);
    timing_end(MKS_K_FORCE);
    g_force_flops += 12.0 * 198 * c.V;
    MKS_CUDA(cudaGetLastError());
    return MKS_OK;
  }

  static int axpby(const T2 *x, T2 *y, double a, double b, size_t n) {
    Context &c = ctx();
    timing_begin(MKS_K_FORCE);
    k_axpby_t<T2><<<c.sm_count * 8, 256, 0, c.stream>>>(x, y, a, b, n);
    timing_end(MKS_K_FORCE);
    MKS_CUDA(cudaGetLastError());
    return MKS_OK;
  }

  // reverse of the fat-link staple recursion (load_fatlinks_cpu, ASQ_OPTIMIZED_FATTENING):
  // KU += d fat(links) / d links contracted with Kfat
  static int fat_adj(T2 *links, const ForceCoeffs &cf, T2 *Kfat, T2 *KU, T2 *S1, T2 *S2, T2 *K1, T2 *K2) {
    Context &c = ctx();
    const size_t Vh = c.Vh, nm = 2 * 9 * Vh;
    const double one_link = cf.one_link - 6.0 * cf.lepage;
    MKS_TRY(axpby(Kfat, KU, one_link, 1.0, 8 * 9 * Vh));
    if (cf.three_staple == 0.0 && cf.lepage == 0.0 && cf.five_staple == 0.0) return MKS_OK;
    const MatT<R> mS1 = mat_field(S1, Vh), mS2 = mat_field(S2, Vh), mK1 = mat_field(K1, Vh), mK2 = mat_field(K2, Vh);
    for (int mu = 0; mu < 4; mu++) {
      const MatT<R> Kd = link_dir(Kfat, mu, Vh), Um = link_dir(links, mu, Vh), KUm = link_dir(KU, mu, Vh);
      for (int nu = 0; nu < 4; nu++) {
        if (nu == mu) continue;
        const MatT<R> Un = link_dir(links, nu, Vh), KUn = link_dir(KU, nu, Vh);
        MKS_TRY(staple_fwd(mu, nu, Un, Um, mS1));
        // K1 = c3 Kfat_mu
        MKS_CUDA(cudaMemsetAsync(K1, 0, nm * sizeof(T2), c.stream));
        for (int p = 0; p < 2; p++)
          MKS_TRY(axpby(Kd.p + p * Kd.ps, K1 + p * 9 * Vh, cf.three_staple, 1.0, 9 * Vh));
        if (cf.lepage != 0.0) MKS_TRY(staple_adj(mu, nu, Un, mS1, Kd, cf.lepage, mK1, KUn));
        for (int rho = 0; rho < 4; rho++) {
          if (rho == mu || rho == nu) continue;
          const MatT<R> Ur = link_dir(links, rho, Vh), KUr = link_dir(KU, rho, Vh);
          MKS_TRY(staple_fwd(mu, rho, Ur, mS1, mS2));
          MKS_CUDA(cudaMemsetAsync(K2, 0, nm * sizeof(T2), c.stream));
          for (int p = 0; p < 2; p++)
            MKS_TRY(axpby(Kd.p + p * Kd.ps, K2 + p * 9 * Vh, cf.five_staple, 1.0, 9 * Vh));
          for (int sig = 0; sig < 4; sig++) {
            if (sig == mu || sig == nu || sig == rho) continue;
            const MatT<R> Us = link_dir(links, sig, Vh), KUs = link_dir(KU, sig, Vh);
            MKS_TRY(staple_adj(mu, sig, Us, mS2, Kd, cf.seven_staple, mK2, KUs));
          }
          MKS_TRY(staple_adj(mu, rho, Ur, mS1, mK2, 1.0, mK1, KUr));
        }
        MKS_TRY(staple_adj(mu, nu, Un, Um, mK1, 1.0, KUm, KUn));
      }
    }
    return MKS_OK;
  }

  static int naik_adj(const T2 *W, const T2 *Kl, T2 *KW, double cn) {
    Context &c = ctx();
    timing_begin(MKS_K_FORCE);
    k_naik_adj<R><<<dim3(grid_for(c.Vh, 128), 2, 4), 128, 0, c.stream>>>(c.geom, W, Kl, KW, cn);
    timing_end(MKS_K_FORCE);
    g_force_flops += 4.0 * 6 * 198 * c.V;
    MKS_CUDA(cudaGetLastError());
    return MKS_OK;
  }

  static int outer(const OuterArgs<R> &a, T2 *Kf, T2 *Kl) {
    Context &c = ctx();
    timing_begin(MKS_K_FORCE);
    k_outer<R><<<dim3(grid_for(c.Vh, 128), 2, 4), 128, 0, c.stream>>>(c.geom, a, Kf, Kl);
    timing_end(MKS_K_FORCE);
    MKS_CUDA(cudaGetLastError());
    return MKS_OK;
  }

  template <typename TO, typename TI>
  static int convert(const TI *x, TO *y, size_t n) {
    Context &c = ctx();
    timing_begin(MKS_K_FORCE);
    k_convert<TO, TI><<<c.sm_count * 8, 256, 0, c.stream>>>(x, y, n);
    timing_end(MKS_K_FORCE);
    MKS_CUDA(cudaGetLastError());
    return MKS_OK;
  }

  // the FP64 resident field in precision R: the field itself for FP64, else
  // a converted copy at dst
  static int field_r(double2 *src, T2 *dst, size_t n, T2 **out) {
    if constexpr (sizeof(R) == 8) {
      (void)dst; (void)n;
      *out = src;
      return MKS_OK;
    } else {
      MKS_TRY((convert<T2, double2>(src, dst, n)));
      *out = dst;
      return MKS_OK;
    }
  }

  // K_U out: FP64 copy of the adjoint for ku_out, or the momentum update
  static int finish(double eps, T2 *KU, double *mom_dev, double2 *ku_out, T2 *scratch_unused) {
    Context &c = ctx();
    const size_t nl = 8 * 9 * c.Vh;
    (void)scratch_unused;
    if (ku_out) {
      if constexpr (sizeof(R) == 8) {
        MKS_CUDA(cudaMemcpyAsync(ku_out, KU, nl * sizeof(double2), cudaMemcpyDeviceToDevice, c.stream));
      } else {
        MKS_TRY((convert<double2, T2>(KU, ku_out, nl)));
      }
      MKS_CUDA(cudaStreamSynchronize(c.stream));
      return MKS_OK;
    }
    timing_begin(MKS_K_FORCE);
    k_force_mom<R><<<dim3(grid_for(c.Vh, 128), 2, 4), 128, 0, c.stream>>>(c.geom, c.auxU, KU, mom_dev, 2.0 * eps);
    timing_end(MKS_K_FORCE);
    MKS_CUDA(cudaGetLastError());
    MKS_CUDA(cudaStreamSynchronize(c.stream));
    return MKS_OK;
  }

  // force inputs in precision R: the FP64 SoA vectors themselves, or FP32 copies in xs32
  static int inputs(double2 *const *xs, int nterms, T2 *xs32, OuterArgs<R> &oa) {
    const size_t nv = 6 * ctx().Vh;
    for (int j = 0; j < nterms; j++) {
      if constexpr (sizeof(R) == 8) {
        (void)xs32; (void)nv;
        oa.x[j] = xs[j];
      } else {
        MKS_TRY((convert<T2, double2>(xs[j], xs32 + (size_t)j * nv, nv)));
        oa.x[j] = xs32 + (size_t)j * nv;
      }
    }
    return MKS_OK;
  }

  // xr: the inputs already in precision R (FP32 SoA), else converted from xs
  static int hisq(double eps, const double *residues, double2 *const *xs, int nterms, const int *orders, int n_naiks,
                  double *mom_dev, double2 *ku_out, T2 *const *xr = nullptr) {
    Context &c = ctx();
    const size_t Vh = c.Vh, nl = 8 * 9 * Vh, nm = 2 * 9 * Vh;
    const ForceCoeffs c1 = {1.0 / 8.0, 0.0, -1.0 / 16.0, 1.0 / 64.0, -1.0 / 384.0, 0.0};
    const ForceCoeffs c2 = {1.0 / 8.0 + 2.0 * 6.0 / 16.0 + 1.0 / 8.0, -1.0 / 24.0, -1.0 / 16.0, 1.0 / 64.0,
                            -1.0 / 384.0, -2.0 / 16.0};
    const ForceCoeffs c3 = {1.0 / 8.0, -1.0 / 24.0, 0, 0, 0, 0};
    const bool low = sizeof(R) < 8;
    // Kf Kl KW KV KU, S1 S2 K1 K2, and in FP32 the U and W copies and the inputs
    const size_t total = 5 * nl + 4 * nm + (low ? 2 * nl + (xr ? 0 : (size_t)nterms * 6 * Vh) : 0);
    T2 *buf = nullptr;
    MKS_TRY(dev_alloc((void **)&buf, total * sizeof(T2)));
    T2 *Kf = buf, *Kl = Kf + nl, *KW = Kl + nl, *KV = KW + nl, *KU = KV + nl;
    T2 *S1 = KU + nl, *S2 = S1 + nm, *K1 = S2 + nm, *K2 = K1 + nm;
    T2 *Ucp = K2 + nm, *Wcp = Ucp + nl, *xs32 = Wcp + nl;
    unsigned int *nfilt = nullptr;
    int rc = MKS_OK;
    do {
      if ((rc = dev_alloc((void **)&nfilt, sizeof(unsigned int))) < 0) break;
      cudaMemsetAsync(nfilt, 0, sizeof(unsigned int), c.stream);
      cudaMemsetAsync(buf, 0, 5 * nl * sizeof(T2), c.stream);
      T2 *U, *W;
      if ((rc = field_r(c.auxU, Ucp, nl, &U)) < 0) break;
      if ((rc = field_r(c.auxW, Wcp, nl, &W)) < 0) break;
      OuterArgs<R> oa;
      memset(&oa, 0, sizeof oa);
      if (xr) {
        for (int j = 0; j < nterms; j++) oa.x[j] = xr[j];
      } else if ((rc = inputs(xs, nterms, xs32, oa)) < 0) {
        break;
      }
      for (int j = 0; j < nterms; j++) oa.res[j] = residues[j];
      // level 2 with every term (the Naik group-0 table covers all terms)
      oa.j0 = 0; oa.j1 = nterms; oa.scale = 1.0;
      if ((rc = outer(oa, Kf, Kl)) < 0) break;
      if ((rc = fat_adj(W, c2, Kf, KW, S1, S2, K1, K2)) < 0) break;
      if ((rc = naik_adj(W, Kl, KW, c2.naik)) < 0) break;
      // Naik-epsilon groups: eps_g (1-link + Naik)(W) for their own terms
      int off = orders[0];
      for (int gi = 1; gi < n_naiks && rc >= 0; gi++) {
        cudaMemsetAsync(Kf, 0, 2 * nl * sizeof(T2), c.stream);
        oa.j0 = off; oa.j1 = off + orders[gi]; oa.scale = c.slots[gi].eps_naik;
        off += orders[gi];
        if ((rc = outer(oa, Kf, Kl)) < 0) break;
        if ((rc = fat_adj(W, c3, Kf, KW, S1, S2, K1, K2)) < 0) break;
        if ((rc = naik_adj(W, Kl, KW, c3.naik)) < 0) break;
      }
      if (rc < 0) break;
      timing_begin(MKS_K_FORCE);
      k_unit_adj<R><<<dim3(grid_for(Vh, 128), 2, 4), 128, 0, c.stream>>>(c.geom, c.auxV, KW, KV, nfilt);
      timing_end(MKS_K_FORCE);
      g_force_flops += 20.0 * 198 * c.V * 4;
      if (cudaGetLastError() != cudaSuccess) { rc = MKS_ERR_CUDA; break; }
      if ((rc = fat_adj(U, c1, KV, KU, S1, S2, K1, K2)) < 0) break;
      if ((rc = finish(eps, KU, mom_dev, ku_out, nullptr)) < 0) break;
      cudaMemcpyAsync(&g_nfilter, nfilt, sizeof(unsigned int), cudaMemcpyDeviceToHost, c.stream);
      if (cudaStreamSynchronize(c.stream) != cudaSuccess) rc = MKS_ERR_CUDA;
    } while (0);
    dev_free(nfilt);
    dev_free(buf);
    return rc;
  }

  // asqtad (generic_ks/fermion_force_fn_multi.c:80-316): one smearing
  // level, the fat and Naik links built from the thin links U with the
  // tadpole-improved coefficients and no projection, so K_U is the fat-link
  // adjoint plus the Naik adjoint of the level-0 outer products.
  static int asqtad(double eps, const double *residues, double2 *const *xs, int nterms, double *mom_dev,
                    double2 *ku_out) {
    Context &c = ctx();
    const size_t Vh = c.Vh, nl = 8 * 9 * Vh, nm = 2 * 9 * Vh;
    g_nfilter = 0;
    const double u2 = c.aux_u0 * c.aux_u0, u4 = u2 * u2, u6 = u4 * u2;
    // asqtad_action.h with the tadpole division of ks_action_paths.c
    const ForceCoeffs ca = {1.0 / 8.0 + 6.0 / 16.0 + 1.0 / 8.0, -1.0 / 24.0 / u2, -1.0 / 16.0 / u2, 1.0 / 64.0 / u4,
                            -1.0 / 384.0 / u6, -1.0 / 16.0 / u4};
    const bool low = sizeof(R) < 8;
    const size_t total = 3 * nl + 4 * nm + (low ? nl + (size_t)nterms * 6 * Vh : 0);
    T2 *buf = nullptr;
    MKS_TRY(dev_alloc((void **)&buf, total * sizeof(T2)));
    T2 *Kf = buf, *Kl = Kf + nl, *KU = Kl + nl;
    T2 *S1 = KU + nl, *S2 = S1 + nm, *K1 = S2 + nm, *K2 = K1 + nm;
    T2 *Ucp = K2 + nm, *xs32 = Ucp + nl;
    int rc = MKS_OK;
    do {
      if (cudaMemsetAsync(buf, 0, 3 * nl * sizeof(T2), c.stream) != cudaSuccess) { rc = MKS_ERR_CUDA; break; }
      T2 *U;
      if ((rc = field_r(c.auxU, Ucp, nl, &U)) < 0) break;
      OuterArgs<R> oa;
      memset(&oa, 0, sizeof oa);
      if ((rc = inputs(xs, nterms, xs32, oa)) < 0) break;
      for (int j = 0; j < nterms; j++) oa.res[j] = residues[j];
      oa.j0 = 0; oa.j1 = nterms; oa.scale = 1.0;
      if ((rc = outer(oa, Kf, Kl)) < 0) break;
      if ((rc = fat_adj(U, ca, Kf, KU, S1, S2, K1, K2)) < 0) break;
      if ((rc = naik_adj(U, Kl, KU, ca.naik)) < 0) break;
      rc = finish(eps, KU, mom_dev, ku_out, nullptr);
    } while (0);
    dev_free(buf);
    return rc;
  }
};

// mom_dev: momentum updated in place; or, with ku_out set, K_U itself
// (dS = 2 Re sum tr(K_U dU), [2][4][9][Vh] SoA) is copied there and mom_dev
// is not touched.
int force_dev(double eps, const double *residues, double2 *const *xs, int nterms, const int *orders, int n_naiks,
              double *mom_dev, double2 *ku_out) {
  g_force_flops = 0.0;
  if (ctx().md_prec == MKS_PREC_SINGLE)
    return ForceRun<float>::hisq(eps, residues, xs, nterms, orders, n_naiks, mom_dev, ku_out);
  return ForceRun<double>::hisq(eps, residues, xs, nterms, orders, n_naiks, mom_dev, ku_out);
}

int force_dev32(double eps, const double *residues, float2 *const *xs32, int nterms, const int *orders,
                int n_naiks, double *mom_dev) {
  g_force_flops = 0.0;
  if (ctx().md_prec != MKS_PREC_SINGLE) return MKS_ERR_STATE;
  return ForceRun<float>::hisq(eps, residues, nullptr, nterms, orders, n_naiks, mom_dev, nullptr, xs32);
}

int force_asqtad_dev(double eps, const double *residues, double2 *const *xs, int nterms, double *mom_dev,
                     double2 *ku_out) {
  g_force_flops = 0.0;
  if (ctx().md_prec == MKS_PREC_SINGLE)
    return ForceRun<float>::asqtad(eps, residues, xs, nterms, mom_dev, ku_out);
  return ForceRun<double>::asqtad(eps, residues, xs, nterms, mom_dev, ku_out);
}

// Host staging shared by the force entry points: xxx[j] (MILC AoS, both
// parities) to device SoA FP64, mom (anti_hermitmat[V][4]) to the device
// and back around run(xs, mom_dev).
template <class Run>
static int force_host(const double *const *xxx, int nterms, double *mom, const Run &run) {
  Context &c = ctx();
  const size_t vbytes = c.V * 6 * sizeof(double), mbytes = c.V * 40 * sizeof(double);
  double *stage = nullptr;
  double2 *xs = nullptr;
  double *mom_dev = nullptr;
  MKS_TRY(dev_alloc((void **)&stage, vbytes));
  int rc = dev_alloc((void **)&xs, (size_t)nterms * 6 * c.V * sizeof(double2) / 2);
  if (rc >= 0) rc = dev_alloc((void **)&mom_dev, mbytes);
  std::vector<double2 *> xp(nterms);
  for (int j = 0; j < nterms && rc >= 0; j++) {
    xp[j] = xs + (size_t)j * 6 * c.Vh;
    if (cudaMemcpyAsync(stage, xxx[j], vbytes, cudaMemcpyHostToDevice, c.stream) != cudaSuccess) rc = MKS_ERR_CUDA;
    if (rc >= 0) rc = vec_aos_to_soa64(stage, xp[j], 0);
    if (rc >= 0) rc = vec_aos_to_soa64(stage, xp[j] + 3 * c.Vh, 1);
    if (rc >= 0 && cudaStreamSynchronize(c.stream) != cudaSuccess) rc = MKS_ERR_CUDA;
  }
  if (rc >= 0 && cudaMemcpyAsync(mom_dev, mom, mbytes, cudaMemcpyHostToDevice, c.stream) != cudaSuccess)
    rc = MKS_ERR_CUDA;
  if (rc >= 0) rc = run(xp.data(), mom_dev);
  if (rc >= 0 && cudaMemcpyAsync(mom, mom_dev, mbytes, cudaMemcpyDeviceToHost, c.stream) != cudaSuccess)
    rc = MKS_ERR_CUDA;
  if (rc >= 0 && cudaStreamSynchronize(c.stream) != cudaSuccess) rc = MKS_ERR_CUDA;
  dev_free(stage); dev_free(xs); dev_free(mom_dev);
  return rc;
}

}  // namespace mks

using namespace mks;

extern "C" {

int mks_fermion_force_multi_hisq(double eps, const double *residues, const double *const *xxx, int nterms,
                                 const int *n_orders_naik, int n_naiks, double *mom) {
  MKS_TRY(check_ready());
  Context &c = ctx();
  if (!c.auxW) return MKS_ERR_STATE;
  if (nterms <= 0 || nterms > 64 || !residues || !xxx || !mom || !n_orders_naik) return MKS_ERR_ARG;
  if (n_naiks < 1 || n_naiks > MKS_MAX_SLOTS) return MKS_ERR_ARG;
  // n_orders_naik[g]: number of consecutive terms in Naik group g (MILC's
  // n_orders_naik[], ks_imp_rhmc/setup.c:295-339); they add up to nterms
  int tot = 0;
  for (int i = 0; i < n_naiks; i++) {
    if (n_orders_naik[i] < 0) return MKS_ERR_ARG;
    tot += n_orders_naik[i];
  }
  if (tot != nterms) return MKS_ERR_ARG;
  for (int i = 1; i < n_naiks; i++)
    if (!c.slots[i].valid) return MKS_ERR_STATE;
  if (c.aux_action != MKS_ACTION_HISQ) return MKS_ERR_STATE;
  return force_host(xxx, nterms, mom, [&](double2 *const *xs, double *mom_dev) {
    return force_dev(eps, residues, xs, nterms, n_orders_naik, n_naiks, mom_dev, nullptr);
  });
}

int mks_fermion_force_multi_asqtad(double eps, const double *residues, const double *const *xxx, int nterms,
                                   double *mom) {
  MKS_TRY(check_ready());
  Context &c = ctx();
  if (!c.auxU || c.aux_action != MKS_ACTION_ASQTAD) return MKS_ERR_STATE;
  if (nterms <= 0 || nterms > 64 || !residues || !xxx || !mom) return MKS_ERR_ARG;
  return force_host(xxx, nterms, mom, [&](double2 *const *xs, double *mom_dev) {
    return force_asqtad_dev(eps, residues, xs, nterms, mom_dev, nullptr);
  });
}

int mks_fermion_force_adjoint(const double *residues, const double *const *xxx, int nterms,
                              const int *n_orders_naik, int n_naiks, double *ku) {
  MKS_TRY(check_ready());
  Context &c = ctx();
  if (!c.auxU || (c.aux_action != MKS_ACTION_HISQ && c.aux_action != MKS_ACTION_ASQTAD)) return MKS_ERR_STATE;
  if (nterms <= 0 || nterms > 64 || !residues || !xxx || !ku) return MKS_ERR_ARG;
  const bool hisq = c.aux_action == MKS_ACTION_HISQ;
  std::vector<int> one(1, nterms);
  if (hisq) {
    if (n_naiks < 1 || n_naiks > MKS_MAX_SLOTS) return MKS_ERR_ARG;
    if (!n_orders_naik) {
      if (n_naiks != 1) return MKS_ERR_ARG;
      n_orders_naik = one.data();
    }
    int tot = 0;
    for (int i = 0; i < n_naiks; i++) {
      if (n_orders_naik[i] < 0) return MKS_ERR_ARG;
      tot += n_orders_naik[i];
    }
    if (tot != nterms) return MKS_ERR_ARG;
    for (int i = 1; i < n_naiks; i++)
      if (!c.slots[i].valid) return MKS_ERR_STATE;
  }
  const size_t nl = 8 * 9 * c.Vh;
  double2 *kd = nullptr;
  double *stage = nullptr, *mom = nullptr;
  MKS_TRY(dev_alloc((void **)&kd, nl * sizeof(double2)));
  int rc = dev_alloc((void **)&stage, nl * sizeof(double2));
  // force_host stages a momentum field; it is not used when K_U is asked for
  std::vector<double> mom_host;
  if (rc >= 0) { mom_host.assign(c.V * 40, 0.0); mom = mom_host.data(); }
  if (rc >= 0)
    rc = force_host(xxx, nterms, mom, [&](double2 *const *xs, double *mom_dev) {
      return hisq ? force_dev(1.0, residues, xs, nterms, n_orders_naik, n_naiks, mom_dev, kd)
                  : force_asqtad_dev(1.0, residues, xs, nterms, mom_dev, kd);
    });
  if (rc >= 0) rc = links_soa64_to_aos(kd, stage);
  if (rc >= 0 && cudaMemcpyAsync(ku, stage, nl * sizeof(double2), cudaMemcpyDeviceToHost, c.stream) != cudaSuccess)
    rc = MKS_ERR_CUDA;
  if (rc >= 0 && cudaStreamSynchronize(c.stream) != cudaSuccess) rc = MKS_ERR_CUDA;
  dev_free(kd); dev_free(stage);
  return rc;
}

double mks_force_flops_last(void) { return g_force_flops; }
int mks_force_filter_count(void) { return (int)g_nfilter; }

}  // extern "C"
