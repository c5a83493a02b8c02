// mks_su3.cuh -- 3x3 matrix helpers and link-field views (FP64 or FP32
// storage) shared by the link-construction and fermion-force kernels.
#pragma once
#include "mks_internal.cuh"

namespace mks {

// storage element of a complex number in precision R
template <typename R> struct Stor;
template <> struct Stor<double> { typedef double2 t; };
template <> struct Stor<float> { typedef float2 t; };

// a 3x3 matrix per site stored in precision R: element k of site (par,h)
// at p[par*ps + k*Vh + h]
template <typename R>
struct MatT {
  typedef typename Stor<R>::t T2;
  T2 *p;
  size_t ps;
  __device__ __forceinline__ M3<R> ld(int par, int h, int Vh) const {
    const T2 *b = p + par * ps + h;
    M3<R> m;
#pragma unroll
    for (int k = 0; k < 9; k++) { T2 a = b[(size_t)k * Vh]; m.e[k / 3][k % 3] = {a.x, a.y}; }
    return m;
  }
  __device__ __forceinline__ void st(int par, int h, int Vh, const M3<R> &m) const {
    T2 *b = p + par * ps + h;
#pragma unroll
    for (int k = 0; k < 9; k++) b[(size_t)k * Vh] = {m.e[k / 3][k % 3].re, m.e[k / 3][k % 3].im};
  }
};
typedef MatT<double> MatF;

// views of a link field [par][dir][9][Vh] (one direction) and of a single
// matrix field [par][9][Vh]
__host__ __device__ inline MatT<double> link_dir(double2 *base, int dir, size_t Vh) {
  return {base + (size_t)dir * 9 * Vh, 36 * Vh};
}
__host__ __device__ inline MatT<float> link_dir(float2 *base, int dir, size_t Vh) {
  return {base + (size_t)dir * 9 * Vh, 36 * Vh};
}
__host__ __device__ inline MatT<double> mat_field(double2 *base, size_t Vh) { return {base, 9 * Vh}; }
__host__ __device__ inline MatT<float> mat_field(float2 *base, size_t Vh) { return {base, 9 * Vh}; }

// y = a x + b y, and precision conversions, over n complex numbers
template <typename T2>
__global__ void k_axpby_t(const T2 *x, T2 *y, double a, double b, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    typedef decltype(T2::x) E;
    const E ae = (E)a, be = (E)b;
    T2 u = x[i], v = y[i];
    y[i] = {ae * u.x + be * v.x, ae * u.y + be * v.y};
  }
}
template <typename TO, typename TI>
__global__ void k_convert(const TI *x, TO *y, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    typedef decltype(TO::x) E;
    TI u = x[i];
    y[i] = {(E)u.x, (E)u.y};
  }
}

__device__ __forceinline__ M3<double> mm_nn(const M3<double> &a, const M3<double> &b) {
  M3<double> c;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      double re = 0, im = 0;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        re = fma(a.e[i][k].re, b.e[k][j].re, re); re = fma(-a.e[i][k].im, b.e[k][j].im, re);
        im = fma(a.e[i][k].re, b.e[k][j].im, im); im = fma(a.e[i][k].im, b.e[k][j].re, im);
      }
      c.e[i][j] = {re, im};
    }
  return c;
}
__device__ __forceinline__ M3<double> mm_na(const M3<double> &a, const M3<double> &b) {  // a b^dag
  M3<double> c;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      double re = 0, im = 0;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        re = fma(a.e[i][k].re, b.e[j][k].re, re); re = fma(a.e[i][k].im, b.e[j][k].im, re);
        im = fma(a.e[i][k].im, b.e[j][k].re, im); im = fma(-a.e[i][k].re, b.e[j][k].im, im);
      }
      c.e[i][j] = {re, im};
    }
  return c;
}
__device__ __forceinline__ M3<double> mm_an(const M3<double> &a, const M3<double> &b) {  // a^dag b
  M3<double> c;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      double re = 0, im = 0;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        re = fma(a.e[k][i].re, b.e[k][j].re, re); re = fma(a.e[k][i].im, b.e[k][j].im, re);
        im = fma(a.e[k][i].re, b.e[k][j].im, im); im = fma(-a.e[k][i].im, b.e[k][j].re, im);
      }
      c.e[i][j] = {re, im};
    }
  return c;
}

// the same products in arithmetic R
template <typename R>
__device__ __forceinline__ M3<R> tnn(const M3<R> &a, const M3<R> &b) {
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
__device__ __forceinline__ M3<R> tna(const M3<R> &a, const M3<R> &b) {  // a b^dag
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
template <typename R>
__device__ __forceinline__ M3<R> tan_(const M3<R> &a, const M3<R> &b) {  // a^dag b
  M3<R> c;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      R re = 0, im = 0;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        re = fma(a.e[k][i].re, b.e[k][j].re, re); re = fma(a.e[k][i].im, b.e[k][j].im, re);
        im = fma(a.e[k][i].re, b.e[k][j].im, im); im = fma(-a.e[k][i].im, b.e[k][j].re, im);
      }
      c.e[i][j] = {re, im};
    }
  return c;
}
template <typename R>
__device__ __forceinline__ M3<R> tadj(const M3<R> &a) {
  M3<R> c;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) c.e[i][j] = {a.e[j][i].re, -a.e[j][i].im};
  return c;
}
template <typename R>
__device__ __forceinline__ void tacc(M3<R> &d, const M3<R> &s, R f) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) { d.e[i][j].re = fma(f, s.e[i][j].re, d.e[i][j].re); d.e[i][j].im = fma(f, s.e[i][j].im, d.e[i][j].im); }
}

// Eigenvalues g[0..2] of the Hermitian, non-negative Q = V^dag V (Q2 = Q Q)
// from its invariants c0 = tr Q, c1 = tr Q^2 / 2, c2 = tr Q^3 / 3 by the
// trigonometric solution of the characteristic cubic -- the first step of
// the analytic U(3) projection W = V Q^(-1/2) (generic_ks/su3_mat_op.c:
// 828-1000) and of its adjoint in the fermion force.  Arithmetic A.
template <typename A>
__device__ __forceinline__ void herm3_eigvals(const M3<A> &Q, const M3<A> &Q2, A g[3]) {
  A c0 = Q.e[0][0].re + Q.e[1][1].re + Q.e[2][2].re;
  A c1 = (Q2.e[0][0].re + Q2.e[1][1].re + Q2.e[2][2].re) / 2;
  A q3 = 0;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int k = 0; k < 3; k++) q3 += Q2.e[i][k].re * Q.e[k][i].re - Q2.e[i][k].im * Q.e[k][i].im;
  A c2 = q3 / 3;
  A S = c1 / 3 - c0 * (c0 / 18);
  if (fabs(S) < (A)1.0e-14) {
    g[0] = g[1] = g[2] = c0 / 3;
  } else {
    A R = c2 / 2 - c0 * (c1 / 3) + c0 * c0 * (c0 / 27);
    S = sqrt(S);
    A RoS = R / (S * S * S), theta;
    if (!(fabs(RoS) < (A)1)) theta = R > 0 ? (A)0 : (A)3.14159265358979323846264338328;
    else theta = acos(RoS);
    A th3 = theta / 3, pi23 = (A)(6.28318530717958647692528676656 / 3);
    g[0] = c0 / 3 + 2 * S * cos(th3);
    g[1] = c0 / 3 + 2 * S * cos(th3 + pi23);
    g[2] = c0 / 3 + 2 * S * cos(th3 + 2 * pi23);
  }
}

// neighbour (checkerboard index) of site (par,h) displaced by d along mu
__device__ __forceinline__ int nbr(const Geom &g, int par, int h, int mu, int d) {
  int c[4];
  site_coords(g, par, h, c[0], c[1], c[2], c[3]);
  const int L[4] = {g.nx, g.ny, g.nz, g.nt};
  c[mu] = wrap_add(c[mu], d, L[mu]);
  return cb_index(g, c[0], c[1], c[2], c[3]);
}
__device__ __forceinline__ int nbr2(const Geom &g, int par, int h, int mu, int d1, int nu, int d2) {
  int c[4];
  site_coords(g, par, h, c[0], c[1], c[2], c[3]);
  const int L[4] = {g.nx, g.ny, g.nz, g.nt};
  c[mu] = wrap_add(c[mu], d1, L[mu]);
  c[nu] = wrap_add(c[nu], d2, L[nu]);
  return cb_index(g, c[0], c[1], c[2], c[3]);
}

// generalised staple S(x) = U_nu(x) A(x+nu) U_nu(x+mu)^dag + U_nu(x-nu)^dag A(x-nu) U_nu(x-nu+mu)
// (generic/general_staple.c:42-140): S saved when sout.p != nullptr, and
// fat_mu(x) += coef * S(x) when fat.p != nullptr; fields stored and
// products computed in precision R
template <typename R>
static __global__ void __launch_bounds__(128) k_staple(Geom g, int mu, int nu, MatT<R> Unu, MatT<R> A, MatT<R> fat,
                                                       double coef, MatT<R> sout) {
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  const int par = blockIdx.y, opar = 1 - par;
  const int Vh = g.Vh;
  if (h >= Vh) return;
  const int xpnu = nbr(g, par, h, nu, 1), xpmu = nbr(g, par, h, mu, 1), xmnu = nbr(g, par, h, nu, -1);
  const int xmnupmu = nbr2(g, par, h, nu, -1, mu, 1);
  // upper: U_nu(x) [A(x+nu) U_nu(x+mu)^dag]
  M3<R> up = tnn<R>(Unu.ld(par, h, Vh), tna<R>(A.ld(opar, xpnu, Vh), Unu.ld(opar, xpmu, Vh)));
  // lower: [U_nu(x-nu)^dag A(x-nu)] U_nu(x-nu+mu)
  M3<R> dn = tnn<R>(tan_<R>(Unu.ld(opar, xmnu, Vh), A.ld(opar, xmnu, Vh)), Unu.ld(par, xmnupmu, Vh));
  M3<R> s;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) s.e[i][j] = {up.e[i][j].re + dn.e[i][j].re, up.e[i][j].im + dn.e[i][j].im};
  if (sout.p) sout.st(par, h, Vh, s);
  if (!fat.p) return;
  M3<R> f = fat.ld(par, h, Vh);
  const R c = (R)coef;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      f.e[i][j].re += c * s.e[i][j].re;
      f.e[i][j].im += c * s.e[i][j].im;
    }
  fat.st(par, h, Vh, f);
}
}  // namespace mks
