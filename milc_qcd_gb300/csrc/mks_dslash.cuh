// mks_dslash.cuh -- the improved-staggered D_eo kernel template.
//
// out(x) = sum_mu F_mu(x) in(x+mu) - F_mu(x-mu)^dag in(x-mu)
//                + L_mu(x) in(x+3mu) - L_mu(x-3mu)^dag in(x-3mu)
// (generic_ks/dslash_fn.c:365-576), for x of parity out_par.
//
// One thread group of G threads handles one output site; each thread of
// the group applies the site's 16 links to NB sources, so a link fetched
// from HBM serves G*NB right-hand sides (the G copies of a link load
// within a warp coalesce into one request).  Neighbour indices are
// computed from the checkerboard index; nothing but links and vectors is
// read.  Epilogues fuse the CG / multi-shift BLAS and their dot products:
//   EPI_PLAIN : out = D in
//   EPI_AXPY  : out = D in + coef_s * p_s, with sums <p,out>, <out,r>, <out,out>
//               (NSUM = 3, FEWSUMS-style CG) or only <p,out> (NSUM = 1)
// followed by a grid reduction whose last block runs the finisher.
#pragma once
#include "mks_internal.cuh"
#include "mks_reduce.cuh"

namespace mks {

constexpr int MAXSRC = 16;
enum { EPI_PLAIN = 0, EPI_AXPY = 1 };

template <class InT, class OutT, class EpiT>
struct DslashArgs {
  Geom g;
  int out_par;
  int nsrc;
  int groups;                 // G (power of two, <= 8)
  InT in[MAXSRC];
  OutT out[MAXSRC];
  EpiT p[MAXSRC];             // epilogue operand (same parity as out)
  EpiT r[MAXSRC];
  double coef[MAXSRC];
  const int *skip;            // kernel returns at once when *skip != 0
  const int *src_done;        // per-source: skip the epilogue update when non-zero
  RedScratch red;             // grid reduction scratch (NSUM > 0)
  double *totals;             // [nsrc][NSUM] written by the last block
};

template <typename R> struct EpiLoad;
template <> struct EpiLoad<double> { typedef VecF64 type; };
template <> struct EpiLoad<float> { typedef VecF32 type; };

// links of a scaled (FP16) type are used unscaled and their global scale
// multiplies the neighbour vector instead: one multiply per vector component
// rather than one per link entry
template <class LinkT>
__device__ __forceinline__ auto load_link(const LinkT &l, int par, int dir, int h, int Vh) {
  if constexpr (LinkT::scaled) return l.load_raw(par, dir, h, Vh);
  else return l.load(par, dir, h, Vh);
}
template <class LinkT, class InT>
__device__ __forceinline__ auto load_in(const InT &v, int h, int Vh, const LinkT &l) {
  if constexpr (LinkT::scaled) return v.load_mul(h, Vh, l.scale);
  else return v.load(h, Vh);
}

struct NoFinish {
  __device__ void operator()(const double *, int) const {}
};

// minimum resident 256-thread blocks per SM asked of the register allocator
// for the single-source kernel (one thread per site, one source): measured on
// GB300, 4 gives the FP32 single-source CG 6-8 % more D_eo throughput; asking
// it of the multi-source shapes slows them (register spills)
#ifndef MKS_DSLASH1_MINB
#define MKS_DSLASH1_MINB 4
#endif

// checkerboard indices of the +-1 and +-3 neighbours along mu of the site with coordinates c0
__device__ __forceinline__ void nbr4(const Geom &g, const int c0[4], const int L[4], int mu, int &hf1, int &hb1,
                                     int &hf3, int &hb3) {
  int cf1[4] = {c0[0], c0[1], c0[2], c0[3]}, cb1[4] = {c0[0], c0[1], c0[2], c0[3]};
  int cf3[4] = {c0[0], c0[1], c0[2], c0[3]}, cb3[4] = {c0[0], c0[1], c0[2], c0[3]};
  cf1[mu] = wrap_add(c0[mu], 1, L[mu]);
  cb1[mu] = wrap_add(c0[mu], -1, L[mu]);
  cf3[mu] = wrap_add(c0[mu], 3, L[mu]);
  cb3[mu] = wrap_add(c0[mu], -3, L[mu]);
  hf1 = cb_index(g, cf1[0], cf1[1], cf1[2], cf1[3]);
  hb1 = cb_index(g, cb1[0], cb1[1], cb1[2], cb1[3]);
  hf3 = cb_index(g, cf3[0], cf3[1], cf3[2], cf3[3]);
  hb3 = cb_index(g, cb3[0], cb3[1], cb3[2], cb3[3]);
}

template <typename R, class LinkT, class InT, class OutT, int NB, int EPI, int NSUM, class Fin>
__device__ __forceinline__ void dslash_body(const LinkT &fat, const LinkT &lng,
                                            const DslashArgs<InT, OutT, typename EpiLoad<R>::type> &a,
                                            const Fin &fin) {
  typedef typename EpiLoad<R>::type EpiT;
  if (a.skip && *a.skip) return;
  const Geom &g = a.g;
  const int G = a.groups;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int h = tid / G, grp = tid - h * G;
  const int Vh = g.Vh;
  const int par = a.out_par, opar = 1 - par;
  R sums[NB][NSUM > 0 ? NSUM : 1];  // per-site dot products in the kernel's precision
#pragma unroll
  for (int s = 0; s < NB; s++)
#pragma unroll
    for (int k = 0; k < (NSUM > 0 ? NSUM : 1); k++) sums[s][k] = R(0);

#ifndef MKS_EPI_PREFETCH
#define MKS_EPI_PREFETCH 1  // measured: 3 % faster 8-source CG on GB300
#endif
  if (MKS_EPI_PREFETCH && EPI == EPI_AXPY && grp == 0 && (h & 15) == 0 && h < Vh) {
    // the epilogue operands are needed only after the 16 neighbour terms:
    // start bringing them into L2 now (one thread per 16 sites)
#pragma unroll
    for (int s = 0; s < NB; s++) {
      const int S = grp * NB + s;
      if (S < a.nsrc) {
        a.p[S].prefetch16(h, Vh);
        if (NSUM >= 3) a.r[S].prefetch16(h, Vh);
      }
    }
  }
  if (h < Vh) {
    int x, y, z, t;
    site_coords(g, par, h, x, y, z, t);
    V3<R> acc[NB];
#pragma unroll
    for (int s = 0; s < NB; s++)
#pragma unroll
      for (int c = 0; c < 3; c++) acc[s].c[c] = {R(0), R(0)};
    const int c0[4] = {x, y, z, t};
    const int L[4] = {g.nx, g.ny, g.nz, g.nt};
#pragma unroll
    for (int mu = 0; mu < 4; mu++) {
      int hf1, hb1, hf3, hb3;
      nbr4(g, c0, L, mu, hf1, hb1, hf3, hb3);
      {
        const M3<R> U = load_link(fat, par, mu, h, Vh);
#pragma unroll
        for (int s = 0; s < NB; s++) {
          const int S = grp * NB + s;
          if (S < a.nsrc) mv_acc(U, load_in<LinkT>(a.in[S], hf1, Vh, fat), acc[s]);
        }
      }
      {
        const M3<R> U = load_link(lng, par, mu, h, Vh);
#pragma unroll
        for (int s = 0; s < NB; s++) {
          const int S = grp * NB + s;
          if (S < a.nsrc) mv_acc(U, load_in<LinkT>(a.in[S], hf3, Vh, lng), acc[s]);
        }
      }
      {
        const M3<R> U = load_link(fat, opar, mu, hb1, Vh);
#pragma unroll
        for (int s = 0; s < NB; s++) {
          const int S = grp * NB + s;
          if (S < a.nsrc) amv_sub(U, load_in<LinkT>(a.in[S], hb1, Vh, fat), acc[s]);
        }
      }
      {
        const M3<R> U = load_link(lng, opar, mu, hb3, Vh);
#pragma unroll
        for (int s = 0; s < NB; s++) {
          const int S = grp * NB + s;
          if (S < a.nsrc) amv_sub(U, load_in<LinkT>(a.in[S], hb3, Vh, lng), acc[s]);
        }
      }
    }
#pragma unroll
    for (int s = 0; s < NB; s++) {
      const int S = grp * NB + s;
      if (S >= a.nsrc) continue;
      if (EPI == EPI_AXPY) {
        const V3<R> p = a.p[S].load(h, Vh);
        const R cf = (R)a.coef[S];
#pragma unroll
        for (int c = 0; c < 3; c++) {
          acc[s].c[c].re = fma(cf, p.c[c].re, acc[s].c[c].re);
          acc[s].c[c].im = fma(cf, p.c[c].im, acc[s].c[c].im);
        }
        if (NSUM >= 1) {
          R d = 0;
#pragma unroll
          for (int c = 0; c < 3; c++) d += p.c[c].re * acc[s].c[c].re + p.c[c].im * acc[s].c[c].im;
          sums[s][0] = d;
        }
        if (NSUM >= 3) {
          const V3<R> r = a.r[S].load(h, Vh);
          R d1 = 0, d2 = 0;
#pragma unroll
          for (int c = 0; c < 3; c++) {
            d1 += acc[s].c[c].re * r.c[c].re + acc[s].c[c].im * r.c[c].im;
            d2 += acc[s].c[c].re * acc[s].c[c].re + acc[s].c[c].im * acc[s].c[c].im;
          }
          sums[s][1] = d1;
          sums[s][2] = d2;
        }
      }
      a.out[S].store(h, Vh, acc[s]);
    }
  }
  if (NSUM > 0) {
    __shared__ double smem[(256 / 32 + 1) * MAXSRC * 3];
    __shared__ double tot[MAXSRC * 3];
    __shared__ double scratch[256];
    block_reduce_grouped<R, NB, (NSUM > 0 ? NSUM : 1)>(sums, G, smem);
    const int nslots = G * NB;
    const double *btot = smem + (blockDim.x >> 5) * nslots * NSUM;
    if (grid_reduce_last(btot, nslots * NSUM, a.red, tot, scratch)) {
      if (threadIdx.x == 0) {
        for (int i = 0; i < a.nsrc * NSUM; i++) a.totals[i] = tot[i];
      }
      __syncthreads();
      fin(tot, a.nsrc);
    }
  }
}

// the multi-source shapes (G threads per site x NB sources per thread)
template <typename R, class LinkT, class InT, class OutT, int NB, int EPI, int NSUM, class Fin>
__global__ void __launch_bounds__(256)
k_dslash(const LinkT fat, const LinkT lng, const DslashArgs<InT, OutT, typename EpiLoad<R>::type> a,
         const Fin fin) {
  dslash_body<R, LinkT, InT, OutT, NB, EPI, NSUM, Fin>(fat, lng, a, fin);
}

// one source, one thread per site (G = NB = 1)
template <typename R, class LinkT, class InT, class OutT, int EPI, int NSUM, class Fin>
__global__ void __launch_bounds__(256, MKS_DSLASH1_MINB)
k_dslash1(const LinkT fat, const LinkT lng, const DslashArgs<InT, OutT, typename EpiLoad<R>::type> a,
          const Fin fin) {
  dslash_body<R, LinkT, InT, OutT, 1, EPI, NSUM, Fin>(fat, lng, a, fin);
}

}  // namespace mks
