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
  int rev;                    // plain D only: blocks take the sites in reverse order
  int nvb;                    // site blocks to cover (0: one per CTA); a smaller grid loops over them
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

// checkerboard indices of the +-1 and +-3 neighbours along mu of the site with
// coordinates c0: from the site's lexicographic index, one add, one select
// and one shift each (a hop of k along mu moves the lexicographic index by
// k * stride, less extent * stride where it wraps; extents are >= 4, so a
// hop of 3 wraps at most once)
#ifndef MKS_NBR_LEX
#define MKS_NBR_LEX 1
#endif
__device__ __forceinline__ void nbr4(const Geom &g, const int c0[4], const int L[4], int mu, int &hf1, int &hb1,
                                     int &hf3, int &hb3) {
  if (!MKS_NBR_LEX) {  // the same indices from the shifted coordinates
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
    return;
  }
  const int i = c0[0] + g.nx * (c0[1] + g.ny * (c0[2] + g.nz * c0[3]));
  const int S = mu == 0 ? g.sx : (mu == 1 ? g.sy : (mu == 2 ? g.sz : g.st));
  const int LS = L[mu] * S, c = c0[mu];
  hf1 = (i + S - (c + 1 >= L[mu] ? LS : 0)) >> 1;
  hb1 = (i - S + (c < 1 ? LS : 0)) >> 1;
  hf3 = (i + 3 * S - (c + 3 >= L[mu] ? LS : 0)) >> 1;
  hb3 = (i - 3 * S + (c < 3 ? LS : 0)) >> 1;
}

// ---- links of a tile staged in shared memory by the TMA engine ----
// A tile is T = R x nx/2 consecutive output sites: R complete x-rows of one
// (z, t) plane.  Its 16 links per site (fat / Naik, forward at the site,
// backward at the -1 / -3 neighbour) are copied by cp.async.bulk into
// shared memory, link l = 4 mu + kind (kind 0 fat forward, 1 Naik forward,
// 2 fat backward, 3 Naik backward) at byte offset 72 T l: the four float4
// planes of FP32 entries 0..7 (T x 16 B each) and the float2 plane of
// entry 8 (T x 8 B).  The backward links along y, z, t are the rows of the
// shifted rows or planes, copied in row order (at most two segments where
// y wraps), so site i of the tile finds its backward link at slot i; along
// x they are the tile's own rows of the other parity, slot hb - h0.
struct TileSmem {
  const unsigned char *base;
  int T;
  __device__ __forceinline__ M3<float> link(int l, int j) const {
    const unsigned char *r = base + (size_t)l * 72 * T;
    M3<float> m;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const float4 q = *reinterpret_cast<const float4 *>(r + (size_t)k * 16 * T + 16 * j);
      m.e[(2 * k) / 3][(2 * k) % 3] = {q.x, q.y};
      m.e[(2 * k + 1) / 3][(2 * k + 1) % 3] = {q.z, q.w};
    }
    const float2 e = *reinterpret_cast<const float2 *>(r + (size_t)64 * T + 8 * j);
    m.e[2][2] = {e.x, e.y};
    return m;
  }
};

// The 16 terms of one output site, links loaded from global memory.
// PIPE = false: each term loads its link and then applies it.  PIPE = true:
// a software pipeline one term deep -- the next term's link loads are issued
// before this term's mat-vecs, so two link fetches from HBM are in flight per
// thread instead of one (more registers per thread, fewer resident warps).
template <typename R, class LinkT, class InT, int NB, bool PIPE>
__device__ __forceinline__ void site_terms(const LinkT &fat, const LinkT &lng, const InT *in, int nsrc, int grp,
                                           const Geom &g, int par, int h, const int c0[4], V3<R> (&acc)[NB]) {
  const int Vh = g.Vh, opar = 1 - par;
  const int L[4] = {g.nx, g.ny, g.nz, g.nt};
  if constexpr (!PIPE) {
#pragma unroll
    for (int mu = 0; mu < 4; mu++) {
      int hf1, hb1, hf3, hb3;
      nbr4(g, c0, L, mu, hf1, hb1, hf3, hb3);
      {
        const M3<R> U = load_link(fat, par, mu, h, Vh);
#pragma unroll
        for (int s = 0; s < NB; s++)
          if (grp * NB + s < nsrc) mv_acc(U, load_in<LinkT>(in[grp * NB + s], hf1, Vh, fat), acc[s]);
      }
      {
        const M3<R> U = load_link(lng, par, mu, h, Vh);
#pragma unroll
        for (int s = 0; s < NB; s++)
          if (grp * NB + s < nsrc) mv_acc(U, load_in<LinkT>(in[grp * NB + s], hf3, Vh, lng), acc[s]);
      }
      {
        const M3<R> U = load_link(fat, opar, mu, hb1, Vh);
#pragma unroll
        for (int s = 0; s < NB; s++)
          if (grp * NB + s < nsrc) amv_sub(U, load_in<LinkT>(in[grp * NB + s], hb1, Vh, fat), acc[s]);
      }
      {
        const M3<R> U = load_link(lng, opar, mu, hb3, Vh);
#pragma unroll
        for (int s = 0; s < NB; s++)
          if (grp * NB + s < nsrc) amv_sub(U, load_in<LinkT>(in[grp * NB + s], hb3, Vh, lng), acc[s]);
      }
    }
  } else {
    int hf1, hb1, hf3, hb3;
    nbr4(g, c0, L, 0, hf1, hb1, hf3, hb3);
    M3<R> U = load_link(fat, par, 0, h, Vh);
#pragma unroll
    for (int mu = 0; mu < 4; mu++) {
      M3<R> Un = load_link(lng, par, mu, h, Vh);  // next: Naik forward
#pragma unroll
      for (int s = 0; s < NB; s++)
        if (grp * NB + s < nsrc) mv_acc(U, load_in<LinkT>(in[grp * NB + s], hf1, Vh, fat), acc[s]);
      U = Un;
      Un = load_link(fat, opar, mu, hb1, Vh);  // next: fat backward
#pragma unroll
      for (int s = 0; s < NB; s++)
        if (grp * NB + s < nsrc) mv_acc(U, load_in<LinkT>(in[grp * NB + s], hf3, Vh, lng), acc[s]);
      U = Un;
      Un = load_link(lng, opar, mu, hb3, Vh);  // next: Naik backward
#pragma unroll
      for (int s = 0; s < NB; s++)
        if (grp * NB + s < nsrc) amv_sub(U, load_in<LinkT>(in[grp * NB + s], hb1, Vh, fat), acc[s]);
      U = Un;
      int nf1 = 0, nb1 = 0, nf3 = 0, nb3 = 0;
      if (mu < 3) {
        nbr4(g, c0, L, mu + 1, nf1, nb1, nf3, nb3);
        Un = load_link(fat, par, mu + 1, h, Vh);  // next: fat forward of the next direction
      }
#pragma unroll
      for (int s = 0; s < NB; s++)
        if (grp * NB + s < nsrc) amv_sub(U, load_in<LinkT>(in[grp * NB + s], hb3, Vh, lng), acc[s]);
      U = Un;
      hf1 = nf1; hb1 = nb1; hf3 = nf3; hb3 = nb3;
    }
  }
}

// ---- cp.async helpers (per-thread asynchronous global -> shared copies) ----
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)),
               "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)),
               "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// The 16 terms of one output site with the FP32 links fetched ahead into
// shared memory by cp.async (a ring of STAGES link buffers per site): the
// copies of the next STAGES-1 terms' links are in flight while this term's
// mat-vecs run, and an in-flight copy holds no register.  The G threads of a
// site share its buffers (each copies some of the link's five 16/8-byte
// pieces) and sit in one warp; __syncwarp orders a buffer's copies before
// its reads and its reads before it is refilled.  Every thread of the warp
// runs the loop; `valid` marks the threads that own a site.  Buffer layout
// per stage: four float4 planes and one float2 plane of the block's sites.
template <int STAGES>
__device__ __forceinline__ void async_issue(const LinkF32 &fat, const LinkF32 &lng, int term, int par, int opar,
                                            int h, int hb1, int hb3, int Vh, int grp, int G, unsigned char *buf,
                                            int spb, int j) {
  const int mu = term >> 2, kind = term & 3;
  const LinkF32 &L = (kind & 1) ? lng : fat;
  const int sp = kind < 2 ? par : opar;
  const int idx = kind < 2 ? h : (kind == 2 ? hb1 : hb3);
  for (int k = grp; k < 5; k += G) {
    if (k < 4)
      cp_async16(buf + (size_t)k * 16 * spb + 16 * j, L.a + ((size_t)(sp * 4 + mu) * 4 + k) * Vh + idx);
    else
      cp_async8(buf + (size_t)64 * spb + 8 * j, L.b + (size_t)(sp * 4 + mu) * Vh + idx);
  }
}

template <class InT, int NB, int STAGES>
__device__ __forceinline__ void site_terms_async(const LinkF32 &fat, const LinkF32 &lng, const InT *in, int nsrc,
                                                 int grp, int G, const Geom &g, int par, int h, const int c0[4],
                                                 V3<float> (&acc)[NB], bool valid, unsigned char *smem) {
  const int Vh = g.Vh, opar = 1 - par;
  const int L[4] = {g.nx, g.ny, g.nz, g.nt};
  const int spb = (int)blockDim.x / G, j = (int)threadIdx.x / G;
  const size_t stage_bytes = (size_t)72 * spb;
  // neighbour indices per direction, for the vectors and the backward links
  int nb[4][4];
#pragma unroll
  for (int mu = 0; mu < 4; mu++) nbr4(g, c0, L, mu, nb[mu][0], nb[mu][1], nb[mu][2], nb[mu][3]);
#pragma unroll
  for (int t = 0; t < STAGES - 1; t++) {
    if (valid)
      async_issue<STAGES>(fat, lng, t, par, opar, h, nb[t >> 2][1], nb[t >> 2][3], Vh, grp, G,
                          smem + (size_t)t * stage_bytes, spb, j);
    cp_async_commit();
  }
#pragma unroll
  for (int term = 0; term < 16; term++) {
    const int nt = term + STAGES - 1;
    __syncwarp();  // every lane has read the buffer about to be refilled
    if (nt < 16 && valid)
      async_issue<STAGES>(fat, lng, nt, par, opar, h, nb[nt >> 2][1], nb[nt >> 2][3], Vh, grp, G,
                          smem + (size_t)(nt % STAGES) * stage_bytes, spb, j);
    cp_async_commit();
    cp_async_wait<STAGES - 1>();  // this thread's pieces of `term` have landed
    __syncwarp();                 // and the other threads' of the site
    if (!valid) continue;
    const unsigned char *b = smem + (size_t)(term % STAGES) * stage_bytes;
    M3<float> U;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const float4 q = *reinterpret_cast<const float4 *>(b + (size_t)k * 16 * spb + 16 * j);
      U.e[(2 * k) / 3][(2 * k) % 3] = {q.x, q.y};
      U.e[(2 * k + 1) / 3][(2 * k + 1) % 3] = {q.z, q.w};
    }
    const float2 e8 = *reinterpret_cast<const float2 *>(b + (size_t)64 * spb + 8 * j);
    U.e[2][2] = {e8.x, e8.y};
    const int mu = term >> 2, kind = term & 3;
    const int n = nb[mu][kind == 0 ? 0 : (kind == 1 ? 2 : (kind == 2 ? 1 : 3))];
#pragma unroll
    for (int s = 0; s < NB; s++) {
      if (grp * NB + s >= nsrc) continue;
      const V3<float> v = in[grp * NB + s].load(n, Vh);
      if (kind < 2) mv_acc(U, v, acc[s]);
      else amv_sub(U, v, acc[s]);
    }
  }
}

// live = false (a TMA tile whose staged links did not arrive): the thread
// computes and writes nothing but still takes part in the grid reduction
// with zero sums, so the arrival counters return to zero as in every launch
// LOOP = true: the CTA loops over site blocks (persistent grid, a.nvb);
// a separate instantiation, since the loop costs registers (loop-invariant
// values held across it)
// ASYNC = STAGES > 0: FP32 links fetched ahead by cp.async into the dynamic
// shared memory `asm_base` (site_terms_async)
template <typename R, class LinkT, class InT, class OutT, int NB, int EPI, int NSUM, class Fin, bool TMA = false,
          bool PIPE = false, bool LOOP = false, int ASYNC = 0>
__device__ __forceinline__ void dslash_body(const LinkT &fat, const LinkT &lng,
                                            const DslashArgs<InT, OutT, typename EpiLoad<R>::type> &a,
                                            const Fin &fin, const TileSmem ts = TileSmem{nullptr, 0},
                                            const bool live = true, unsigned char *asm_base = nullptr) {
  typedef typename EpiLoad<R>::type EpiT;
  if (a.skip && *a.skip) return;
  const Geom &g = a.g;
  const int G = a.groups;
  const int Vh = g.Vh;
  const int par = a.out_par, opar = 1 - par;
  // per-thread dot products in the kernel's precision: one site's, or the
  // sum over the sites the thread visits when the grid loops
  R sums[NB][NSUM > 0 ? NSUM : 1];
#pragma unroll
  for (int s = 0; s < NB; s++)
#pragma unroll
    for (int k = 0; k < (NSUM > 0 ? NSUM : 1); k++) sums[s][k] = R(0);
  // blockDim.x is a multiple of G, so a thread's source group is fixed
  const int grp = (int)threadIdx.x % G;
  // site blocks: one per CTA, or (a.nvb > gridDim.x) a persistent grid that
  // loops over them in the same order, so each CTA reduces its dot products
  // once at the end
  const int nvb = (LOOP && a.nvb > 0) ? a.nvb : (int)gridDim.x;
  auto site_block = [&](const int vb) {
  // a plain D may sweep the sites from the end: it then reads first the part
  // of its input that the previous kernel wrote last (still in L2) and
  // leaves the start of its output in L2 for a following forward sweep
  const int bid = (!TMA && EPI == EPI_PLAIN && a.rev) ? nvb - 1 - vb : vb;
  const int h = (bid * (int)blockDim.x + (int)threadIdx.x) / G;

#ifndef MKS_EPI_PREFETCH
#define MKS_EPI_PREFETCH 1  // measured: 3 % faster 8-source CG on GB300
#endif
  if (MKS_EPI_PREFETCH && EPI == EPI_AXPY && grp == 0 && (h & 15) == 0 && h < Vh && live) {
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
  const bool valid = h < Vh && live;
  if (valid || ASYNC > 0) {  // the async loop runs on every lane of the warp
    int x = 0, y = 0, z = 0, t = 0;
    if (valid) site_coords(g, par, h, x, y, z, t);
    V3<R> acc[NB];
#pragma unroll
    for (int s = 0; s < NB; s++)
#pragma unroll
      for (int c = 0; c < 3; c++) acc[s].c[c] = {R(0), R(0)};
    const int c0[4] = {x, y, z, t};
    if constexpr (ASYNC > 0) {
      site_terms_async<InT, NB, ASYNC>(fat, lng, a.in, a.nsrc, grp, G, g, par, h, c0, acc, valid, asm_base);
    } else if constexpr (!TMA) {
      site_terms<R, LinkT, InT, NB, PIPE>(fat, lng, a.in, a.nsrc, grp, g, par, h, c0, acc);
    } else {
    const int L[4] = {g.nx, g.ny, g.nz, g.nt};
#pragma unroll
    for (int mu = 0; mu < 4; mu++) {
      int hf1, hb1, hf3, hb3;
      nbr4(g, c0, L, mu, hf1, hb1, hf3, hb3);
      // tile-local slots of the staged links (TMA): the site's own slot, or
      // along x the slot of the backward neighbour within the tile's rows
      const int i0 = TMA ? h - (int)(blockIdx.x * ts.T) : 0;
      const int jb1 = (TMA && mu == 0) ? hb1 - (h - i0) : i0, jb3 = (TMA && mu == 0) ? hb3 - (h - i0) : i0;
      {
        M3<R> U;
        if constexpr (TMA) U = ts.link(4 * mu + 0, i0);
        else U = load_link(fat, par, mu, h, Vh);
#pragma unroll
        for (int s = 0; s < NB; s++) {
          const int S = grp * NB + s;
          if (S < a.nsrc) mv_acc(U, load_in<LinkT>(a.in[S], hf1, Vh, fat), acc[s]);
        }
      }
      {
        M3<R> U;
        if constexpr (TMA) U = ts.link(4 * mu + 1, i0);
        else U = load_link(lng, par, mu, h, Vh);
#pragma unroll
        for (int s = 0; s < NB; s++) {
          const int S = grp * NB + s;
          if (S < a.nsrc) mv_acc(U, load_in<LinkT>(a.in[S], hf3, Vh, lng), acc[s]);
        }
      }
      {
        M3<R> U;
        if constexpr (TMA) U = ts.link(4 * mu + 2, jb1);
        else U = load_link(fat, opar, mu, hb1, Vh);
#pragma unroll
        for (int s = 0; s < NB; s++) {
          const int S = grp * NB + s;
          if (S < a.nsrc) amv_sub(U, load_in<LinkT>(a.in[S], hb1, Vh, fat), acc[s]);
        }
      }
      {
        M3<R> U;
        if constexpr (TMA) U = ts.link(4 * mu + 3, jb3);
        else U = load_link(lng, opar, mu, hb3, Vh);
#pragma unroll
        for (int s = 0; s < NB; s++) {
          const int S = grp * NB + s;
          if (S < a.nsrc) amv_sub(U, load_in<LinkT>(a.in[S], hb3, Vh, lng), acc[s]);
        }
      }
    }
    }  // TMA
#pragma unroll
    for (int s = 0; s < NB; s++) {
      const int S = grp * NB + s;
      if (S >= a.nsrc || !valid) continue;
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
          sums[s][0] += d;
        }
        if (NSUM >= 3) {
          const V3<R> r = a.r[S].load(h, Vh);
          R d1 = 0, d2 = 0;
#pragma unroll
          for (int c = 0; c < 3; c++) {
            d1 += acc[s].c[c].re * r.c[c].re + acc[s].c[c].im * r.c[c].im;
            d2 += acc[s].c[c].re * acc[s].c[c].re + acc[s].c[c].im * acc[s].c[c].im;
          }
          sums[s][1] += d1;
          sums[s][2] += d2;
        }
      }
      // the fused-epilogue result is read once, by the next kernel
      if (EPI == EPI_AXPY) a.out[S].store_stream(h, Vh, acc[s]);
      else a.out[S].store(h, Vh, acc[s]);
    }
  }
  };  // site_block
  if constexpr (LOOP) {
#pragma unroll 1
    for (int vb = blockIdx.x; vb < nvb; vb += gridDim.x) site_block(vb);
  } else {
    site_block((int)blockIdx.x);
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

// the multi-source shapes (G threads per site x NB sources per thread);
// the FP32/FP16 plain D with up to 4 sources per thread is held to 64
// registers (4 resident 256-thread blocks per SM), which it needs without
// spilling
#ifndef MKS_DSLASH_MINB
#define MKS_DSLASH_MINB 4
#endif
template <typename R, class LinkT, class InT, class OutT, int NB, int EPI, int NSUM, class Fin>
__global__ void __launch_bounds__(256, (sizeof(R) == 4 && NB <= 4 && EPI == EPI_PLAIN && !LinkT::scaled) ? MKS_DSLASH_MINB : 0)
k_dslash(const LinkT fat, const LinkT lng, const DslashArgs<InT, OutT, typename EpiLoad<R>::type> a,
         const Fin fin) {
  dslash_body<R, LinkT, InT, OutT, NB, EPI, NSUM, Fin>(fat, lng, a, fin);
}

// the multi-source shapes on a persistent grid: as many CTAs as fit on the
// GPU loop over the site blocks (a.nvb), so a fused-epilogue launch reduces
// its dot products once per CTA; at least 3 resident 256-thread blocks per
// SM are asked of the register allocator (the loop holds more values live)
template <typename R, class LinkT, class InT, class OutT, int NB, int EPI, int NSUM, class Fin>
__global__ void __launch_bounds__(256, 3)
k_dslash_g(const LinkT fat, const LinkT lng, const DslashArgs<InT, OutT, typename EpiLoad<R>::type> a,
           const Fin fin) {
  dslash_body<R, LinkT, InT, OutT, NB, EPI, NSUM, Fin, false, false, true>(fat, lng, a, fin);
}

// the multi-source FP32 shapes with the links fetched ahead into shared
// memory by cp.async, STAGES link buffers per site (dynamic shared memory
// STAGES x 72 B x sites per block); at least 3 resident 256-thread blocks
// per SM (80 registers: 4 sources per thread spill a few bytes, a bound of 4
// blocks spills hundreds)
template <class InT, class OutT, int NB, int EPI, int NSUM, class Fin, int STAGES>
__global__ void __launch_bounds__(256, 3)
k_dslash_a(const LinkF32 fat, const LinkF32 lng, const DslashArgs<InT, OutT, VecF32> a, const Fin fin) {
  extern __shared__ __align__(16) unsigned char adsm[];
  dslash_body<float, LinkF32, InT, OutT, NB, EPI, NSUM, Fin, false, false, false, STAGES>(
      fat, lng, a, fin, TileSmem{nullptr, 0}, true, adsm);
}

// the same shapes with the link loads software-pipelined one term deep
// (site_terms<PIPE = true>); the register allocator is asked for at least
// MKS_DSLASHP_MINB resident 256-thread blocks per SM (3: up to 80 registers
// per thread, room for the second link without spills up to 4 sources per
// thread; with 2 the allocator took 126 registers and the kernel ran 1.5x
// slower on GB300)
#ifndef MKS_DSLASHP_MINB
#define MKS_DSLASHP_MINB 3
#endif
template <typename R, class LinkT, class InT, class OutT, int NB, int EPI, int NSUM, class Fin>
__global__ void __launch_bounds__(256, MKS_DSLASHP_MINB)
k_dslash_p(const LinkT fat, const LinkT lng, const DslashArgs<InT, OutT, typename EpiLoad<R>::type> a,
           const Fin fin) {
  dslash_body<R, LinkT, InT, OutT, NB, EPI, NSUM, Fin, false, true>(fat, lng, a, fin);
}

// one source, one thread per site (G = NB = 1)
template <typename R, class LinkT, class InT, class OutT, int EPI, int NSUM, class Fin>
__global__ void __launch_bounds__(256, MKS_DSLASH1_MINB)
k_dslash1(const LinkT fat, const LinkT lng, const DslashArgs<InT, OutT, typename EpiLoad<R>::type> a,
          const Fin fin) {
  dslash_body<R, LinkT, InT, OutT, 1, EPI, NSUM, Fin>(fat, lng, a, fin);
}

// ---- TMA (cp.async.bulk) helpers ----
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}
// bounded wait: false when the phase did not complete within `limit` polls
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t phase, int limit) {
  for (int it = 0; it < limit; it++)
    if (mbar_try_wait(bar, phase)) return true;
  return false;
}
// global -> shared bulk copy (16-byte aligned addresses, size a multiple of 16)
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// the (up to two) contiguous source segments of link l = 4 mu + kind for the
// tile that starts at h0: seg 0 / 1 -> (first source site, first slot, sites);
// false when the segment does not exist
__device__ __forceinline__ bool tile_segment(const Geom &g, int T, int R, int h0, int l, int seg, int &src0,
                                             int &loc0, int &cnt) {
  const int mu = l >> 2, kind = l & 3;
  const int s = kind < 2 ? 0 : (kind == 2 ? 1 : 3);
  const int nx2 = g.nx >> 1;
  const int row = h0 / nx2, y0 = row % g.ny, pz = row / g.ny, z = pz % g.nz, t = pz / g.nz;
  if (s == 0 || mu == 0) {
    if (seg) return false;
    src0 = h0; loc0 = 0; cnt = T;
    return true;
  }
  if (mu == 1) {
    int yr = y0 - s;
    if (yr < 0) yr += g.ny;
    const int n1 = min(R, g.ny - yr);
    const int pbase = pz * g.ny * nx2;
    if (seg == 0) { src0 = pbase + yr * nx2; loc0 = 0; cnt = n1 * nx2; return true; }
    if (n1 == R) return false;
    src0 = pbase; loc0 = n1 * nx2; cnt = (R - n1) * nx2;
    return true;
  }
  if (seg) return false;
  if (mu == 2) {
    int zz = z - s;
    if (zz < 0) zz += g.nz;
    src0 = ((t * g.nz + zz) * g.ny + y0) * nx2;
  } else {
    int tt = t - s;
    if (tt < 0) tt += g.nt;
    src0 = ((tt * g.nz + z) * g.ny + y0) * nx2;
  }
  loc0 = 0; cnt = T;
  return true;
}

// FP32 multi-source D_eo with the links of each tile of T sites staged in
// shared memory by the TMA engine (one thread per site and source, G
// threads per site; blockDim = T G).  Warp 0 issues the bulk copies, every
// thread waits on the tile's mbarrier with a bounded poll.  A thread whose
// wait runs out ORs the value 2 (bit 1) into the reduction error flag, which
// the host reads at its next poll, waits once more (bounded) for the copies
// in flight to land in the block's shared memory, and then computes and
// writes nothing: it only takes part in the grid reduction with zero sums so
// that the reduction's arrival counters end at zero.  If the second wait
// runs out too, it ORs in the value 4 (bit 2).  The host treats either bit
// as fatal for the staged kernel: it stops using it for the rest of the
// process and the solver call repeats its work with the plain kernel.
template <int EPI, int NSUM, class Fin>
__global__ void __launch_bounds__(256)
k_dslash_tma(const LinkF32 fat, const LinkF32 lng, const DslashArgs<VecF32, VecF32, VecF32> a, const Fin fin,
             int T, int R) {
  extern __shared__ __align__(128) unsigned char tsm[];
  __shared__ __align__(8) uint64_t bar;
  if (a.skip && *a.skip) return;
  const Geom &g = a.g;
  const int Vh = g.Vh, par = a.out_par, opar = 1 - par;
  const int h0 = blockIdx.x * T;
  if (threadIdx.x == 0) mbar_init(&bar, 1);
  __syncthreads();
  if (threadIdx.x < 32) {
    if (threadIdx.x == 0) mbar_expect_tx(&bar, (uint32_t)T * 1152u);
    __syncwarp();
    for (int c = threadIdx.x; c < 160; c += 32) {
      const int l = c / 10, q = (c % 10) >> 1, seg = c & 1;
      int src0, loc0, cnt;
      if (!tile_segment(g, T, R, h0, l, seg, src0, loc0, cnt)) continue;
      const int mu = l >> 2, kind = l & 3;
      const LinkF32 &L = (kind & 1) ? lng : fat;
      const int sp = kind < 2 ? par : opar;
      unsigned char *reg = tsm + (size_t)l * 72 * T;
      if (q < 4)
        bulk_g2s(reg + (size_t)q * 16 * T + 16 * loc0, L.a + ((size_t)(sp * 4 + mu) * 4 + q) * Vh + src0,
                 (uint32_t)cnt * 16u, &bar);
      else
        bulk_g2s(reg + (size_t)64 * T + 8 * loc0, L.b + (size_t)(sp * 4 + mu) * Vh + src0, (uint32_t)cnt * 8u, &bar);
    }
  }
  bool live = true;
  if (!mbar_wait_bounded(&bar, 0, 1 << 22)) {
    live = false;
    if (a.red.err) atomicOr(a.red.err, 2);
    // let copies in flight land before the block's shared memory is released
    if (!mbar_wait_bounded(&bar, 0, 1 << 22) && a.red.err) atomicOr(a.red.err, 4);
  }
  dslash_body<float, LinkF32, VecF32, VecF32, 1, EPI, NSUM, Fin, true>(fat, lng, a, fin, TileSmem{tsm, T}, live);
}

}  // namespace mks
