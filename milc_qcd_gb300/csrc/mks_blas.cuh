// mks_blas.cuh -- site-loop kernel framework for the Krylov BLAS steps.
//
// k_site<Op, NSUM, Fin> runs Op on every checkerboard site of one source
// per blockIdx.y, accumulates NSUM FP64 sums, reduces them
// deterministically (grid_reduce_last: per-block rows summed in a fixed
// order) and lets the block that ends the reduction run the finisher Fin,
// which updates the solver scalars held in device memory.
#pragma once
#include "mks_internal.cuh"
#include "mks_reduce.cuh"

namespace mks {

constexpr int BLAS_MAXSRC = 16;

template <class Op, int NSUM, class Fin>
__global__ void __launch_bounds__(256) k_site(const Op op, const Fin fin, const int *skip, int Vh,
                                              const RedScratch red, double *totals) {
  if (skip && *skip) return;
  constexpr int NS = NSUM > 0 ? NSUM : 1;
  const int s = blockIdx.y;
  double acc[NS];
#pragma unroll
  for (int k = 0; k < NS; k++) acc[k] = 0.0;
  for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < Vh; h += gridDim.x * blockDim.x) {
    double loc[NS];
    op(h, s, loc);
#pragma unroll
    for (int k = 0; k < NSUM; k++) acc[k] += loc[k];
  }
  if (NSUM == 0) return;
  __shared__ double smem[(256 / 32) * NS];
  __shared__ double row[2 * BLAS_MAXSRC * NS];  // gridDim.y <= 2 * BLAS_MAXSRC
  __shared__ double tot[2 * BLAS_MAXSRC * NS];
  __shared__ double scratch[256];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < NS; k++) {
    double x = acc[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) smem[warp * NS + k] = x;
  }
  const int nsrc = gridDim.y, n = nsrc * NS;
  for (int i = threadIdx.x; i < n; i += blockDim.x) row[i] = 0.0;
  __syncthreads();
  if (threadIdx.x < NS) {
    double t = 0;
    for (int w = 0; w < nwarps; w++) t += smem[w * NS + threadIdx.x];
    row[s * NS + threadIdx.x] = t;
  }
  __syncthreads();
  // each block's row carries its own source's NS sums and zeros elsewhere
  if (!grid_reduce_last(row, n, red, tot, scratch)) return;
  if (threadIdx.x == 0 && totals)
    for (int i = 0; i < n; i++) totals[i] = tot[i];
  __syncthreads();
  fin(tot, nsrc);
}

}  // namespace mks
