// mks_blas.cuh -- site-loop kernel framework for the Krylov BLAS steps.
//
// k_site<Op, NSUM, Fin> runs Op on every checkerboard site of one source
// per blockIdx.y, accumulates NSUM FP64 sums, reduces them
// deterministically (per-block partials, summed in a fixed order by the
// last block to arrive) and lets that last block run the finisher Fin,
// which updates the solver scalars held in device memory.
#pragma once
#include "mks_internal.cuh"
#include "mks_reduce.cuh"

namespace mks {

constexpr int BLAS_MAXSRC = 16;

template <class Op, int NSUM, class Fin>
__global__ void __launch_bounds__(256) k_site(const Op op, const Fin fin, const int *skip, int Vh,
                                              double *partials, unsigned int *count, double *totals) {
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
  __shared__ double tot[2 * BLAS_MAXSRC * NS];  // gridDim.y <= 2 * BLAS_MAXSRC
  __shared__ double scratch[32];
  __shared__ bool am_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < NS; k++) {
    double x = acc[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) smem[warp * NS + k] = x;
  }
  __syncthreads();
  const int gx = gridDim.x, nsrc = gridDim.y;
  if (threadIdx.x < NS) {
    double t = 0;
    for (int w = 0; w < nwarps; w++) t += smem[w * NS + threadIdx.x];
    partials[(size_t)(s * NS + threadIdx.x) * gx + blockIdx.x] = t;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) am_last = (atomicAdd(count, 1u) == (unsigned)(gx * nsrc) - 1);
  __syncthreads();
  if (!am_last) return;
  __threadfence();
  const int n = nsrc * NS;
  for (int i = 0; i < n; i++) {
    double a = 0;
    for (int b = threadIdx.x; b < gx; b += blockDim.x) a += ((volatile double *)partials)[(size_t)i * gx + b];
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (lane == 0) scratch[warp] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0;
      for (int w = 0; w < nwarps; w++) t += scratch[w];
      tot[i] = t;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    *count = 0;
    if (totals)
      for (int i = 0; i < n; i++) totals[i] = tot[i];
  }
  __syncthreads();
  fin(tot, nsrc);
}

}  // namespace mks
