// mks_reduce.cuh -- deterministic in-kernel FP64 reductions.
//
// Every thread contributes NSUM doubles per source.  A block reduces them
// with warp shuffles (keeping the G thread groups of a site apart) and
// shared memory, writes one partial per block, and the last block to
// arrive (arrival counter + __threadfence) sums the partials in a fixed
// order, so results do not depend on block scheduling.  The last block
// then runs a "finisher" that updates solver scalars on the device, so the
// host never waits on a reduction inside an iteration.
#pragma once
#include "mks_internal.cuh"

namespace mks {

// Block-wide reduction of vals[NV] (per thread) where thread t's values
// belong to slot (t % G)*NB + s for s < NB.  Result: tot[slot*NSUM + k] in
// shared memory on return (valid after the trailing __syncthreads), for
// slots < nslots = G*NB.  smem must hold (blockDim/32) * G*NB*NSUM doubles.
// The per-thread values and the warp-level shuffles use T (float in the
// sloppy solvers: GB300 runs FP64 at a small fraction of the FP32 rate, so
// per-site products and the first 32-way sums stay in FP32); from the warp
// totals on, everything is FP64.
template <typename T, int NB, int NSUM>
__device__ __forceinline__ void block_reduce_grouped(T (&v)[NB][NSUM], int G, double *smem) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int nslots = G * NB;
#pragma unroll
  for (int s = 0; s < NB; s++)
#pragma unroll
    for (int k = 0; k < NSUM; k++) {
      T x = v[s][k];
      for (int o = 16; o >= G; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
      v[s][k] = x;
    }
  if (lane < G) {
#pragma unroll
    for (int s = 0; s < NB; s++)
#pragma unroll
      for (int k = 0; k < NSUM; k++) smem[(warp * nslots + lane * NB + s) * NSUM + k] = (double)v[s][k];
  }
  __syncthreads();
  // sum over warps, in warp order
  for (int i = threadIdx.x; i < nslots * NSUM; i += blockDim.x) {
    double acc = 0;
    for (int w = 0; w < nwarps; w++) acc += smem[w * nslots * NSUM + i];
    smem[nwarps * nslots * NSUM + i] = acc;
  }
  __syncthreads();
}

// Writes this block's totals (n doubles in `tot`, shared) to the partial
// buffer, and returns true in the block that arrives last.  In that block,
// out[i] (shared, n doubles) holds the grid totals on return.
__device__ __forceinline__ bool grid_reduce_last(const double *tot, int n, double *partials,
                                                 unsigned int *count, double *out, double *scratch) {
  __shared__ bool am_last;
  const int nb = gridDim.x;
  for (int i = threadIdx.x; i < n; i += blockDim.x) partials[(size_t)i * nb + blockIdx.x] = tot[i];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned int prev = atomicAdd(count, 1u);
    am_last = (prev == (unsigned)nb - 1);
  }
  __syncthreads();
  if (!am_last) return false;
  __threadfence();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (int i = 0; i < n; i++) {
    double acc = 0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) acc += ((volatile double *)partials)[(size_t)i * nb + b];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) scratch[warp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0;
      for (int w = 0; w < nwarps; w++) t += scratch[w];
      out[i] = t;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *count = 0;  // ready for the next launch
  return true;
}

}  // namespace mks
