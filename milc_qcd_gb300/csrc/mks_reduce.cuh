// mks_reduce.cuh -- deterministic in-kernel FP64 reductions.
//
// Every thread contributes NSUM doubles per source.  A block reduces them
// with warp shuffles (keeping the G thread groups of a site apart) and
// shared memory, writes one row of partials per block, and a two-level
// last-block-to-arrive scheme sums the rows in a fixed order, so results
// do not depend on block scheduling.  The last block
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

// out[i] = sum over r < nrows of rows[r*n + i], i < n, summed by the whole
// block in an order fixed by (nrows, n, blockDim.x) alone.  The rows were
// written by other blocks of this launch, so they are read through L2
// (__ldcg; L1 is not coherent) with four independent loads in flight per
// thread.  scratch holds blockDim.x doubles.  Ends with __syncthreads.
__device__ __forceinline__ void sum_rows(const double *rows, int nrows, int n, double *out, double *scratch) {
  const int nt = blockDim.x, t = threadIdx.x;
  for (int i0 = 0; i0 < n; i0 += nt) {
    const int m = min(n - i0, nt), nchunk = nt / m, ch = t / m, i = i0 + t % m;
    if (ch < nchunk) {
      double a0 = 0, a1 = 0, a2 = 0, a3 = 0;
      int r = ch;
      for (; r + 3 * nchunk < nrows; r += 4 * nchunk) {
        a0 += __ldcg(rows + (size_t)r * n + i);
        a1 += __ldcg(rows + (size_t)(r + nchunk) * n + i);
        a2 += __ldcg(rows + (size_t)(r + 2 * nchunk) * n + i);
        a3 += __ldcg(rows + (size_t)(r + 3 * nchunk) * n + i);
      }
      for (; r < nrows; r += nchunk) a0 += __ldcg(rows + (size_t)r * n + i);
      scratch[t] = (a0 + a1) + (a2 + a3);
    }
    __syncthreads();
    if (t < m) {
      double acc = 0;
      for (int c = 0; c < nchunk; c++) acc += scratch[c * m + t];
      out[i0 + t] = acc;
    }
    __syncthreads();
  }
}

// Grid-wide sum of each block's n totals (`tot`, shared).  Two levels, each
// closed by the last block to arrive (arrival counters + __threadfence):
// the last block of every group of RED_GROUP consecutive blocks sums the
// group's rows into a group row, and the last group to finish sums the
// group rows.  Every sum runs in a fixed order, so the result does not
// depend on block scheduling.  Returns true in the one block that holds
// the grid totals in out[0..n) (shared) on return.
//
// red.partials: (nblocks + ngroups) * n doubles; red.count: 1 + ngroups
// counters, zero on entry and zero again when the launch ends.  scratch: blockDim.x
// doubles of shared memory.  The grid may be 2-D; blocks are numbered
// x-fastest.
__device__ __forceinline__ bool grid_reduce_last(const double *tot, int n, const RedScratch &red, double *out,
                                                 double *scratch) {
  __shared__ bool am_last;
  const int nb = gridDim.x * gridDim.y, bid = blockIdx.y * gridDim.x + blockIdx.x;
  const int ngroups = (nb + RED_GROUP - 1) / RED_GROUP, g = bid / RED_GROUP;
  const int gsize = min(RED_GROUP, nb - g * RED_GROUP);
  // the host sizes the scratch first (ensure_red); a launch that would not
  // fit writes nothing, flags the error and runs no finisher
  if ((size_t)(nb + ngroups) * n > red.max_partials || (size_t)(1 + ngroups) > red.max_count) {
    if (bid == 0 && threadIdx.x == 0) atomicExch(red.err, 1);
    return false;
  }
  double *partials = red.partials;
  unsigned int *count = red.count;
  double *grows = partials + (size_t)nb * n;
  // one thread writes the block's row, publishes it (fence) and arrives, so
  // a single fence per block orders every store the arrival covers
  if (threadIdx.x == 0) {
    for (int i = 0; i < n; i++) partials[(size_t)bid * n + i] = tot[i];
    __threadfence();
    am_last = (atomicAdd(&count[1 + g], 1u) == (unsigned)gsize - 1);
  }
  __syncthreads();
  if (!am_last) return false;
  __threadfence();
  sum_rows(partials + (size_t)g * RED_GROUP * n, gsize, n, out, scratch);  // out: shared staging
  if (threadIdx.x == 0) {
    for (int i = 0; i < n; i++) grows[(size_t)g * n + i] = out[i];
    count[1 + g] = 0;  // every block of the group has arrived
    __threadfence();
    am_last = (atomicAdd(&count[0], 1u) == (unsigned)ngroups - 1);
  }
  __syncthreads();
  if (!am_last) return false;
  __threadfence();
  sum_rows(grows, ngroups, n, out, scratch);
  if (threadIdx.x == 0) count[0] = 0;  // ready for the next launch
  return true;
}

}  // namespace mks
