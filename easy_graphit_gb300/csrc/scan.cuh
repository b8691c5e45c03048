// Device-wide exclusive scan of int32 values produced by a functor, in three
// passes (per-tile sums, scan of tile sums, per-tile scan with offsets).
// out[0..n) = exclusive prefix, out[n] = total.
#pragma once

#include "common.cuh"

namespace gg {

constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int32_t block_scan_excl(int32_t x, int32_t *warp_sums, int32_t *total) {
  const int32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int32_t v = x;
#pragma unroll
  for (int32_t d = 1; d < 32; d <<= 1) {
    const int32_t t = __shfl_up_sync(0xffffffffu, v, d);
    if (lane >= d) v += t;
  }
  if (lane == 31) warp_sums[wid] = v;
  __syncthreads();
  if (wid == 0) {
    const int32_t nwarps = blockDim.x >> 5;
    int32_t ws = lane < nwarps ? warp_sums[lane] : 0;
#pragma unroll
    for (int32_t d = 1; d < 32; d <<= 1) {
      const int32_t t = __shfl_up_sync(0xffffffffu, ws, d);
      if (lane >= d) ws += t;
    }
    if (lane < nwarps) warp_sums[lane] = ws;
  }
  __syncthreads();
  const int32_t base = wid ? warp_sums[wid - 1] : 0;
  *total = warp_sums[(blockDim.x >> 5) - 1];
  __syncthreads();
  return base + v - x;
}

template <class In>
__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(In in, int64_t n, int32_t *partial) {
  __shared__ int32_t ws[32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int32_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i)
    if (base + i < n) s += in(base + i);
  int32_t tot;
  block_scan_excl(s, ws, &tot);
  if (threadIdx.x == 0) partial[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(1024) k_scan_partials(int32_t *partial, int32_t nb);

template <class In>
__global__ void __launch_bounds__(kScanThreads)
    k_scan_apply(In in, int64_t n, const int32_t *partial, int32_t *out) {
  __shared__ int32_t ws[32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int32_t vals[kScanItems];
  int32_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    vals[i] = base + i < n ? in(base + i) : 0;
    s += vals[i];
  }
  int32_t tot;
  int32_t run = block_scan_excl(s, ws, &tot) + partial[blockIdx.x];
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    if (base + i < n) out[base + i] = run;
    run += vals[i];
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) out[n] = run;
}

// Scratch needed for n items: one int per tile (+1).
inline size_t scan_scratch_ints(int64_t n) { return (size_t)((n + kScanTile - 1) / kScanTile) + 1; }

template <class In>
cudaError_t exclusive_scan(In in, int64_t n, int32_t *out, int32_t *partial, cudaStream_t st) {
  if (n <= 0) return cudaMemsetAsync(out, 0, sizeof(int32_t), st);
  const int32_t nb = (int32_t)((n + kScanTile - 1) / kScanTile);
  { gg::note_launch(); k_scan_tiles<In><<<nb, kScanThreads, 0, st>>>(in, n, partial); }
  { gg::note_launch(); k_scan_partials<<<1, 1024, 0, st>>>(partial, nb); }
  { gg::note_launch(); k_scan_apply<In><<<nb, kScanThreads, 0, st>>>(in, n, partial, out); }
  return cudaGetLastError();
}

}  // namespace gg
