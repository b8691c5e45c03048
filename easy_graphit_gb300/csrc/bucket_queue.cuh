// Delta-stepping bucket queue for single-source runs: the next bucket of
// graphit_runtime::GPUPriorityQueue (runtime/infra_gpu/gpu_priority_queue.h:
// 115-153, 250-297) found from two far piles instead of two scans of all V.
//
// Reference rule (kept exactly): when the frontier runs empty, the window
// moves to cur = min{P[v] >= cur+delta, P[v] != INT_MAX} and every v with
// cur <= P[v] < cur+delta becomes the frontier.
//
// Why the piles hold every candidate: a vertex whose priority is at or above
// the window's cutoff got that priority from a relaxation at or above the
// cutoff of its own time (cutoffs only grow), and such a relaxation parks it
// (DFar::park).  Parking goes to the low pile when the priority is below the
// horizon and to the high pile otherwise; the tag in stamp[v] keeps a vertex
// listed at most once per pile generation, so a pile never holds more than V
// entries.  An entry whose vertex has since dropped below the cutoff was
// queued at that time and is stale; an advance skips it.
//
// An advance takes the exact minimum over the low pile (bq_pile_min): every
// pending vertex below the horizon is there, and every one in the high pile is
// at or above it.  The split (bq_pile_split) then sends window entries to the
// frontier and the rest to the next low-pile generation.  A window that
// reaches past the horizon also splits the high pile, with a new horizon
// above the window: a vertex parked high and later low sits on both piles
// then, so appends to the low pile exchange the tag and keep one copy.  When
// the low pile holds no live entry the high pile is scanned instead (a
// refill): its minimum starts the window, the new horizon is set a few buckets
// above it, and the split sends window entries to the frontier, entries below
// the horizon to the low pile and the rest to the next high generation.  The
// horizon width (in buckets) adapts so a refill moves about `fill_target`
// high entries to the low pile.
#pragma once

#include "common.cuh"

namespace gg {

// Pile tags: even for low-pile generations, odd for high ones; 0 = never
// parked (stamps are cleared at the start of every run).
__host__ __device__ __forceinline__ int32_t bq_lo_tag(int32_t gen) { return 2 * gen + 2; }
__host__ __device__ __forceinline__ int32_t bq_hi_tag(int32_t gen) { return 2 * gen + 1; }

__host__ __device__ __forceinline__ int32_t bq_clamp(int64_t x) {
  return x >= (int64_t)INT_MAX ? INT_MAX : (int32_t)x;
}

// Control words of one queue (ints).  Counts and minima used by the
// persistent loop rotate so that a step never clears a word another CTA may
// still read (fused.cu); the host-driven queue uses slot 0 of each.
enum : int32_t {
  BQ_NEAR = 0,    // [3] frontier counts, by step
  BQ_MIN = 3,     // [3] pile minima, by step
  BQ_LO = 6,      // [2] low-pile counts, by generation parity
  BQ_HI = 8,      // [2] high-pile counts, by generation parity
  BQ_FILL = 10,   // [2] entries a refill moved to the low pile, by high generation parity
  BQ_STOP = 12,   // loop time-limit flag
  BQ_STATS = 13,  // [2] relax steps, bucket advances
  BQ_PUB = 16,    // [16] loop state published by the one-CTA mode
  BQ_CTL_INTS = 32
};

// Device buffers of one queue: stamps, two generations of each pile, control.
struct BqBuffers {
  int32_t *stamp = nullptr;
  int32_t *lo[2] = {nullptr, nullptr};
  int32_t *hi[2] = {nullptr, nullptr};
  int32_t *ctl = nullptr;
  int32_t V = 0;
  void *base = nullptr;  // one allocation holds all of them
};

// Block-wide minimum; every thread of the block calls it; thread 0 gets it.
__device__ __forceinline__ int32_t bq_block_min(int32_t m, int32_t *red) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) m = min(m, __shfl_xor_sync(0xffffffffu, m, d));
  __syncthreads();  // red may still be read by a previous call
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : INT_MAX;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) m = min(m, __shfl_xor_sync(0xffffffffu, m, d));
  }
  return m;
}

// Minimum of the live priorities (>= U) listed in pile[0, n), folded into
// *out with one atomicMin per CTA.  CTA `rank` of `nparts` takes its share.
__device__ __forceinline__ void bq_pile_min(const int32_t *__restrict__ pile, int32_t n,
                                            const int32_t *P, int32_t U, int32_t *out, int32_t rank,
                                            int32_t nparts, int32_t *red) {
  int32_t m = INT_MAX;
  const int32_t stride = nparts * blockDim.x;
  constexpr int kIn = 4;  // entries per thread in flight
  for (int32_t i0 = rank * blockDim.x + threadIdx.x; i0 < n; i0 += kIn * stride) {
    int32_t v[kIn], p[kIn];
#pragma unroll
    for (int j = 0; j < kIn; ++j) v[j] = i0 + j * stride < n ? __ldcg(pile + i0 + j * stride) : -1;
#pragma unroll
    for (int j = 0; j < kIn; ++j) p[j] = v[j] >= 0 ? __ldcg(P + v[j]) : INT_MAX;
#pragma unroll
    for (int j = 0; j < kIn; ++j)
      if (p[j] >= U && p[j] < m) m = p[j];
  }
  m = bq_block_min(m, red);
  if (threadIdx.x == 0 && m != INT_MAX) atomicMin(out, m);
}

// Where bq_pile_split sends what it does not put on the frontier.
struct BqSplitOut {
  int32_t *stamp;
  int32_t *lo, *lo_cnt;
  int32_t lo_tag;
  int32_t *hi, *hi_cnt;  // null: everything goes to the low pile
  int32_t hi_tag;
  int32_t horizon;
  int32_t *fill;         // optional count of entries sent to the low pile
  int32_t cap;
  bool dedup;            // two piles feed the low pile in this step: append once per vertex
};

// Splits pile[0, n): stale entries (P < U) are dropped, the window
// [U', win_hi) goes to the frontier, the rest below the horizon to the low
// pile and the remainder to the high pile, each re-tagged with its new
// generation.  Every live entry has P >= the window start, so "P < win_hi" is
// the window test.
__device__ __forceinline__ void bq_pile_split(const int32_t *__restrict__ pile, int32_t n, const int32_t *P,
                                              int32_t U, int32_t win_hi, const DOut &front,
                                              const BqSplitOut &o, int32_t *err, int32_t rank,
                                              int32_t nparts) {
  const int32_t stride = nparts * blockDim.x;
  constexpr int kIn = 4;  // entries per thread in flight
  for (int32_t i0 = rank * blockDim.x + threadIdx.x; i0 < n; i0 += kIn * stride) {
    int32_t vs[kIn], ps[kIn];
#pragma unroll
    for (int j = 0; j < kIn; ++j) vs[j] = i0 + j * stride < n ? __ldcg(pile + i0 + j * stride) : -1;
#pragma unroll
    for (int j = 0; j < kIn; ++j) ps[j] = vs[j] >= 0 ? __ldcg(P + vs[j]) : -1;
#pragma unroll
    for (int j = 0; j < kIn; ++j) {
      const int32_t v = vs[j], p = ps[j];
      if (v < 0 || p < U) continue;
      if (p < win_hi) {
        front.sparse(v);
      } else if (!o.hi || p < o.horizon) {
        if (o.dedup) {
          if (atomicExch(o.stamp + v, o.lo_tag) == o.lo_tag) continue;
        } else {
          o.stamp[v] = o.lo_tag;
        }
        const int32_t pos = agg_inc(o.lo_cnt);
        if (pos < o.cap)
          o.lo[pos] = v;
        else
          atomicOr(err, DEV_ERR_OVERFLOW);
        if (o.fill) agg_inc(o.fill);
      } else {
        o.stamp[v] = o.hi_tag;
        const int32_t pos = agg_inc(o.hi_cnt);
        if (pos < o.cap)
          o.hi[pos] = v;
        else
          atomicOr(err, DEV_ERR_OVERFLOW);
      }
    }
  }
}

// Horizon width for the next refill from what the last one moved to the low
// pile (fill < 0: no refill yet).
__host__ __device__ __forceinline__ int32_t bq_adapt_width(int32_t k, int32_t fill, int32_t target) {
  if (fill < 0) return k;
  if (fill > 2 * target) return k > 1 ? k / 2 : 1;
  if (fill < target / 2) return k < (1 << 20) ? 2 * k : k;
  return k;
}

}  // namespace gg
