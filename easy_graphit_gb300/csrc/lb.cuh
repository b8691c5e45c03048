// Load-balancing strategies of GraphIt's edgeset.apply
// (src/graphit/operators.cpp:72-492), each written as a device function that
// processes one *virtual CTA* of work.  Kernels (unfused launches, persistent
// fused kernels) loop over virtual CTAs, so every strategy runs unchanged in
// both modes -- the multiplexing the reference does for fused kernels
// (operators.cpp:337-342) is the normal path here.
//
// F is an edge functor (udf.cuh) with
//   bool src_ok(s)  -- source filter, checked before every edge (pull early exit)
//   bool dst_ok(d)  -- destination filter
//   int  apply(s, d, w) -> vertex to enqueue into the output frontier or -1
//   static constexpr bool kWeight -- whether apply reads the edge weight
#pragma once

#include "common.cuh"

namespace gg {

constexpr int kStage1 = 8;  // TWCE stage-1 group width (operators.cpp:201)

template <class F>
__device__ __forceinline__ void do_edge(const DGraph &g, const F &f, const DOut &out, int32_t s,
                                        int32_t k) {
  const int32_t d = __ldg(g.dst + k);
  if (!f.dst_ok(d)) return;
  const int32_t w = F::kWeight ? __ldg(g.w + k) : 0;
  const int32_t t = f.apply(s, d, w);
  if (t >= 0) out.push(t);
}

template <class F, class = void>
struct lb_batch {
  static constexpr bool value = false;
};
template <class F>
struct lb_batch<F, decltype(void(F::kBatch))> {
  static constexpr bool value = F::kBatch;
};

// Edges [b, e) of source s processed by `width` cooperating threads (rank r).
// A functor with a batched range relax (push, no per-edge source test beyond
// the first) takes the whole range at once.
template <class F>
__device__ __forceinline__ void do_range(const DGraph &g, const F &f, const DOut &out, int32_t s,
                                         int32_t b, int32_t e, int32_t r, int32_t width) {
  if constexpr (lb_batch<F>::value) {
    if (b + r < e && f.src_ok(s)) f.relax_range(g, out, s, b, e, r, width);
    return;
  }
  for (int32_t k = b + r; k < e; k += width) {
    if (!f.src_ok(s)) break;
    do_edge(g, f, out, s, k);
  }
}

// ------------------------------------------------------------ VERTEX_BASED
// One thread per enumerated vertex, serial neighbour loop with the early exit
// of operators.cpp:83-94.  Virtual CTA = blockDim.x vertices.
template <class F>
__device__ __forceinline__ void lb_vertex(const DGraph &g, const Enum &en, int32_t n, const F &f,
                                          const DOut &out, int32_t vcta) {
  const int32_t i = vcta * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t s = en.at(i);
  do_range(g, f, out, s, __ldg(g.off + s), __ldg(g.off + s + 1), 0, 1);
}

// ---------------------------------------------------------------------- WM
// Warp-mapped: one warp per enumerated vertex, lanes stride the neighbour list
// (coalesced dst loads).  Virtual CTA = blockDim.x/32 vertices.  No reference
// implementation (schedule.h lists WM, operators.cpp:645-646 rejects it).
template <class F>
__device__ __forceinline__ void lb_wm(const DGraph &g, const Enum &en, int32_t n, const F &f,
                                      const DOut &out, int32_t vcta) {
  const int32_t nw = blockDim.x >> 5;
  const int32_t i = vcta * nw + (threadIdx.x >> 5);
  if (i >= n) return;
  const int32_t s = en.at(i);
  do_range(g, f, out, s, __ldg(g.off + s), __ldg(g.off + s + 1), threadIdx.x & 31, 32);
}

// -------------------------------------------------------------------- TWCE
// Thread/warp/CTA binning inside one CTA (operators.cpp:203-323): 8 threads
// read one vertex; its degree splits into a CTA part (multiples of blockDim),
// a warp part (multiples of 32) and a remainder for the 8-thread group.
// Warp-bin entries are taken round-robin by the warps, CTA-bin entries by the
// whole CTA.  Virtual CTA = blockDim.x/8 vertices.
struct TwceSmem {
  int32_t nw, nc;
  int32_t data[1];  // 6 * (blockDim/8) ints: warp bin (s,b,e), CTA bin (s,b,e)
};
__host__ __device__ inline size_t twce_smem_bytes(int cta) {
  return sizeof(int32_t) * (2 + 6 * (cta / kStage1)) + 16;
}

template <class F, bool kCtaBin = true>
__device__ __forceinline__ void lb_twce(const DGraph &g, const Enum &en, int32_t n, const F &f,
                                        const DOut &out, int32_t vcta, TwceSmem &sm,
                                        int32_t *chunk_list = nullptr, int32_t *chunk_cnt = nullptr,
                                        int32_t chunk = 0) {
  const int32_t per = blockDim.x / kStage1;
  int32_t *wv = sm.data, *wb = wv + per, *we = wb + per;
  int32_t *cv = we + per, *cb = cv + per, *ce = cb + per;
  if (threadIdx.x == 0) {
    sm.nw = 0;
    sm.nc = 0;
  }
  __syncthreads();
  const int32_t sub = threadIdx.x & (kStage1 - 1);
  const int32_t i = vcta * per + (int32_t)(threadIdx.x / kStage1);
  int32_t s = -1, b = 0, e = 0;
  if (i < n) {
    s = en.at(i);
    b = __ldg(g.off + s);
    e = __ldg(g.off + s + 1);
    const int32_t deg = e - b;
    const int32_t big = deg / (int32_t)blockDim.x * (int32_t)blockDim.x;
    const int32_t mid = (deg - big) / 32 * 32;
    if (sub == 0) {
      if (big) {
        if (kCtaBin) {
          const int32_t p = atomicAdd(&sm.nc, 1);
          cv[p] = s;
          cb[p] = b;
          ce[p] = b + big;
        } else {
          // ETWC: hub edges become fixed-size chunks on a global list that all
          // CTAs drain afterwards.
          const int32_t nch = ceil_div(big, chunk);
          const int32_t p = atomicAdd(chunk_cnt, nch);
          for (int32_t c = 0; c < nch; ++c) {
            chunk_list[3 * (p + c) + 0] = s;
            chunk_list[3 * (p + c) + 1] = b + c * chunk;
            chunk_list[3 * (p + c) + 2] = min(b + (c + 1) * chunk, b + big);
          }
        }
      }
      if (mid) {
        const int32_t p = atomicAdd(&sm.nw, 1);
        wv[p] = s;
        wb[p] = b + big;
        we[p] = b + big + mid;
      }
    }
    b += big + mid;
  }
  __syncthreads();
  if (s >= 0) do_range(g, f, out, s, b, e, sub, kStage1);  // stage 1
  const int32_t nw = sm.nw;
  for (int32_t j = (int32_t)(threadIdx.x >> 5); j < nw; j += (int32_t)(blockDim.x >> 5))  // stage 2
    do_range(g, f, out, wv[j], wb[j], we[j], threadIdx.x & 31, 32);
  if (kCtaBin) {
    const int32_t nc = sm.nc;
    for (int32_t j = 0; j < nc; ++j)  // stage 3
      do_range(g, f, out, cv[j], cb[j], ce[j], threadIdx.x, blockDim.x);
  }
  __syncthreads();
}

// ETWC second phase: a virtual CTA processes one hub chunk.
template <class F>
__device__ __forceinline__ void lb_chunk(const DGraph &g, const int32_t *chunk_list, const F &f,
                                         const DOut &out, int32_t vcta) {
  const int32_t s = chunk_list[3 * vcta], b = chunk_list[3 * vcta + 1], e = chunk_list[3 * vcta + 2];
  do_range(g, f, out, s, b, e, threadIdx.x, blockDim.x);
}

// ---------------------------------------------------------------------- CM
// CTA-wide exclusive scan of the degrees of blockDim.x frontier vertices, then
// every thread takes edges i, i+blockDim.x, ... and finds its source by an
// upper-bound search in the scan (operators.cpp:359-457).  The reference passes
// weight 0 to the UDF here (operators.cpp:451-452); this one passes the edge's
// weight.
struct CmSmem {
  int32_t total;
  int32_t warp_sums[32];
  int32_t data[1];  // 3*blockDim ints: vertex, begin, exclusive scan
};
__host__ __device__ inline size_t cm_smem_bytes(int cta) {
  return sizeof(int32_t) * (1 + 32 + 3 * cta) + 16;
}

// Block-wide exclusive scan of x; returns the exclusive prefix, total in *tot.
__device__ __forceinline__ int32_t block_exclusive_scan(int32_t x, int32_t *warp_sums,
                                                        int32_t *tot) {
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
    if (lane < nwarps) warp_sums[lane] = ws;  // inclusive over warps
  }
  __syncthreads();
  const int32_t base = wid ? warp_sums[wid - 1] : 0;
  *tot = warp_sums[(blockDim.x >> 5) - 1];
  return base + v - x;
}

template <class F>
__device__ __forceinline__ void lb_cm(const DGraph &g, const Enum &en, int32_t n, const F &f,
                                      const DOut &out, int32_t vcta, CmSmem &sm) {
  const int32_t C = blockDim.x;
  int32_t *sv = sm.data, *sb = sv + C, *sx = sb + C;
  const int32_t i = vcta * C + threadIdx.x;
  int32_t deg = 0;
  if (i < n) {
    const int32_t s = en.at(i);
    const int32_t b = __ldg(g.off + s);
    deg = __ldg(g.off + s + 1) - b;
    sv[threadIdx.x] = s;
    sb[threadIdx.x] = b;
  }
  int32_t total;
  const int32_t ex = block_exclusive_scan(deg, sm.warp_sums, &total);
  sx[threadIdx.x] = ex;
  __syncthreads();
  const int32_t width = min(C, n - vcta * C);
  for (int32_t e = threadIdx.x; e < total; e += C) {
    // upper_bound(sx[0..width), e) - 1
    int32_t lo = 0, len = width;
    while (len > 0) {
      const int32_t half = len >> 1;
      if (sx[lo + half] > e) {
        len = half;
      } else {
        lo += half + 1;
        len -= half + 1;
      }
    }
    const int32_t j = lo - 1;
    const int32_t s = sv[j];
    if (!f.src_ok(s)) continue;
    do_edge(g, f, out, s, sb[j] + e - sx[j]);
  }
  __syncthreads();
}

// ------------------------------------------------------------------ STRICT
// Edge-balanced over the whole frontier: `sum` holds the exclusive scan of the
// enumerated vertices' degrees (n+1 entries); virtual CTA c owns edge ranks
// [c*per, (c+1)*per).  (The reference allocates strict_* scratch,
// graph.h:56-59, but implements no kernel.)
template <class F>
__device__ __forceinline__ void lb_strict(const DGraph &g, const Enum &en, int32_t n,
                                          const int32_t *__restrict__ sum, const F &f,
                                          const DOut &out, int32_t vcta, int32_t per) {
  const int64_t total = sum[n];
  const int64_t r0 = (int64_t)vcta * per;
  const int64_t r1 = r0 + per < total ? r0 + per : total;
  for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
    int32_t lo = 0, len = n;
    while (len > 0) {
      const int32_t half = len >> 1;
      if (__ldg(sum + lo + half) > r) {
        len = half;
      } else {
        lo += half + 1;
        len -= half + 1;
      }
    }
    const int32_t j = lo - 1;
    const int32_t s = en.at(j);
    if (!f.src_ok(s)) continue;
    do_edge(g, f, out, s, __ldg(g.off + s) + (int32_t)(r - __ldg(sum + j)));
  }
}

// --------------------------------------------------------------- EDGE_ONLY
// Thread per COO edge over every edge of the graph (operators.cpp:175-200);
// both endpoints go through the filters.  `r`/`width` index the calling
// thread within the grid.
template <class F>
__device__ __forceinline__ void lb_edge_only(const DGraph &g, const F &f, const DOut &out,
                                             int64_t r, int64_t width) {
  for (int64_t k = r; k < g.E; k += width) {
    const int32_t s = __ldg(g.src + k);
    if (!f.src_ok(s)) continue;
    do_edge(g, f, out, s, (int32_t)k);
  }
}

// Blocked variant (operators.cpp:131-172): edges bucketed by destination
// block, buckets walked in order with a CTA barrier between them so the CTAs
// of a wave work on the same block of destinations.
template <class F>
__device__ __forceinline__ void lb_edge_only_blocked(const DGraph &g, const F &f, const DOut &out,
                                                     int64_t r, int64_t width) {
  for (int32_t b = 0; b < g.nbuckets; ++b) {
    const int32_t e1 = __ldg(g.bucket + b + 1);
    for (int64_t k = __ldg(g.bucket + b) + r; k < e1; k += width) {
      const int32_t s = __ldg(g.src + k);
      if (!f.src_ok(s)) continue;
      do_edge(g, f, out, s, (int32_t)k);
    }
    __syncthreads();
  }
}

}  // namespace gg
