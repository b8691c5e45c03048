// Device-side building blocks of the engine: graph and frontier views passed
// to kernels by value, the enqueue primitives of runtime/infra_gpu/
// vertex_frontier.h:176-216 and support.h:14-54 re-done for sm_103a, and a
// bounded grid barrier for persistent kernels.
#pragma once

#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <climits>
#include <cstdint>

#include "gg_internal.h"

namespace cg = cooperative_groups;

namespace gg {

// Error bits of the per-graph device status word.
enum : int32_t {
  DEV_ERR_OVERFLOW = 1,  // a sparse queue ran past its capacity
  DEV_ERR_TIMEOUT = 2,   // a grid barrier wait gave up
};

// --------------------------------------------------------------- graph view
// CSR (or CSC for a transposed graph) plus optional COO sources and dst-block
// buckets, as in graphit_runtime::GraphT (graph.h:17-88).
struct DGraph {
  int32_t V;
  int32_t E;
  const int32_t *__restrict__ off;     // V+1
  const int32_t *__restrict__ dst;     // E
  const int32_t *__restrict__ w;       // E
  const int32_t *__restrict__ src;     // E (COO row of each edge), may be null
  const int32_t *__restrict__ bucket;  // nbuckets+1 bucket starts (blocked graphs)
  int32_t nbuckets;
};

// Which vertices an LB kernel enumerates: q[0..n) or 0..n when q is null.
struct Enum {
  const int32_t *__restrict__ q;
  const int32_t *__restrict__ n_dev;  // device count (read when n < 0)
  int32_t n;
  __device__ __forceinline__ int32_t count() const {
    return n >= 0 ? n : *(volatile const int32_t *)n_dev;
  }
  // L2-coherent load: persistent kernels refill the queue they enumerate.
  __device__ __forceinline__ int32_t at(int32_t i) const { return q ? __ldcg(q + i) : i; }
};

// Membership test against an input frontier (bitmap / boolmap), or "all".
enum : int32_t { IN_ALL = 0, IN_BITMAP = 1, IN_BOOLMAP = 2 };
struct DIn {
  int32_t mode;
  const uint32_t *__restrict__ bm;
  const uint8_t *__restrict__ by;
  __device__ __forceinline__ bool has(int32_t v) const {
    if (mode == IN_ALL) return true;
    if (mode == IN_BITMAP) return (bm[v >> 5] >> (v & 31)) & 1u;
    return by[v] != 0;
  }
};

// Warp-aggregated counter increment (support.h:14-25 atomicAggInc), using a
// coalesced group so it is safe under independent thread scheduling.
__device__ __forceinline__ int32_t agg_inc(int32_t *ctr) {
  cg::coalesced_group g = cg::coalesced_threads();
  int32_t base = 0;
  if (g.thread_rank() == 0) base = atomicAdd(ctr, (int32_t)g.size());
  base = g.shfl(base, 0);
  return base + (int32_t)g.thread_rank();
}

// writeMin / writeMax / CAS of support.h:26-54: an early-out read, then the
// atomic; true when this call changed the value.
__device__ __forceinline__ bool write_min(int32_t *p, int32_t v) {
  if (*(volatile int32_t *)p <= v) return false;
  return atomicMin(p, v) > v;
}
__device__ __forceinline__ bool write_max(int32_t *p, int32_t v) {
  if (*(volatile int32_t *)p >= v) return false;
  return atomicMax(p, v) < v;
}
__device__ __forceinline__ bool cas(int32_t *p, int32_t expect, int32_t v) {
  if (*(volatile int32_t *)p != expect) return false;
  return atomicCAS(p, expect, v) == expect;
}

// Output frontier writer: the enqueue_* family of gpu_intrinsics.h:95-110.
enum : int32_t {
  OUT_NONE = 0,
  OUT_SPARSE = 1,        // enqueue_sparse (duplicates allowed)
  OUT_SPARSE_DEDUP = 2,  // enqueue_sparse_no_dupes (writeMax epoch counter)
  OUT_BITMAP = 3,        // enqueue_bitmap (atomicOr + count of new bits)
  OUT_BOOLMAP = 4,       // enqueue_boolmap (byte set + count of new bytes)
};
struct DOut {
  int32_t mode;
  int32_t *__restrict__ q;
  int32_t *cnt;
  int64_t cap;
  uint32_t *bm;
  uint8_t *by;
  int32_t *dedup;
  int32_t epoch;
  int32_t *err;

  __device__ __forceinline__ void sparse(int32_t v) const {
    const int32_t pos = agg_inc(cnt);
    if (pos < cap)
      q[pos] = v;
    else
      atomicOr(err, DEV_ERR_OVERFLOW);
  }
  __device__ __forceinline__ void push(int32_t v) const {
    switch (mode) {
      case OUT_SPARSE:
        sparse(v);
        break;
      case OUT_SPARSE_DEDUP:
        if (write_max(dedup + v, epoch)) sparse(v);
        break;
      case OUT_BITMAP: {
        const uint32_t bit = 1u << (v & 31);
        uint32_t *word = bm + (v >> 5);
        if (!(*(volatile uint32_t *)word & bit) && !(atomicOr(word, bit) & bit)) agg_inc(cnt);
        break;
      }
      case OUT_BOOLMAP: {
        // The reference sets the byte without an atomic and may count a vertex
        // twice (vertex_frontier.h:195-201); an OR on the containing word keeps
        // the count exact.
        if (by[v]) break;
        const uint32_t sh = 8u * (v & 3);
        uint32_t *word = reinterpret_cast<uint32_t *>(by + (v & ~3));
        if (!((atomicOr(word, 1u << sh) >> sh) & 0xffu)) agg_inc(cnt);
        break;
      }
      default:
        break;
    }
  }
};

// Far piles of the single-source delta-stepping queue (bucket_queue.cuh).  A
// relaxation that lowers P[v] to p at or above the window's cutoff parks v on
// the low pile (p below the horizon) or the high pile.  stamp[v] holds the tag
// of the pile generation that already lists v, so each vertex is listed at most
// once per pile: the exchange that writes the tag decides who appends.  With
// stamp == nullptr nothing is parked (a plain edgeset.apply of the relax UDF).
struct DFar {
  int32_t *stamp;           // [V]
  int32_t *lo, *lo_cnt;     // low pile of the current generation and its count
  int32_t *hi, *hi_cnt;     // high pile of the current generation and its count
  int32_t lo_tag, hi_tag;
  int32_t horizon;          // p < horizon -> low pile
  int32_t cap;              // entries a pile can hold (V)
  int32_t *err;

  __device__ __forceinline__ void park(int32_t v, int32_t p) const {
    const bool low = p < horizon;
    const int32_t tag = low ? lo_tag : hi_tag;
    if (atomicExch(stamp + v, tag) == tag) return;
    if (low) {
      const int32_t pos = agg_inc(lo_cnt);
      if (pos < cap)
        lo[pos] = v;
      else
        atomicOr(err, DEV_ERR_OVERFLOW);
    } else {
      const int32_t pos = agg_inc(hi_cnt);
      if (pos < cap)
        hi[pos] = v;
      else
        atomicOr(err, DEV_ERR_OVERFLOW);
    }
  }
};

// --------------------------------------------------------------- barriers
__device__ __forceinline__ uint32_t ld_acquire(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Grid-wide barrier for persistent (cooperatively launched) kernels.
// bar[0] = arrival count, bar[1] = generation.  The wait is bounded by
// timeout_ns; on expiry DEV_ERR_TIMEOUT is raised in *err and the function
// returns false so the caller can leave its loop.  Replaces
// cooperative_groups::this_grid().sync() (gpu_intrinsics.h:113-117), whose wait
// has no limit.
__device__ __forceinline__ bool grid_barrier(uint32_t *bar, uint32_t nblocks, int32_t *err,
                                             uint64_t timeout_ns) {
  __syncthreads();
  __shared__ int ok_s;
  if (threadIdx.x == 0) {
    ok_s = 1;
    const uint32_t gen = ld_acquire(bar + 1);
    __threadfence();
    const uint32_t arrived = atomicAdd(bar, 1u);
    if (arrived == nblocks - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      const uint64_t t0 = globaltimer_ns();
      uint32_t spins = 0;
      while (ld_acquire(bar + 1) == gen) {
        if ((++spins & 255u) == 0) {
          if (*(volatile int32_t *)err & DEV_ERR_TIMEOUT) { ok_s = 0; break; }
          if (globaltimer_ns() - t0 > timeout_ns) {
            atomicOr(err, DEV_ERR_TIMEOUT);
            ok_s = 0;
            break;
          }
        }
        __nanosleep(32);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok_s != 0;
}

// Waits, without arriving, until every other block has arrived at the next
// grid_barrier (bar[0] counts arrivals and the previous barrier's last block
// reset it, so nblocks-1 arrivals means all others are inside the wait).  The
// caller then works alone and completes the barrier by calling grid_barrier
// itself.  Bounded like grid_barrier; false after the limit.
__device__ __forceinline__ bool grid_wait_others(const uint32_t *bar, uint32_t nblocks, int32_t *err,
                                                 uint64_t timeout_ns) {
  __shared__ int ok_o;
  if (threadIdx.x == 0) {
    ok_o = 1;
    const uint64_t t0 = globaltimer_ns();
    uint32_t spins = 0;
    while (ld_acquire(bar) < nblocks - 1) {
      if ((++spins & 255u) == 0) {
        if (*(volatile int32_t *)err & DEV_ERR_TIMEOUT) { ok_o = 0; break; }
        if (globaltimer_ns() - t0 > timeout_ns) {
          atomicOr(err, DEV_ERR_TIMEOUT);
          ok_o = 0;
          break;
        }
      }
      __nanosleep(32);
    }
  }
  __syncthreads();
  return ok_o != 0;
}

// Wall-clock bound of a persistent loop.  In iteration `iter`, just before its
// closing grid barrier, block 0 checks the clock and, the first time it has
// passed, records DEV_ERR_TIMEOUT and writes iter + 1 into *stop: the number
// of the iteration at whose top every block leaves.  A number rather than a
// flag: a block that reads *stop late at the top of iteration `iter` (block 0
// may already be past that point) sees iter + 1 and goes on, so all blocks
// still leave together at the top of iteration iter + 1.
struct LoopClock {
  uint64_t deadline;
  __device__ __forceinline__ void start(uint64_t limit_ns) { deadline = globaltimer_ns() + limit_ns; }
  __device__ __forceinline__ void tick(int32_t *stop, int32_t iter, int32_t *err) const {
    if (blockIdx.x == 0 && threadIdx.x == 0 && globaltimer_ns() > deadline &&
        atomicCAS(stop, 0, iter + 1) == 0)
      atomicOr(err, DEV_ERR_TIMEOUT);
  }
};
// True at the top of iteration `iter` once a stop has been set for it.
__device__ __forceinline__ bool stopped(const int32_t *stop, int32_t iter) {
  const int32_t s = *(volatile const int32_t *)stop;
  return s != 0 && iter >= s;
}
// The same stop for a reason other than the clock (block 0, before the
// iteration's closing barrier): a sparse queue that overflowed.
__device__ __forceinline__ void stop_on_overflow(int32_t *stop, int32_t iter, const int32_t *err) {
  if (blockIdx.x == 0 && threadIdx.x == 0 && (*(volatile const int32_t *)err & DEV_ERR_OVERFLOW))
    atomicCAS(stop, 0, iter + 1);
}

__host__ __device__ __forceinline__ int32_t ceil_div(int64_t a, int64_t b) {
  return (int32_t)((a + b - 1) / b);
}

}  // namespace gg

#define GG_CUDA(call)                                                              \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess)                                                         \
      return gg::set_error(e_ == cudaErrorMemoryAllocation ? GG_ERR_OOM : GG_ERR_CUDA, \
                           "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                           __FILE__, __LINE__);                                    \
  } while (0)

#define GG_TRY(expr)                  \
  do {                                \
    gg_status s_ = (expr);            \
    if (s_ != GG_OK) return s_;       \
  } while (0)
