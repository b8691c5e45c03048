// Edge UDFs of the five apps as device functors, and the direction wrapper
// that turns a UDF plus the to() filter into the src/dst filters of
// edgeset_apply::apply (operators.cpp:550-620).
#pragma once

#include "common.cuh"
#include "engine.h"

namespace gg {

template <class T>
__device__ __forceinline__ T vload(const T *p) {
  return *(volatile const T *)p;
}

// bfs.cpp:23-29: parent[dst] = src on unvisited dst; the shared write becomes
// CAS(&parent[dst], -1, src) (graphit.cpp:96-111) and the tracked parent
// enqueues dst.  depth[dst] = level is written with it.
struct UBfs {
  static constexpr bool kWeight = false;
  int32_t *parent, *depth;
  int32_t level;
  __device__ __forceinline__ bool filter(int32_t v) const { return vload(parent + v) == -1; }
  __device__ __forceinline__ bool apply(int32_t s, int32_t d, int32_t) const {
    if (!cas(parent + d, -1, s)) return false;
    if (depth) depth[d] = level;
    return true;
  }
};

// sssp.cpp:24-27 + PriorityQueue::updatePriorityMin (graphit_types.h:426-430):
// writeMin(&SP[dst], SP[src]+w) && new < prio_cutoff  => enqueue dst.  An
// improvement at or above the cutoff parks dst on the queue's far piles
// (when the queue keeps them), which is how the next bucket is found without
// scanning every vertex.
struct USssp {
  static constexpr bool kWeight = true;
  static constexpr bool kBatch = true;  // push relax over a range: relax_range
  static constexpr int kEdgesInFlight = 4;
  int32_t *dist;
  int32_t cutoff;
  DFar far;
  __device__ __forceinline__ bool filter(int32_t) const { return true; }
  __device__ __forceinline__ bool apply(int32_t s, int32_t d, int32_t w) const {
    const int32_t ds = vload(dist + s);
    if (ds == INT_MAX) return false;
    const int32_t np = ds + w;
    if (!write_min(dist + d, np)) return false;
    if (np < cutoff) return true;
    if (far.stamp) far.park(d, np);
    return false;
  }
  // Edges k = b + r, b + r + width, ... of source s, kEdgesInFlight at a time:
  // their targets and weights, then the targets' distances, then the
  // atomicMins of the improving ones are each issued together, so one thread
  // keeps that many edges in flight instead of one (a hub's list on a thread
  // of VERTEX_BASED is otherwise a chain of dependent round trips).  Same
  // outcome as apply() per edge: an improvement below the cutoff queues the
  // target, one above it parks it.
  template <class G, class Out>
  __device__ __forceinline__ void relax_range(const G &g, const Out &out, int32_t s, int32_t b, int32_t e,
                                              int32_t r, int32_t width) const {
    const int32_t ds = vload(dist + s);
    if (ds == INT_MAX) return;
    constexpr int B = kEdgesInFlight;
    for (int32_t k0 = b + r; k0 < e; k0 += B * width) {
      int32_t d[B], np[B], prev[B];
#pragma unroll
      for (int j = 0; j < B; ++j) {
        const int32_t k = k0 + j * width;
        d[j] = k < e ? __ldg(g.dst + k) : -1;
        np[j] = k < e ? ds + __ldg(g.w + k) : INT_MAX;
      }
#pragma unroll
      for (int j = 0; j < B; ++j) prev[j] = d[j] >= 0 ? __ldcg(dist + d[j]) : INT_MIN;
      // The minimum is a fire-and-forget reduction and the improvement is
      // decided against the value just read: a distance only decreases, so a
      // target read at or below np needs nothing, and one read above it is
      // queued or parked -- redundantly at worst, when a lighter path landed
      // in between (its own relaxation registers it too).
#pragma unroll
      for (int j = 0; j < B; ++j)
        if (np[j] < prev[j])
          asm volatile("red.relaxed.gpu.global.min.s32 [%0], %1;" ::"l"(__cvta_generic_to_global(dist + d[j])),
                       "r"(np[j])
                       : "memory");
#pragma unroll
      for (int j = 0; j < B; ++j) {
        if (prev[j] <= np[j]) continue;
        if (np[j] < cutoff)
          out.push(d[j]);
        else if (far.stamp)
          far.park(d[j], np[j]);
      }
    }
  }
};

// pr.cpp:32-34: new_rank[dst] += contrib[src] (fp32 atomicAdd, writeSum).
struct UPr {
  static constexpr bool kWeight = false;
  const float *contrib;
  float *new_rank;
  __device__ __forceinline__ bool filter(int32_t) const { return true; }
  __device__ __forceinline__ bool apply(int32_t s, int32_t d, int32_t) const {
    atomicAdd(new_rank + d, __ldg(contrib + s));
    return false;
  }
};

// cc.cpp:23-36: hook both endpoints' roots to the smaller label and raise
// updates[0] when something moved.  The min writes are always atomic here (the
// reference's access kind for ID[src_id] is left uninitialised,
// graphit_types.h:374-383).
struct UCc {
  static constexpr bool kWeight = false;
  int32_t *ids, *updates;
  __device__ __forceinline__ bool filter(int32_t) const { return true; }
  __device__ __forceinline__ bool apply(int32_t s, int32_t d, int32_t) const {
    const int32_t si = vload(ids + s), di = vload(ids + d);
    const int32_t ps = vload(ids + si), pd = vload(ids + di);
    if (ps == pd) return false;
    write_min(ids + si, pd);
    write_min(ids + di, ps);
    if (pd != vload(ids + di) || ps != vload(ids + si))
      if (vload(updates) == 0) updates[0] = 1;
    return false;
  }
};

// bc.cpp:34-40 forward: num_paths[dst] += num_paths[src] on unvisited dst; the
// tracked num_paths enqueues dst (deduplicated: allow_dupes=false).
struct UBcF {
  static constexpr bool kWeight = false;
  double *sigma;
  const uint8_t *visited;
  __device__ __forceinline__ bool filter(int32_t v) const { return vload(visited + v) == 0; }
  __device__ __forceinline__ bool apply(int32_t s, int32_t d, int32_t) const {
    atomicAdd(sigma + d, vload(sigma + s));
    return true;
  }
};

// bc.cpp:52-54 backward: dependences[dst] += dependences[src] on unvisited dst.
// T = float is the reference's VertexData<float>; gg_bc accumulates in double.
template <class T>
struct UBcB {
  static constexpr bool kWeight = false;
  T *dep;
  const uint8_t *visited;
  __device__ __forceinline__ bool filter(int32_t v) const { return vload(visited + v) == 0; }
  __device__ __forceinline__ bool apply(int32_t s, int32_t d, int32_t) const {
    atomicAdd(dep + d, vload(dep + s));
    return false;
  }
};

// Direction wrapper.  PUSH: enumerate sources, dst filter = to(); an EDGE_ONLY
// push with a from-frontier also requires the source to be a member (the
// reference iterates every edge and ignores the frontier, operators.cpp:186-195).
// PULL: enumerate the reverse frontier on the transposed graph, src filter =
// to() (checked before every edge: the early exit), dst filter = membership in
// the from-frontier, and the UDF called with swapped arguments.
template <class U, class = void>
struct batch_of {
  static constexpr bool value = false;
};
template <class U>
struct batch_of<U, decltype(void(U::kBatch))> {
  static constexpr bool value = U::kBatch;
};

template <class U, bool PULL>
struct EdgeF {
  static constexpr bool kWeight = U::kWeight;
  // push direction with a UDF that has a batched range relax (its to() filter
  // passes every vertex, so the range needs no per-edge destination test)
  static constexpr bool kBatch = !PULL && batch_of<U>::value;
  U u;
  DIn in_src, in_dst;
  bool filt;
  __device__ __forceinline__ bool src_ok(int32_t s) const {
    if (PULL) return !filt || u.filter(s);
    return in_src.has(s);
  }
  __device__ __forceinline__ bool dst_ok(int32_t d) const {
    if (PULL) return in_dst.has(d);
    return !filt || u.filter(d);
  }
  __device__ __forceinline__ int32_t apply(int32_t s, int32_t d, int32_t w) const {
    if (PULL) return u.apply(d, s, w) ? s : -1;
    return u.apply(s, d, w) ? d : -1;
  }
  // Only used when kBatch; the source filter (in_src) is checked by the caller.
  template <class G, class Out>
  __device__ __forceinline__ void relax_range(const G &g, const Out &out, int32_t s, int32_t b, int32_t e,
                                              int32_t r, int32_t width) const {
    if constexpr (kBatch) u.relax_range(g, out, s, b, e, r, width);
  }
};

}  // namespace gg
