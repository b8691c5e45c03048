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
// writeMin(&SP[dst], SP[src]+w) && new < prio_cutoff  => enqueue dst.
struct USssp {
  static constexpr bool kWeight = true;
  int32_t *dist;
  int32_t cutoff;
  __device__ __forceinline__ bool filter(int32_t) const { return true; }
  __device__ __forceinline__ bool apply(int32_t s, int32_t d, int32_t w) const {
    const int32_t ds = vload(dist + s);
    if (ds == INT_MAX) return false;
    const int32_t np = ds + w;
    return write_min(dist + d, np) && np < cutoff;
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
template <class U, bool PULL>
struct EdgeF {
  static constexpr bool kWeight = U::kWeight;
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
};

}  // namespace gg
