// Connected components in one pass over the edges (the CC app with
// fuse_kernel on): a lock-free union-find whose roots are always the smallest
// id of their tree.
//
//   init    parent[v] = min(v, first neighbour of v)  (adjacency lists are sorted,
//           so that is v's smallest neighbour)
//   edges   union(u, v): find both roots with path halving; hook the larger root
//           under the smaller with a CAS; retry from the new roots if another
//           thread hooked first
//   final   label[v] = find(v)
//
// Every step keeps parent[x] <= x, so a tree's root is its smallest vertex and
// the final labels are the minimum id of each (weakly) connected component --
// the canonical labels cc.cpp's hook / pointer-jump rounds converge to
// (apps/cc.cpp:23-77).  A symmetric graph stores each edge twice; one direction
// is enough.  Concurrent path-halving stores only ever move a vertex up its own
// tree, so the races are benign.
#include "engine.h"

namespace gg {

__device__ __forceinline__ int32_t uf_find(int32_t *parent, int32_t x) {
  for (;;) {
    const int32_t p = __ldcg(parent + x);
    if (p == x) return x;
    const int32_t gp = __ldcg(parent + p);
    if (gp == p) return p;
    parent[x] = gp;  // path halving
    x = gp;
  }
}

__device__ __forceinline__ void uf_union(int32_t *parent, int32_t u, int32_t v) {
  int32_t ru = uf_find(parent, u), rv = uf_find(parent, v);
  while (ru != rv) {
    if (ru < rv) {
      const int32_t t = ru;
      ru = rv;
      rv = t;
    }
    const int32_t old = atomicCAS(parent + ru, ru, rv);  // hook the larger root
    if (old == ru) return;
    ru = uf_find(parent, old);
    rv = uf_find(parent, rv);
  }
}

__global__ void k_uf_init(const int32_t *__restrict__ off, const int32_t *__restrict__ dst, int32_t V,
                          int32_t *__restrict__ parent) {
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    const int32_t b = off[v];
    parent[v] = (off[v + 1] > b) ? min(v, dst[b]) : v;
  }
}

__global__ void k_uf_edges(const int32_t *__restrict__ src, const int32_t *__restrict__ dst, int64_t E,
                           int32_t symmetric, int32_t *__restrict__ parent) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < E; k += (int64_t)gridDim.x * blockDim.x) {
    const int32_t u = src[k], v = dst[k];
    if (u == v || (symmetric && u < v)) continue;
    uf_union(parent, u, v);
  }
}

__global__ void k_uf_final(int32_t *__restrict__ parent, int32_t V, int32_t *__restrict__ labels) {
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
    labels[v] = uf_find(parent, v);
}

gg_status cc_union_find(gg_graph *g, int32_t *labels, int32_t *parent) {
  GG_TRY(ensure_coo(g->csr, g->stream));
  const GraphStore &f = g->csr;
  cudaStream_t st = g->stream;
  const int grid = g->sm_count * 8;
  note_launch();
  k_uf_init<<<grid, 256, 0, st>>>(f.off, f.dst, f.V, parent);
  note_launch();
  k_uf_edges<<<grid * 4, 256, 0, st>>>(f.src, f.dst, f.E, g->symmetric ? 1 : 0, parent);
  note_launch();
  k_uf_final<<<grid, 256, 0, st>>>(parent, f.V, labels);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

}  // namespace gg
