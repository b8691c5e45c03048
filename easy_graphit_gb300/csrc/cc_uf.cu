// Connected components with fuse_kernel on: a lock-free union-find whose roots
// are always the smallest id of their tree, driven in the sampling order of
// Afforest (Sutton, Ben-Nun, Barak: "Optimizing Parallel Graph Connectivity
// Computation via Subgraph Sampling", IPDPS 2018).
//
//   init     parent[v] = min(v, first neighbour of v)  (adjacency lists are
//            sorted, so that is v's smallest neighbour)
//   sample   compress init's chains; union(v, first neighbour of v) where that
//            neighbour is larger (init joined a smaller one) and union(v, second
//            neighbour of v); compress every vertex to its root
//   giant    c = the most frequent root among 1,024 spread-out vertices
//   finish   every vertex whose root is not c unions with the rest of its
//            neighbours -- out-neighbours after the two sampled ones and, on a
//            directed graph, all in-neighbours -- so every edge with an end
//            outside c's tree is seen from that end; edges inside c's tree
//            change nothing and are skipped
//   final    label[v] = find(v)
//
// union(u, v) finds both roots with path halving and hooks the larger root
// under the smaller with a CAS, retrying from the new roots if another thread
// hooked first.  Every step keeps parent[x] <= x, so a tree's root is its
// smallest vertex and the final labels are the minimum id of each (weakly)
// connected component -- the canonical labels cc.cpp's hook / pointer-jump
// rounds converge to (apps/cc.cpp:23-77).  Concurrent path-halving stores only
// ever move a vertex up its own tree, so the races are benign.
#include <algorithm>
#include <vector>

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

// Link v with its out-neighbour number r (the sampling rounds).
__global__ void k_uf_sample(const int32_t *__restrict__ off, const int32_t *__restrict__ dst, int32_t V, int32_t r,
                            int32_t *__restrict__ parent) {
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    const int32_t b = off[v];
    if (off[v + 1] - b > r) {
      const int32_t u = dst[b + r];
      if (u != v && (r > 0 || u > v)) uf_union(parent, v, u);  // init joined a smaller first one
    }
  }
}

__global__ void k_uf_compress(int32_t *__restrict__ parent, int32_t V) {
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
    parent[v] = uf_find(parent, v);
}

// roots[i] = parent of vertex floor(i * V / n) (spread over the id range).
__global__ void k_uf_probe(const int32_t *__restrict__ parent, int32_t V, int32_t n, int32_t *__restrict__ roots) {
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    roots[i] = parent[(int32_t)((int64_t)i * V / n)];
}

// Unions of the vertices outside c's tree with list entries [off[v] + skip,
// off[v+1]).  A thread walks a short list; lists longer than 64 entries are
// walked by the whole warp, one after another.
__global__ void k_uf_finish(const int32_t *__restrict__ off, const int32_t *__restrict__ adj, int32_t V,
                            int32_t skip, int32_t c, int32_t *__restrict__ parent) {
  const int32_t lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t end = (V + stride - 1) / stride * stride;  // whole warps iterate together
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < end; i += stride) {
    const int32_t v = (int32_t)i;
    int32_t b = 0, e = 0;
    if (v < V && __ldcg(parent + v) != c) {
      b = off[v] + skip;
      e = off[v + 1];
    }
    uint32_t big = __ballot_sync(0xffffffffu, e - b > 64);
    while (big) {
      const int32_t l = __ffs(big) - 1;
      big &= big - 1;
      const int32_t vv = __shfl_sync(0xffffffffu, v, l);
      const int32_t bb = __shfl_sync(0xffffffffu, b, l), ee = __shfl_sync(0xffffffffu, e, l);
      for (int32_t k = bb + lane; k < ee; k += 32) {
        const int32_t u = adj[k];
        if (u != vv) uf_union(parent, vv, u);
      }
    }
    if (e - b <= 64)
      for (int32_t k = b; k < e; ++k) {
        const int32_t u = adj[k];
        if (u != v) uf_union(parent, v, u);
      }
  }
}

__global__ void k_uf_final(int32_t *__restrict__ parent, int32_t V, int32_t *__restrict__ labels) {
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
    labels[v] = uf_find(parent, v);
}

constexpr int32_t kUfProbes = 1024;

gg_status cc_union_find(gg_graph *g, int32_t *labels, int32_t *parent) {
  const GraphStore &f = g->csr;
  const int32_t V = f.V;
  if (V == 0) return GG_OK;
  if (!g->symmetric) GG_TRY(ensure_transpose(g));  // in-lists: weak components
  cudaStream_t st = g->stream;
  const int grid = g->sm_count * 8;
  note_launch();
  k_uf_init<<<grid, 256, 0, st>>>(f.off, f.dst, V, parent);
  // flatten init's first-neighbour chains before the unions walk them
  note_launch();
  k_uf_compress<<<grid, 256, 0, st>>>(parent, V);
  for (int32_t r = 0; r < 2; ++r) {
    note_launch();
    k_uf_sample<<<grid, 256, 0, st>>>(f.off, f.dst, V, r, parent);
  }
  note_launch();
  k_uf_compress<<<grid, 256, 0, st>>>(parent, V);
  // the giant tree's root, by majority over spread-out vertices
  const int32_t n = std::min(kUfProbes, std::max(V, 1));
  void *p = nullptr;
  GG_TRY(scratch_get(g, 1, sizeof(int32_t) * kUfProbes, &p));
  int32_t *d_roots = (int32_t *)p;
  note_launch();
  k_uf_probe<<<ceil_div(n, 256), 256, 0, st>>>(parent, V, n, d_roots);
  GG_CUDA(cudaGetLastError());
  std::vector<int32_t> roots(n);
  GG_CUDA(cudaMemcpyAsync(roots.data(), d_roots, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st));
  GG_CUDA(cudaStreamSynchronize(st));
  std::sort(roots.begin(), roots.end());
  int32_t c = V > 0 ? roots[0] : 0, best = 0;
  for (int32_t i = 0, j; i < n; i = j) {
    for (j = i; j < n && roots[j] == roots[i]; ++j) {
    }
    if (j - i > best) {
      best = j - i;
      c = roots[i];
    }
  }
  note_launch();
  k_uf_finish<<<grid, 256, 0, st>>>(f.off, f.dst, V, 2, c, parent);
  if (!g->symmetric) {
    note_launch();
    k_uf_finish<<<grid, 256, 0, st>>>(g->csc->off, g->csc->dst, V, 0, c, parent);
  }
  note_launch();
  k_uf_final<<<grid, 256, 0, st>>>(parent, V, labels);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

}  // namespace gg
