// Degree-ordered relabelling for the batched kernels.
//
// Batched SSSP keeps 32 distances (one 128-byte line) per vertex and reads the
// line of every neighbour it relaxes; on R-MAT graphs most relaxations land on
// the few vertices of high in-degree.  Renumbering vertices by descending
// in-degree class -- floor(log2(in-degree + 1)), stable by id inside a class --
// packs those lines together at the front of the array, where they stay in L2.
// The renumbered CSR, the map old -> new (perm) and new -> old (inv) are built
// once per graph on the device and kept with it; sources go through perm and
// result rows come back through it, so callers never see new ids.  Results are
// unchanged: the relabelled graph is isomorphic to the original.
#include "engine.h"
#include "scan.cuh"

namespace gg {

constexpr int32_t kRlClasses = 32;
constexpr int32_t kRlTile = 4096;  // vertices per block range of the counting sort

// Class key = 31 - floor(log2(in-degree + 1)): key 0 holds the largest in-degrees.
__device__ __forceinline__ int32_t rl_class_key(int32_t indeg) { return __clz((uint32_t)indeg + 1u); }

__global__ void k_rl_indeg(const int32_t *__restrict__ dst, int64_t E, int32_t *__restrict__ cnt) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < E; k += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(cnt + dst[k], 1);
}

__global__ void k_rl_outdeg(const int32_t *__restrict__ off, int32_t V, int32_t *__restrict__ cnt) {
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
    cnt[v] = off[v + 1] - off[v];
}

// hist[key * nb + b] = vertices of class key in block b's range.
__global__ void __launch_bounds__(256) k_rl_hist(const int32_t *__restrict__ indeg, int32_t V, int32_t nb,
                                                 int32_t *__restrict__ hist) {
  __shared__ int32_t h[kRlClasses];
  if (threadIdx.x < kRlClasses) h[threadIdx.x] = 0;
  __syncthreads();
  const int32_t b = blockIdx.x, v0 = b * kRlTile, v1 = min(V, v0 + kRlTile);
  for (int32_t v = v0 + threadIdx.x; v < v1; v += blockDim.x) atomicAdd(h + rl_class_key(indeg[v]), 1);
  __syncthreads();
  if (threadIdx.x < kRlClasses) hist[threadIdx.x * nb + b] = h[threadIdx.x];
}

// Stable scatter: block b walks its range in order, 256 vertices at a time;
// a vertex's new id = base[key][b] + earlier vertices of its class in the range.
__global__ void __launch_bounds__(256) k_rl_scatter(const int32_t *__restrict__ indeg, int32_t V, int32_t nb,
                                                    const int32_t *__restrict__ base, int32_t *__restrict__ perm,
                                                    int32_t *__restrict__ inv) {
  __shared__ int32_t run[kRlClasses];        // vertices of each class placed so far
  __shared__ int32_t wcnt[8][kRlClasses];    // per-warp counts of the current chunk
  const int32_t b = blockIdx.x, v0 = b * kRlTile, v1 = min(V, v0 + kRlTile);
  const int32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (threadIdx.x < kRlClasses) run[threadIdx.x] = base[threadIdx.x * nb + b];
  __syncthreads();
  for (int32_t c0 = v0; c0 < v1; c0 += blockDim.x) {
    const int32_t v = c0 + threadIdx.x;
    const int32_t key = v < v1 ? rl_class_key(indeg[v]) : -1;
    // rank among earlier lanes of the same class, and the warp's class counts
    int32_t rank = 0;
    for (int32_t k = 0; k < kRlClasses; ++k) {
      const uint32_t m = __ballot_sync(0xffffffffu, key == k);
      if (key == k) rank = __popc(m & ((1u << lane) - 1u));
      if (lane == 0) wcnt[wid][k] = __popc(m);
    }
    __syncthreads();
    if (key >= 0) {
      int32_t before = 0;
      for (int32_t w = 0; w < wid; ++w) before += wcnt[w][key];
      const int32_t nid = run[key] + before + rank;
      perm[v] = nid;
      inv[nid] = v;
    }
    __syncthreads();
    if (threadIdx.x < kRlClasses) {
      int32_t tot = 0;
      for (int32_t w = 0; w < (int32_t)(blockDim.x >> 5); ++w) tot += wcnt[w][threadIdx.x];
      run[threadIdx.x] += tot;
    }
    __syncthreads();
  }
}

struct RlDegIn {  // out-degree of the vertex now numbered i
  const int32_t *off, *inv;
  __device__ int32_t operator()(int64_t i) const { return off[inv[i] + 1] - off[inv[i]]; }
};

struct RlHistIn {
  const int32_t *a;
  __device__ int32_t operator()(int64_t i) const { return a[i]; }
};

// Warp per new vertex: its list, neighbours renamed, weights carried along.
__global__ void k_rl_lists(const int32_t *__restrict__ off, const int32_t *__restrict__ dst,
                           const int32_t *__restrict__ w, const int32_t *__restrict__ perm,
                           const int32_t *__restrict__ inv, int32_t V, const int32_t *__restrict__ noff,
                           int32_t *__restrict__ ndst, int32_t *__restrict__ nw) {
  const int32_t lane = threadIdx.x & 31;
  for (int32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < V; i += (gridDim.x * blockDim.x) >> 5) {
    const int32_t u = inv[i];
    const int32_t b = off[u], n = off[u + 1] - b, o = noff[i];
    for (int32_t j = lane; j < n; j += 32) {
      ndst[o + j] = perm[dst[b + j]];
      nw[o + j] = w[b + j];
    }
  }
}

gg_status ensure_relabel(gg_graph *g) {
  if (g->rel) return GG_OK;
  cudaStream_t st = g->stream;
  const GraphStore &f = g->csr;
  const int32_t V = f.V;
  auto r = std::make_unique<Relabeled>();
  r->g.V = V;
  r->g.E = f.E;
  const int32_t nb = std::max(1, ceil_div(V, kRlTile));
  int32_t *indeg = nullptr, *hist = nullptr, *base = nullptr, *partial = nullptr;
  GG_CUDA(dev_alloc(&r->perm, sizeof(int32_t) * std::max(V, 1), st));
  GG_CUDA(dev_alloc(&r->inv, sizeof(int32_t) * std::max(V, 1), st));
  GG_CUDA(dev_alloc(&r->g.off, sizeof(int32_t) * (V + 1), st));
  GG_CUDA(dev_alloc(&r->g.dst, sizeof(int32_t) * std::max(f.E, 1), st));
  GG_CUDA(dev_alloc(&r->g.w, sizeof(int32_t) * std::max(f.E, 1), st));
  GG_CUDA(dev_alloc(&indeg, sizeof(int32_t) * std::max(V, 1), st));
  GG_CUDA(dev_alloc(&hist, sizeof(int32_t) * kRlClasses * nb, st));
  GG_CUDA(dev_alloc(&base, sizeof(int32_t) * (kRlClasses * nb + 1), st));
  const size_t scan_n = std::max<size_t>(V, (size_t)kRlClasses * nb);
  GG_CUDA(dev_alloc(&partial, sizeof(int32_t) * scan_scratch_ints((int64_t)scan_n), st));
  const int grid = g->sm_count * 8;
  if (g->symmetric) {
    note_launch();
    k_rl_outdeg<<<grid, 256, 0, st>>>(f.off, V, indeg);
  } else {
    GG_CUDA(cudaMemsetAsync(indeg, 0, sizeof(int32_t) * std::max(V, 1), st));
    note_launch();
    k_rl_indeg<<<grid, 256, 0, st>>>(f.dst, f.E, indeg);
  }
  note_launch();
  k_rl_hist<<<nb, 256, 0, st>>>(indeg, V, nb, hist);
  GG_CUDA(exclusive_scan(RlHistIn{hist}, (int64_t)kRlClasses * nb, base, partial, st));
  note_launch();
  k_rl_scatter<<<nb, 256, 0, st>>>(indeg, V, nb, base, r->perm, r->inv);
  GG_CUDA(exclusive_scan(RlDegIn{f.off, r->inv}, V, r->g.off, partial, st));
  note_launch();
  k_rl_lists<<<grid, 256, 0, st>>>(f.off, f.dst, f.w, r->perm, r->inv, V, r->g.off, r->g.dst, r->g.w);
  GG_CUDA(cudaGetLastError());
  for (void *p : {(void *)indeg, (void *)hist, (void *)base, (void *)partial}) cudaFreeAsync(p, st);
  g->rel = std::move(r);
  return GG_OK;
}

// The renumbered in-lists: row i holds the in-neighbours of inv[i], renamed.
gg_status ensure_relabel_csc(gg_graph *g) {
  if (!g->rel) return set_error(GG_ERR_STATE, "relabelled graph missing");
  if (g->symmetric || g->rel->csc.off) return GG_OK;  // a symmetric graph's CSR is its CSC
  GG_TRY(ensure_transpose(g));
  cudaStream_t st = g->stream;
  const GraphStore &t = *g->csc;
  Relabeled &r = *g->rel;
  const int32_t V = t.V;
  int32_t *partial = nullptr;
  GG_CUDA(dev_alloc(&r.csc.off, sizeof(int32_t) * (V + 1), st));
  GG_CUDA(dev_alloc(&r.csc.dst, sizeof(int32_t) * std::max(t.E, 1), st));
  GG_CUDA(dev_alloc(&r.csc.w, sizeof(int32_t) * std::max(t.E, 1), st));
  GG_CUDA(dev_alloc(&partial, sizeof(int32_t) * scan_scratch_ints(V), st));
  r.csc.V = V;
  r.csc.E = t.E;
  GG_CUDA(exclusive_scan(RlDegIn{t.off, r.inv}, V, r.csc.off, partial, st));
  note_launch();
  k_rl_lists<<<g->sm_count * 8, 256, 0, st>>>(t.off, t.dst, t.w, r.perm, r.inv, V, r.csc.off, r.csc.dst, r.csc.w);
  GG_CUDA(cudaGetLastError());
  cudaFreeAsync(partial, st);
  return GG_OK;
}

void free_relabel(gg_graph *g) {
  if (!g->rel) return;
  cudaStream_t st = g->stream;
  for (void *p : {(void *)g->rel->perm, (void *)g->rel->inv, (void *)g->rel->g.off, (void *)g->rel->g.dst,
                  (void *)g->rel->g.w, (void *)g->rel->csc.off, (void *)g->rel->csc.dst, (void *)g->rel->csc.w})
    if (p) cudaFreeAsync(p, st);
  g->rel.reset();
}

}  // namespace gg
