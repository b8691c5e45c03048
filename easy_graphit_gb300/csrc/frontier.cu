// Vertex frontiers and vertex-level operators.
//  - graphit_runtime::VertexFrontier (runtime/infra_gpu/vertex_frontier.h) and
//    its representation changes (vertex_representation.h:72-158): sparse queue,
//    bitmap (uint32 words) and boolmap (bytes).  Conversions compact with warp
//    ballots (one atomic per warp) instead of one atomic per vertex.
//  - dedup_frontier_perfect (vertex_frontier.h:371-386).
//  - VertexFrontierList (list.h:18-116), the BC level stack.
//  - vertexset_apply (operators.cpp:10-65) with the apps' vertex UDFs.
//  - create_reverse_frontier (operators.cpp:494-512) for the pull direction.
#include <algorithm>
#include <vector>

#include "engine.h"
#include "scan.cuh"

namespace gg {

constexpr int kFrontierMultiplier = 6;  // FRONTIER_MULTIPLIER, vertex_frontier.h:6-8
constexpr int kThreads = 256;

static int grid_of(gg_graph *g) { return g->sm_count * 8; }

__global__ void k_iota(int32_t *q, int32_t n, int32_t *cnt) {
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) q[i] = i;
  if (blockIdx.x == 0 && threadIdx.x == 0) *cnt = n;
}

// Appends the lanes of a warp whose `pred` is set, in lane order, with one
// atomic per warp.  All 32 lanes must call it.
__device__ __forceinline__ void warp_append(bool pred, int32_t v, int32_t *q, int32_t *cnt) {
  const uint32_t m = __ballot_sync(0xffffffffu, pred);
  if (!m) return;
  const int32_t lane = threadIdx.x & 31;
  int32_t base = 0;
  if (lane == 0) base = atomicAdd(cnt, __popc(m));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (pred) q[base + __popc(m & ((1u << lane) - 1))] = v;
}

__global__ void k_sparse_to_bitmap(const int32_t *__restrict__ q, const int32_t *__restrict__ n_dev,
                                   uint32_t *__restrict__ bm, int32_t *__restrict__ cnt) {
  const int32_t n = *n_dev;
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int32_t v = q[i];
    const uint32_t bit = 1u << (v & 31);
    if (!(atomicOr(bm + (v >> 5), bit) & bit)) agg_inc(cnt);
  }
}

__global__ void k_sparse_to_boolmap(const int32_t *__restrict__ q, const int32_t *__restrict__ n_dev,
                                    uint8_t *__restrict__ by, int32_t *__restrict__ cnt) {
  const int32_t n = *n_dev;
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int32_t v = q[i];
    const uint32_t sh = 8u * (v & 3);
    uint32_t *word = reinterpret_cast<uint32_t *>(by + (v & ~3));
    if (!((atomicOr(word, 1u << sh) >> sh) & 0xffu)) agg_inc(cnt);
  }
}

// Bitmap -> sparse: a warp reads 32 words; each lane expands its word.
__global__ void k_bitmap_to_sparse(const uint32_t *__restrict__ bm, int32_t nwords, int32_t V,
                                   int32_t *__restrict__ q, int32_t *__restrict__ cnt) {
  const int32_t lane = threadIdx.x & 31;
  const int32_t warps = (gridDim.x * blockDim.x) >> 5;
  const int32_t total = ceil_div(nwords, 32) * 32;
  for (int32_t base = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; base < total;
       base += warps * 32) {
    const int32_t wi = base + lane;
    uint32_t word = wi < nwords ? bm[wi] : 0u;
    const int32_t c = __popc(word);
    int32_t ex = c;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int32_t t = __shfl_up_sync(0xffffffffu, ex, d);
      if (lane >= d) ex += t;
    }
    const int32_t tot = __shfl_sync(0xffffffffu, ex, 31);
    int32_t at = 0;
    if (lane == 0 && tot) at = atomicAdd(cnt, tot);
    at = __shfl_sync(0xffffffffu, at, 0) + ex - c;
    while (word) {
      const int32_t b = __ffs(word) - 1;
      word &= word - 1;
      const int32_t v = wi * 32 + b;
      if (v < V) q[at++] = v;
    }
  }
}

// Boolmap -> sparse: each lane reads 4 bytes (one word).
__global__ void k_boolmap_to_sparse(const uint8_t *__restrict__ by, int32_t V,
                                    int32_t *__restrict__ q, int32_t *__restrict__ cnt) {
  const int32_t lane = threadIdx.x & 31;
  const int32_t nwords = ceil_div(V, 4);
  const int32_t warps = (gridDim.x * blockDim.x) >> 5;
  const int32_t total = ceil_div(nwords, 32) * 32;
  const uint32_t *w4 = reinterpret_cast<const uint32_t *>(by);
  for (int32_t base = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; base < total;
       base += warps * 32) {
    const int32_t wi = base + lane;
    const uint32_t word = wi < nwords ? w4[wi] : 0u;
    int32_t c = 0;
#pragma unroll
    for (int b = 0; b < 4; ++b) c += ((word >> (8 * b)) & 0xffu) != 0 && wi * 4 + b < V;
    int32_t ex = c;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int32_t t = __shfl_up_sync(0xffffffffu, ex, d);
      if (lane >= d) ex += t;
    }
    const int32_t tot = __shfl_sync(0xffffffffu, ex, 31);
    int32_t at = 0;
    if (lane == 0 && tot) at = atomicAdd(cnt, tot);
    at = __shfl_sync(0xffffffffu, at, 0) + ex - c;
#pragma unroll
    for (int b = 0; b < 4; ++b)
      if (((word >> (8 * b)) & 0xffu) != 0 && wi * 4 + b < V) q[at++] = wi * 4 + b;
  }
}

// Bitmap <-> boolmap, one bitmap word per thread; counts set members.
__global__ void k_bitmap_to_boolmap(const uint32_t *__restrict__ bm, int32_t nwords, int32_t V,
                                    uint8_t *__restrict__ by, int32_t *__restrict__ cnt) {
  for (int32_t wi = blockIdx.x * blockDim.x + threadIdx.x; wi < nwords; wi += gridDim.x * blockDim.x) {
    const uint32_t word = bm[wi];
    uint32_t *dst = reinterpret_cast<uint32_t *>(by + wi * 32);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      uint32_t o = 0;
#pragma unroll
      for (int b = 0; b < 4; ++b) o |= ((word >> (4 * k + b)) & 1u) << (8 * b);
      if (wi * 32 + 4 * k < V) dst[k] = o;
    }
    if (word) atomicAdd(cnt, __popc(word));
  }
}

__global__ void k_boolmap_to_bitmap(const uint8_t *__restrict__ by, int32_t nwords, int32_t V,
                                    uint32_t *__restrict__ bm, int32_t *__restrict__ cnt) {
  for (int32_t wi = blockIdx.x * blockDim.x + threadIdx.x; wi < nwords; wi += gridDim.x * blockDim.x) {
    const uint32_t *src = reinterpret_cast<const uint32_t *>(by + wi * 32);
    uint32_t word = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (wi * 32 + 4 * k >= V) break;
      const uint32_t x = src[k];
#pragma unroll
      for (int b = 0; b < 4; ++b) word |= (((x >> (8 * b)) & 0xffu) != 0) << (4 * k + b);
    }
    bm[wi] = word;
    if (word) atomicAdd(cnt, __popc(word));
  }
}

// dedup_frontier_device_perfect (vertex_frontier.h:371-378).
__global__ void k_dedup(const int32_t *__restrict__ q, const int32_t *__restrict__ n_dev,
                        int32_t *__restrict__ dedup, int32_t epoch, int32_t *__restrict__ qo,
                        int32_t *__restrict__ cnt) {
  const int32_t n = *n_dev;
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int32_t v = q[i];
    if (write_max(dedup + v, epoch)) qo[agg_inc(cnt)] = v;
  }
}

// ------------------------------------------------------------ vertex UDFs
__device__ __forceinline__ void vertex_udf(int32_t op, int32_t v, const VData &d,
                                           const int32_t *__restrict__ off, float beta,
                                           float inv_v) {
  switch (op) {
    case GG_VUDF_BFS_RESET:  // bfs.cpp:31-33, then parent[src] = src
      d.parent[v] = v == d.src ? v : -1;
      if (d.depth) d.depth[v] = v == d.src ? 0 : -1;
      break;
    case GG_VUDF_SSSP_RESET:  // sssp.cpp:29-31, then SP[src] = 0
      d.dist[v] = v == d.src ? 0 : INT_MAX;
      break;
    case GG_VUDF_PR_RESET:  // pr.cpp:43-46
      d.old_rank[v] = inv_v;
      d.new_rank[v] = 0.0f;
      break;
    case GG_VUDF_PR_CONTRIB:  // pr.cpp:28-30 (a sink divides by 0, as in the reference)
      d.contrib[v] = d.old_rank[v] / (float)(off[v + 1] - off[v]);
      break;
    case GG_VUDF_PR_UPDATE: {  // pr.cpp:36-41
      const float nr = beta + d.damping * d.new_rank[v];
      d.old_rank[v] = nr;
      d.new_rank[v] = 0.0f;
      break;
    }
    case GG_VUDF_CC_INIT:  // cc.cpp:37-39
      d.ids[v] = v;
      break;
    case GG_VUDF_CC_PJUMP: {  // cc.cpp:41-49
      const int32_t y = *(volatile int32_t *)(d.ids + v);
      const int32_t x = *(volatile int32_t *)(d.ids + y);
      if (x != y) {
        d.ids[v] = x;
        if (*(volatile int32_t *)(d.updates + 1) == 0) d.updates[1] = 1;
      }
      break;
    }
    case GG_VUDF_BC_RESET:  // bc.cpp:28-32, then num_paths[src] = 1, visited[src] = 1
      if (d.dep64)
        d.dep64[v] = 0.0;
      else
        d.dependences[v] = 0.0f;
      d.num_paths[v] = v == d.src ? 1.0 : 0.0;
      d.visited[v] = v == d.src;
      break;
    case GG_VUDF_BC_MARK_VISITED:  // bc.cpp:42-44
      d.visited[v] = 1;
      break;
    case GG_VUDF_BC_MARK_UNVISITED:  // bc.cpp:45-47
      d.visited[v] = 0;
      break;
    case GG_VUDF_BC_BACKWARD_VERTEX:  // bc.cpp:48-51
      d.visited[v] = 1;
      if (d.dep64)
        d.dep64[v] += 1.0 / d.num_paths[v];
      else
        d.dependences[v] = (float)(d.dependences[v] + 1.0 / d.num_paths[v]);
      break;
    case GG_VUDF_BC_FINAL: {  // bc.cpp:56-61
      const double np = d.num_paths[v];
      const double dv = d.dep64 ? d.dep64[v] : (double)d.dependences[v];
      d.dependences[v] = np != 0 ? (float)((dv - 1.0 / np) * np) : 0.0f;
      break;
    }
    default:
      break;
  }
}

__global__ void k_vertexset(int32_t op, VData d, const int32_t *__restrict__ q,
                            const int32_t *__restrict__ n_dev, int32_t n_all,
                            const int32_t *__restrict__ off, float beta, float inv_v) {
  const int32_t n = q ? *n_dev : n_all;
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    vertex_udf(op, q ? q[i] : i, d, off, beta, inv_v);
}

// create_reverse_frontier: every v passing the to() filter, compacted by warps.
__global__ void k_reverse(int32_t filter, VData d, int32_t V, int32_t *__restrict__ q,
                          int32_t *__restrict__ cnt) {
  const int32_t stride = gridDim.x * blockDim.x;
  const int32_t total = ceil_div(V, 32) * 32;
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < ceil_div(total, stride) * stride;
       v += stride) {
    bool p = false;
    if (v < V) {
      if (filter == GG_FILTER_PARENT_UNSET)
        p = d.parent[v] == -1;
      else if (filter == GG_FILTER_UNVISITED)
        p = d.visited[v] == 0;
      else
        p = true;
    }
    warp_append(p, v, q, cnt);
  }
}

// TWC binning pass: small (< 32 edges) -> thread, mid (< cta) -> warp,
// large -> CTA (the twc_*_bin scratch of graph.h:48-54).
__global__ void k_twc_bin(DGraph g, Enum en, int32_t cta, int32_t *__restrict__ bins, int64_t cap,
                          int32_t *__restrict__ bin_cnt) {
  const int32_t n = en.count();
  const int32_t stride = gridDim.x * blockDim.x;
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < ceil_div(n, stride) * stride; i += stride) {
    int32_t s = -1, deg = 0;
    if (i < n) {
      s = en.at(i);
      deg = g.off[s + 1] - g.off[s];
    }
    const bool live = i < n && deg > 0;
    warp_append(live && deg < 32, s, bins, bin_cnt + 0);
    warp_append(live && deg >= 32 && deg < cta, s, bins + cap, bin_cnt + 1);
    warp_append(live && deg >= cta, s, bins + 2 * cap, bin_cnt + 2);
  }
}

struct DegIn {
  DGraph g;
  Enum en;
  __device__ int32_t operator()(int64_t i) const {
    const int32_t s = en.at((int32_t)i);
    return g.off[s + 1] - g.off[s];
  }
};

// ------------------------------------------------------------- host helpers
static gg_status frontier_alloc(gg_frontier *f) {
  cudaStream_t st = f->g->stream;
  const int32_t V = f->V;
  f->cap = (int64_t)kFrontierMultiplier * V;
  f->nwords = ceil_div(V, 32);
  f->bytes_padded = f->nwords * 32;  // boolmap padded to whole bitmap words
  GG_CUDA(dev_alloc(&f->q_in, sizeof(int32_t) * f->cap, st));
  GG_CUDA(dev_alloc(&f->q_out, sizeof(int32_t) * f->cap, st));
  GG_CUDA(dev_alloc(&f->cnt, sizeof(int32_t) * 2, st));
  GG_CUDA(dev_alloc(&f->bm_in, sizeof(uint32_t) * f->nwords, st));
  GG_CUDA(dev_alloc(&f->bm_out, sizeof(uint32_t) * f->nwords, st));
  GG_CUDA(dev_alloc(&f->by_in, f->bytes_padded, st));
  GG_CUDA(dev_alloc(&f->by_out, f->bytes_padded, st));
  GG_CUDA(dev_alloc(&f->dedup, sizeof(int32_t) * V, st));
  f->cnt_in = f->cnt;
  f->cnt_out = f->cnt + 1;
  GG_CUDA(cudaMemsetAsync(f->cnt, 0, sizeof(int32_t) * 2, st));
  GG_CUDA(cudaMemsetAsync(f->bm_in, 0, sizeof(uint32_t) * f->nwords, st));
  GG_CUDA(cudaMemsetAsync(f->bm_out, 0, sizeof(uint32_t) * f->nwords, st));
  GG_CUDA(cudaMemsetAsync(f->by_in, 0, f->bytes_padded, st));
  GG_CUDA(cudaMemsetAsync(f->by_out, 0, f->bytes_padded, st));
  GG_CUDA(cudaMemsetAsync(f->dedup, 0, sizeof(int32_t) * V, st));
  f->epoch = 0;
  f->fmt = GG_FMT_SPARSE;
  return GG_OK;
}

gg_status frontier_size(gg_frontier *f, int32_t *n) {
  gg_graph *g = f->g;
  GG_CUDA(cudaMemcpyAsync(g->h_pinned, f->cnt_in, sizeof(int32_t), cudaMemcpyDeviceToHost, g->stream));
  GG_CUDA(cudaStreamSynchronize(g->stream));
  *n = g->h_pinned[0];
  if (*n > f->cap) {
    // enqueues past the capacity were dropped (and flagged); a count this
    // large must never bound a loop over the queue
    *n = 0;
    GG_TRY(check_device_error(g, "frontier"));
    return set_error(GG_ERR_OVERFLOW, "frontier queue capacity exceeded");
  }
  return GG_OK;
}

static void swap_counts(gg_frontier *f) { std::swap(f->cnt_in, f->cnt_out); }

// The new representation is built in the output buffers and swapped in, as
// vertex_representation.h does (generalized_prepare_from_to + swap_*).
gg_status frontier_prepare_sparse(gg_frontier *f) {
  if (f->fmt == GG_FMT_SPARSE) return GG_OK;
  gg_graph *g = f->g;
  cudaStream_t st = g->stream;
  GG_CUDA(cudaMemsetAsync(f->cnt_out, 0, sizeof(int32_t), st));
  if (f->fmt == GG_FMT_BITMAP)
    { gg::note_launch(); k_bitmap_to_sparse<<<grid_of(g), kThreads, 0, st>>>(f->bm_in, f->nwords, f->V, f->q_out, f->cnt_out); }
  else
    { gg::note_launch(); k_boolmap_to_sparse<<<grid_of(g), kThreads, 0, st>>>(f->by_in, f->V, f->q_out, f->cnt_out); }
  GG_CUDA(cudaGetLastError());
  std::swap(f->q_in, f->q_out);
  swap_counts(f);
  f->fmt = GG_FMT_SPARSE;
  return GG_OK;
}

gg_status frontier_prepare_bitmap(gg_frontier *f) {
  if (f->fmt == GG_FMT_BITMAP) return GG_OK;
  gg_graph *g = f->g;
  cudaStream_t st = g->stream;
  GG_CUDA(cudaMemsetAsync(f->cnt_out, 0, sizeof(int32_t), st));
  if (f->fmt == GG_FMT_SPARSE) {
    GG_CUDA(cudaMemsetAsync(f->bm_out, 0, sizeof(uint32_t) * f->nwords, st));
    { gg::note_launch(); k_sparse_to_bitmap<<<grid_of(g), kThreads, 0, st>>>(f->q_in, f->cnt_in, f->bm_out, f->cnt_out); }
  } else {
    { gg::note_launch(); k_boolmap_to_bitmap<<<grid_of(g), kThreads, 0, st>>>(f->by_in, f->nwords, f->V, f->bm_out, f->cnt_out); }
  }
  GG_CUDA(cudaGetLastError());
  std::swap(f->bm_in, f->bm_out);
  swap_counts(f);
  f->fmt = GG_FMT_BITMAP;
  return GG_OK;
}

gg_status frontier_prepare_boolmap(gg_frontier *f) {
  if (f->fmt == GG_FMT_BOOLMAP) return GG_OK;
  gg_graph *g = f->g;
  cudaStream_t st = g->stream;
  GG_CUDA(cudaMemsetAsync(f->cnt_out, 0, sizeof(int32_t), st));
  if (f->fmt == GG_FMT_SPARSE) {
    GG_CUDA(cudaMemsetAsync(f->by_out, 0, f->bytes_padded, st));
    { gg::note_launch(); k_sparse_to_boolmap<<<grid_of(g), kThreads, 0, st>>>(f->q_in, f->cnt_in, f->by_out, f->cnt_out); }
  } else {
    { gg::note_launch(); k_bitmap_to_boolmap<<<grid_of(g), kThreads, 0, st>>>(f->bm_in, f->nwords, f->V, f->by_out, f->cnt_out); }
  }
  GG_CUDA(cudaGetLastError());
  std::swap(f->by_in, f->by_out);
  swap_counts(f);
  f->fmt = GG_FMT_BOOLMAP;
  return GG_OK;
}

DIn frontier_in_view(const gg_frontier *f) {
  DIn d{IN_ALL, nullptr, nullptr};
  if (f->fmt == GG_FMT_BITMAP) {
    d.mode = IN_BITMAP;
    d.bm = f->bm_in;
  } else if (f->fmt == GG_FMT_BOOLMAP) {
    d.mode = IN_BOOLMAP;
    d.by = f->by_in;
  }
  return d;
}

// Clears the output side for `creation` and returns the writer.  The reference
// clears at swap time (vertex_frontier.h:217-316); clearing before the launch
// is equivalent.
DOut frontier_out_view(gg_frontier *f, int32_t creation, bool dedup) {
  cudaStream_t st = f->g->stream;
  DOut o{};
  o.cnt = f->cnt_out;
  o.err = f->g->d_err;
  cudaMemsetAsync(f->cnt_out, 0, sizeof(int32_t), st);
  if (creation == GG_FC_BITMAP) {
    o.mode = OUT_BITMAP;
    o.bm = f->bm_out;
    cudaMemsetAsync(f->bm_out, 0, sizeof(uint32_t) * f->nwords, st);
  } else if (creation == GG_FC_BOOLMAP) {
    o.mode = OUT_BOOLMAP;
    o.by = f->by_out;
    cudaMemsetAsync(f->by_out, 0, f->bytes_padded, st);
  } else {
    o.mode = dedup ? OUT_SPARSE_DEDUP : OUT_SPARSE;
    o.q = f->q_out;
    o.cap = f->cap;
    o.dedup = f->dedup;
    o.epoch = f->epoch;
  }
  return o;
}

gg_status frontier_swap(gg_frontier *f, int32_t creation) {
  if (creation == GG_FC_BITMAP) {
    std::swap(f->bm_in, f->bm_out);
    f->fmt = GG_FMT_BITMAP;
  } else if (creation == GG_FC_BOOLMAP) {
    std::swap(f->by_in, f->by_out);
    f->fmt = GG_FMT_BOOLMAP;
  } else {
    std::swap(f->q_in, f->q_out);
    f->fmt = GG_FMT_SPARSE;
  }
  swap_counts(f);
  return GG_OK;
}

gg_status frontier_dedup(gg_frontier *f) {
  GG_TRY(frontier_prepare_sparse(f));
  gg_graph *g = f->g;
  cudaStream_t st = g->stream;
  f->epoch++;
  GG_CUDA(cudaMemsetAsync(f->cnt_out, 0, sizeof(int32_t), st));
  { gg::note_launch(); k_dedup<<<grid_of(g), kThreads, 0, st>>>(f->q_in, f->cnt_in, f->dedup, f->epoch, f->q_out, f->cnt_out); }
  GG_CUDA(cudaGetLastError());
  std::swap(f->q_in, f->q_out);
  swap_counts(f);
  return GG_OK;
}

gg_status reverse_frontier(gg_graph *g, int32_t filter, const VData &vd, int32_t **q, int32_t **cnt) {
  const int32_t V = g->csr.V;
  void *p = nullptr;
  GG_TRY(scratch_get(g, 0, sizeof(int32_t) * ((size_t)V + 32), &p));
  *q = (int32_t *)p;
  *cnt = *q + V + 16;
  GG_CUDA(cudaMemsetAsync(*cnt, 0, sizeof(int32_t), g->stream));
  { gg::note_launch(); k_reverse<<<grid_of(g), kThreads, 0, g->stream>>>(filter, vd, V, *q, *cnt); }
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

gg_status twc_bin(gg_graph *G, const DGraph &g, const Enum &en, int32_t n_host, int32_t cta,
                  int32_t **bins, int32_t **bin_cnt) {
  const int64_t cap = n_host < 0 ? g.V : n_host;
  void *p = nullptr;
  GG_TRY(scratch_get(G, 1, sizeof(int32_t) * (3 * cap + 16), &p));
  *bins = (int32_t *)p;
  *bin_cnt = *bins + 3 * cap + 4;
  GG_CUDA(cudaMemsetAsync(*bin_cnt, 0, sizeof(int32_t) * 3, G->stream));
  { gg::note_launch(); k_twc_bin<<<grid_of(G), kThreads, 0, G->stream>>>(g, en, cta, *bins, cap, *bin_cnt); }
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

gg_status strict_scan(gg_graph *G, const DGraph &g, const Enum &en, int32_t n_host, int32_t **sum) {
  if (n_host < 0) return set_error(GG_ERR_UNSUPPORTED, "STRICT needs a host-known frontier size");
  void *p = nullptr;
  const size_t need = (size_t)n_host + 1 + scan_scratch_ints(n_host) + 8;
  GG_TRY(scratch_get(G, 2, sizeof(int32_t) * need, &p));
  *sum = (int32_t *)p;
  int32_t *partial = *sum + n_host + 4;
  GG_CUDA(exclusive_scan(DegIn{g, en}, n_host, *sum, partial, G->stream));
  return GG_OK;
}

gg_status etwc_scratch(gg_graph *G, int64_t max_chunks, int32_t **chunks, int32_t **cnt) {
  void *p = nullptr;
  GG_TRY(scratch_get(G, 3, sizeof(int32_t) * (3 * max_chunks + 8), &p));
  *chunks = (int32_t *)p;
  *cnt = *chunks + 3 * max_chunks + 4;
  return GG_OK;
}

VData to_vdata(const gg_vertex_data *v) {
  VData d{};
  if (!v) return d;
  d.parent = v->parent;
  d.depth = v->depth;
  d.dist = v->dist;
  d.ids = v->ids;
  d.updates = v->updates;
  d.old_rank = v->old_rank;
  d.new_rank = v->new_rank;
  d.contrib = v->contrib;
  d.num_paths = v->num_paths;
  d.dependences = v->dependences;
  d.visited = v->visited;
  d.level = v->level;
  d.src = v->src;
  d.damping = v->damping;
  return d;
}

gg_status vertexset_apply_impl(gg_graph *g, gg_frontier *set, int32_t vudf, const VData &vd) {
  const int32_t V = g->csr.V;
  const int32_t *q = nullptr, *n_dev = nullptr;
  if (set) {
    GG_TRY(frontier_prepare_sparse(set));  // to_sparse_host, operators.cpp:29
    q = set->q_in;
    n_dev = set->cnt_in;
  }
  const float beta = (float)((1.0 - (double)vd.damping) / V);
  const float inv_v = (float)(1.0 / V);
  { gg::note_launch(); k_vertexset<<<grid_of(g), kThreads, 0, g->stream>>>(vudf, vd, q, n_dev, V, g->csr.off, beta, inv_v); }
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

}  // namespace gg

using namespace gg;

extern "C" {

gg_status gg_frontier_create(gg_graph *g, int32_t init_all, gg_frontier **out) {
  GG_CHECK_ARG(g && out, "bad arguments");
  auto f = new (std::nothrow) gg_frontier();
  if (!f) return set_error(GG_ERR_OOM, "frontier allocation failed");
  f->g = g;
  f->V = g->csr.V;
  gg_status s = frontier_alloc(f);
  if (s != GG_OK) {
    delete f;
    return s;
  }
  if (init_all) {  // create_new_vertex_set(V, V): initialize_frontier_all
    { gg::note_launch(); k_iota<<<grid_of(g), kThreads, 0, g->stream>>>(f->q_in, f->V, f->cnt_in); }
    GG_CUDA(cudaGetLastError());
  }
  GG_CUDA(cudaStreamSynchronize(g->stream));
  *out = f;
  return GG_OK;
}

gg_status gg_frontier_destroy(gg_frontier *f) {
  if (!f) return GG_OK;
  if (f->owned_by_pq)
    return set_error(GG_ERR_STATE, "the frontier belongs to a priority queue; gg_pq_destroy releases it");
  cudaStream_t st = f->g->stream;
  cudaError_t e = cudaSuccess;
  for (void *p : {(void *)f->q_in, (void *)f->q_out, (void *)f->cnt, (void *)f->bm_in,
                  (void *)f->bm_out, (void *)f->by_in, (void *)f->by_out, (void *)f->dedup})
    if (p) {
      const cudaError_t r = cudaFreeAsync(p, st);
      if (e == cudaSuccess) e = r;
    }
  const cudaError_t r = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = r;
  delete f;
  if (e != cudaSuccess) {
    cudaGetLastError();  // reported here, not by the next call's launch check
    return set_error(GG_ERR_CUDA, "releasing the frontier failed: %s", cudaGetErrorString(e));
  }
  return GG_OK;
}

// builtin_addVertex (vertex_frontier.h:168-175), for any representation.
gg_status gg_frontier_add(gg_frontier *f, int32_t v) {
  GG_CHECK_ARG(f, "frontier is NULL");
  GG_CHECK_ARG(v >= 0 && v < f->V, "vertex out of range");
  gg_graph *g = f->g;
  cudaStream_t st = g->stream;
  int32_t n = 0;
  GG_TRY(frontier_size(f, &n));
  if (f->fmt == GG_FMT_SPARSE) {
    if (n >= f->cap) return set_error(GG_ERR_OVERFLOW, "frontier queue full");
    g->h_pinned[1] = v;
    g->h_pinned[2] = n + 1;
    GG_CUDA(cudaMemcpyAsync(f->q_in + n, g->h_pinned + 1, sizeof(int32_t), cudaMemcpyHostToDevice, st));
    GG_CUDA(cudaMemcpyAsync(f->cnt_in, g->h_pinned + 2, sizeof(int32_t), cudaMemcpyHostToDevice, st));
  } else {
    // Reuse the sparse conversion kernels on a 1-entry queue.
    g->h_pinned[1] = v;
    g->h_pinned[2] = 1;
    int32_t *one = g->d_misc + 8;
    GG_CUDA(cudaMemcpyAsync(one, g->h_pinned + 1, sizeof(int32_t) * 2, cudaMemcpyHostToDevice, st));
    if (f->fmt == GG_FMT_BITMAP)
      { gg::note_launch(); k_sparse_to_bitmap<<<1, 32, 0, st>>>(one, one + 1, f->bm_in, f->cnt_in); }
    else
      { gg::note_launch(); k_sparse_to_boolmap<<<1, 32, 0, st>>>(one, one + 1, f->by_in, f->cnt_in); }
    GG_CUDA(cudaGetLastError());
  }
  GG_CUDA(cudaStreamSynchronize(st));
  return GG_OK;
}

gg_status gg_frontier_size(gg_frontier *f, int32_t *n) {
  GG_CHECK_ARG(f && n, "bad arguments");
  return frontier_size(f, n);
}

gg_status gg_frontier_clear(gg_frontier *f) {
  GG_CHECK_ARG(f, "frontier is NULL");
  cudaStream_t st = f->g->stream;
  GG_CUDA(cudaMemsetAsync(f->cnt, 0, sizeof(int32_t) * 2, st));
  GG_CUDA(cudaMemsetAsync(f->bm_in, 0, sizeof(uint32_t) * f->nwords, st));
  GG_CUDA(cudaMemsetAsync(f->by_in, 0, f->bytes_padded, st));
  f->fmt = GG_FMT_SPARSE;
  GG_CUDA(cudaStreamSynchronize(st));
  return GG_OK;
}

gg_status gg_frontier_format(const gg_frontier *f, int32_t *fmt) {
  GG_CHECK_ARG(f && fmt, "bad arguments");
  *fmt = f->fmt;
  return GG_OK;
}

gg_status gg_frontier_to_sparse(gg_frontier *f) {
  GG_CHECK_ARG(f, "frontier is NULL");
  GG_TRY(frontier_prepare_sparse(f));
  GG_CUDA(cudaStreamSynchronize(f->g->stream));
  return GG_OK;
}
gg_status gg_frontier_to_bitmap(gg_frontier *f) {
  GG_CHECK_ARG(f, "frontier is NULL");
  GG_TRY(frontier_prepare_bitmap(f));
  GG_CUDA(cudaStreamSynchronize(f->g->stream));
  return GG_OK;
}
gg_status gg_frontier_to_boolmap(gg_frontier *f) {
  GG_CHECK_ARG(f, "frontier is NULL");
  GG_TRY(frontier_prepare_boolmap(f));
  GG_CUDA(cudaStreamSynchronize(f->g->stream));
  return GG_OK;
}

gg_status gg_frontier_dedup(gg_frontier *f) {
  GG_CHECK_ARG(f, "frontier is NULL");
  GG_TRY(frontier_dedup(f));
  GG_CUDA(cudaStreamSynchronize(f->g->stream));
  return GG_OK;
}

gg_status gg_frontier_read(gg_frontier *f, int32_t *out, int32_t cap, int32_t *n) {
  GG_CHECK_ARG(f && n, "bad arguments");
  GG_TRY(frontier_prepare_sparse(f));
  int32_t cnt = 0;
  GG_TRY(frontier_size(f, &cnt));
  *n = cnt;
  if (!out) return GG_OK;
  if (cnt > cap) return set_error(GG_ERR_INVALID, "output capacity %d < frontier size %d", cap, cnt);
  std::vector<int32_t> h(cnt);
  GG_CUDA(cudaMemcpyAsync(h.data(), f->q_in, sizeof(int32_t) * cnt, cudaMemcpyDeviceToHost, f->g->stream));
  GG_CUDA(cudaStreamSynchronize(f->g->stream));
  std::sort(h.begin(), h.end());
  GG_CUDA(cudaMemcpy(out, h.data(), sizeof(int32_t) * cnt, cudaMemcpyDefault));
  return GG_OK;
}

gg_status gg_vertexset_apply(gg_graph *g, gg_frontier *set, int32_t vudf, const gg_vertex_data *vd) {
  GG_CHECK_ARG(g && vd, "bad arguments");
  GG_CHECK_ARG(vudf >= GG_VUDF_BFS_RESET && vudf <= GG_VUDF_BC_FINAL, "unknown vertex UDF");
  GG_TRY(vertexset_apply_impl(g, set, vudf, to_vdata(vd)));
  GG_CUDA(cudaStreamSynchronize(g->stream));
  return GG_OK;
}

// ---------------------------------------------------------- frontier list
gg_status gg_frontier_list_create(gg_graph *g, gg_frontier_list **out) {
  GG_CHECK_ARG(g && out, "bad arguments");
  auto l = new gg_frontier_list();
  l->g = g;
  if (dev_alloc(&l->vertices, sizeof(int32_t) * (size_t)g->csr.V, g->stream) != cudaSuccess) {
    delete l;
    return set_error(GG_ERR_OOM, "frontier list allocation failed");
  }
  *out = l;
  return GG_OK;
}

gg_status gg_frontier_list_destroy(gg_frontier_list *l) {
  if (!l) return GG_OK;
  if (l->vertices) cudaFreeAsync(l->vertices, l->g->stream);
  cudaStreamSynchronize(l->g->stream);
  delete l;
  return GG_OK;
}

// builtin_insert (list.h:61-76): append the frontier as a new level.
gg_status gg_frontier_list_insert(gg_frontier_list *l, gg_frontier *f) {
  GG_CHECK_ARG(l && f, "bad arguments");
  GG_TRY(frontier_prepare_sparse(f));
  int32_t n = 0;
  GG_TRY(frontier_size(f, &n));
  const int32_t at = l->level_start.back();
  if ((int64_t)at + n > l->g->csr.V)
    return set_error(GG_ERR_OVERFLOW, "frontier list holds more than V vertices");
  if (n)
    GG_CUDA(cudaMemcpyAsync(l->vertices + at, f->q_in, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice,
                            l->g->stream));
  l->level_start.push_back(at + n);
  return GG_OK;
}

// builtin_retrieve (list.h:92-107): pop the last level into the frontier.
gg_status gg_frontier_list_retrieve(gg_frontier_list *l, gg_frontier *f) {
  GG_CHECK_ARG(l && f, "bad arguments");
  if (l->level_start.size() < 2)
    return set_error(GG_ERR_STATE, "Too deep into vertex frontier list");
  const int32_t end = l->level_start.back();
  l->level_start.pop_back();
  const int32_t at = l->level_start.back();
  const int32_t n = end - at;
  cudaStream_t st = l->g->stream;
  if (n)
    GG_CUDA(cudaMemcpyAsync(f->q_in, l->vertices + at, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, st));
  l->g->h_pinned[3] = n;
  GG_CUDA(cudaMemcpyAsync(f->cnt_in, l->g->h_pinned + 3, sizeof(int32_t), cudaMemcpyHostToDevice, st));
  GG_CUDA(cudaStreamSynchronize(st));
  f->fmt = GG_FMT_SPARSE;
  return GG_OK;
}

}  // extern "C"
