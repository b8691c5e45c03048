// PageRank pull iteration for PULL + TWC schedules: the in-degree bins of the
// transposed graph are built once per call (thread / warp / tiles of a CTA per
// vertex, the TWC binning of graph.h:48-54 applied to the pull gather), and
// every iteration is one gather per bin that fuses pr.cpp's three steps
//   contrib[u] = old[u] / outdeg[u];   new[v] = sum contrib[u];
//   old[v] = (1-d)/V + d * new[v]
// (apps/pr.cpp:28-41).  Each vertex's sum is formed in a fixed order -- by its
// owner, or for hubs from per-tile partial sums added in tile order -- so there
// are no atomics and results are bit-identical across runs.  The next
// iteration's contributions go to the other half of a double buffer.
//
// The gathers are latency-bound (contrib is L2-resident, its reads random), so
// every lane keeps four independent contrib loads in flight, and the iteration
// runs on the degree-ordered copy of the graph (relabel.cu): the contributions
// of the high-degree vertices, read by most in-edges, share cache lines.  Ranks
// come back to the caller's ids at the end.
#include <algorithm>
#include <vector>

#include "engine.h"

namespace gg {

constexpr int32_t kPrSmallMax = 32;   // in-degree < 32: one thread
constexpr int32_t kPrMidMax = 4096;   // < 4096: one warp; else tiles of kPrTile edges
constexpr int32_t kPrTile = 8192;     // in-edges per CTA tile of a hub

struct PrArgs {
  const int32_t *toff, *tsrc;   // CSC
  const int32_t *off;           // forward CSR (out-degrees)
  const float *contrib;         // this iteration
  float *contrib_next;          // next iteration
  float *rank;                  // old_rank
  float beta, damp;
};

__device__ __forceinline__ void pr_finish(const PrArgs &a, int32_t v, float s) {
  const float r = a.beta + a.damp * s;
  a.rank[v] = r;
  a.contrib_next[v] = r / (float)(a.off[v + 1] - a.off[v]);  // a sink divides by 0, as pr.cpp
}

// Sum of contrib over in-edges k = k0, k0 + step, ... < k1, four loads in flight.
__device__ __forceinline__ float pr_gather(const PrArgs &a, int32_t k0, int32_t k1, int32_t step) {
  float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
  int32_t k = k0;
  for (; k + 3 * step < k1; k += 4 * step) {
    const int32_t u0 = __ldg(a.tsrc + k), u1 = __ldg(a.tsrc + k + step);
    const int32_t u2 = __ldg(a.tsrc + k + 2 * step), u3 = __ldg(a.tsrc + k + 3 * step);
    s0 += __ldg(a.contrib + u0);
    s1 += __ldg(a.contrib + u1);
    s2 += __ldg(a.contrib + u2);
    s3 += __ldg(a.contrib + u3);
  }
  for (; k < k1; k += step) s0 += __ldg(a.contrib + __ldg(a.tsrc + k));
  return (s0 + s1) + (s2 + s3);
}

__global__ void k_pr_small(PrArgs a, const int32_t *__restrict__ bin, int32_t n) {
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int32_t v = bin[i];
    pr_finish(a, v, pr_gather(a, __ldg(a.toff + v), __ldg(a.toff + v + 1), 1));
  }
}

__global__ void k_pr_mid(PrArgs a, const int32_t *__restrict__ bin, int32_t n) {
  const int32_t lane = threadIdx.x & 31;
  const int32_t w0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  for (int32_t i = w0; i < n; i += nw) {
    const int32_t v = bin[i];
    float s = pr_gather(a, __ldg(a.toff + v) + lane, __ldg(a.toff + v + 1), 32);
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) s += __shfl_xor_sync(0xffffffffu, s, d);
    if (lane == 0) pr_finish(a, v, s);
  }
}

// One CTA per hub tile: partial[t] = sum over the tile's in-edges.
__global__ void __launch_bounds__(512) k_pr_tile(PrArgs a, const int32_t *__restrict__ tile_v,
                                                 const int32_t *__restrict__ tile_k, int32_t ntiles,
                                                 float *__restrict__ partial) {
  __shared__ float part[32];
  for (int32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int32_t v = tile_v[t];
    const int32_t kb = tile_k[t], ke = min(kb + kPrTile, __ldg(a.toff + v + 1));
    float s = pr_gather(a, kb + (int32_t)threadIdx.x, ke, (int32_t)blockDim.x);
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) s += __shfl_xor_sync(0xffffffffu, s, d);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
      s = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0.f;
#pragma unroll
      for (int d = 16; d > 0; d >>= 1) s += __shfl_xor_sync(0xffffffffu, s, d);
      if (threadIdx.x == 0) partial[t] = s;
    }
    __syncthreads();
  }
}

// Hub i owns tiles [first[i], first[i+1]): their partial sums in tile order.
__global__ void k_pr_hub_finish(PrArgs a, const int32_t *__restrict__ hubs, const int32_t *__restrict__ first,
                                int32_t nhubs, const float *__restrict__ partial) {
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nhubs; i += gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int32_t t = first[i]; t < first[i + 1]; ++t) s += partial[t];
    pr_finish(a, hubs[i], s);
  }
}

__global__ void k_pr_bin(const int32_t *__restrict__ toff, int32_t V, int32_t *__restrict__ bins, int32_t *cnt) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t end = (V + stride - 1) / stride * stride;  // whole warps iterate together
  for (int64_t v = blockIdx.x * blockDim.x + threadIdx.x; v < end; v += stride) {
    int32_t d = -1;
    if (v < V) d = toff[v + 1] - toff[v];
    const int which = d < 0 ? -1 : (d < kPrSmallMax ? 0 : (d < kPrMidMax ? 1 : 2));
    for (int b = 0; b < 3; ++b) {
      const bool p = which == b;
      const uint32_t m = __ballot_sync(0xffffffffu, p);
      if (!m) continue;
      const int32_t lane = threadIdx.x & 31;
      int32_t base = 0;
      if (lane == 0) base = atomicAdd(cnt + b, __popc(m));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (p) bins[(int64_t)b * V + base + __popc(m & ((1u << lane) - 1))] = (int32_t)v;
    }
  }
}

__global__ void k_pr_unperm(const float *__restrict__ rank_new, const int32_t *__restrict__ perm, int32_t V,
                            float *__restrict__ rank) {
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
    rank[v] = rank_new[perm[v]];
}

__global__ void k_pr_init(const int32_t *__restrict__ off, int32_t V, float inv_v, float *rank, float *contrib) {
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    rank[v] = inv_v;  // pr.cpp:43-46
    contrib[v] = inv_v / (float)(off[v + 1] - off[v]);
  }
}

__global__ void k_pr_hub_bounds(const int32_t *__restrict__ toff, const int32_t *__restrict__ hubs, int32_t nh,
                                int32_t *__restrict__ bounds) {
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nh; i += gridDim.x * blockDim.x) {
    bounds[2 * i] = toff[hubs[i]];
    bounds[2 * i + 1] = toff[hubs[i] + 1];
  }
}

// In-degree bins of the transposed graph (in the TWC-bin scratch slot: no
// load-balancing strategy runs during the PageRank loop) and the tiles of the
// hub bin: tile t covers in-edges [tile_k[t], tile_k[t] + kPrTile) of tile_v[t].
struct PrPlan {
  int32_t *bins = nullptr;
  int32_t cnt[3] = {0, 0, 0};
  int32_t *hubs = nullptr, *first = nullptr, *tile_v = nullptr, *tile_k = nullptr;
  float *partial = nullptr;
  int32_t ntiles = 0;
};

static gg_status pr_plan(gg_graph *g, const GraphStore &t, PrPlan *P) {
  const int32_t V = g->csr.V;
  void *p = nullptr;
  GG_TRY(scratch_get(g, 1, sizeof(int32_t) * (3 * (size_t)V + 16), &p));
  P->bins = (int32_t *)p;
  int32_t *cnt = P->bins + 3 * (size_t)V + 4;
  GG_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * 3, g->stream));
  note_launch();
  k_pr_bin<<<g->sm_count * 8, 256, 0, g->stream>>>(t.off, V, P->bins, cnt);
  GG_CUDA(cudaGetLastError());
  GG_CUDA(cudaMemcpyAsync(P->cnt, cnt, sizeof(int32_t) * 3, cudaMemcpyDeviceToHost, g->stream));
  GG_CUDA(cudaStreamSynchronize(g->stream));
  const int32_t nh = P->cnt[2];
  if (nh == 0) return GG_OK;
  // hubs are few: their tile list is laid out on the host, in vertex order
  std::vector<int32_t> hubs(nh), lo(nh), hi(nh);
  GG_CUDA(cudaMemcpy(hubs.data(), P->bins + 2 * (size_t)V, sizeof(int32_t) * nh, cudaMemcpyDeviceToHost));
  std::sort(hubs.begin(), hubs.end());
  {  // in-list bounds of the hubs, gathered on the device
    GG_TRY(scratch_get(g, 3, sizeof(int32_t) * 3 * (size_t)nh, &p));
    int32_t *hd = (int32_t *)p, *bounds = hd + nh;
    GG_CUDA(cudaMemcpyAsync(hd, hubs.data(), sizeof(int32_t) * nh, cudaMemcpyHostToDevice, g->stream));
    note_launch();
    k_pr_hub_bounds<<<std::max(1, std::min(ceil_div(nh, 256), g->sm_count)), 256, 0, g->stream>>>(t.off, hd, nh,
                                                                                                   bounds);
    GG_CUDA(cudaGetLastError());
    std::vector<int32_t> b2(2 * (size_t)nh);
    GG_CUDA(cudaMemcpyAsync(b2.data(), bounds, sizeof(int32_t) * b2.size(), cudaMemcpyDeviceToHost, g->stream));
    GG_CUDA(cudaStreamSynchronize(g->stream));
    for (int32_t i = 0; i < nh; ++i) {
      lo[i] = b2[2 * (size_t)i];
      hi[i] = b2[2 * (size_t)i + 1];
    }
  }
  std::vector<int32_t> tv, tk, first(nh + 1, 0);
  for (int32_t i = 0; i < nh; ++i) {
    first[i] = (int32_t)tv.size();
    for (int32_t k = lo[i]; k < hi[i]; k += kPrTile) {
      tv.push_back(hubs[i]);
      tk.push_back(k);
    }
  }
  first[nh] = (int32_t)tv.size();
  P->ntiles = (int32_t)tv.size();
  // layout: hubs[nh] first[nh+1] tile_v[ntiles] tile_k[ntiles] partial[ntiles]
  const size_t words = (size_t)nh + first.size() + 3 * tv.size();
  GG_TRY(scratch_get(g, 2, sizeof(int32_t) * words, &p));
  P->hubs = (int32_t *)p;
  P->first = P->hubs + nh;
  P->tile_v = P->first + first.size();
  P->tile_k = P->tile_v + tv.size();
  P->partial = reinterpret_cast<float *>(P->tile_k + tv.size());
  GG_CUDA(cudaMemcpyAsync(P->hubs, hubs.data(), sizeof(int32_t) * nh, cudaMemcpyHostToDevice, g->stream));
  GG_CUDA(cudaMemcpyAsync(P->first, first.data(), sizeof(int32_t) * first.size(), cudaMemcpyHostToDevice,
                          g->stream));
  GG_CUDA(cudaMemcpyAsync(P->tile_v, tv.data(), sizeof(int32_t) * tv.size(), cudaMemcpyHostToDevice, g->stream));
  GG_CUDA(cudaMemcpyAsync(P->tile_k, tk.data(), sizeof(int32_t) * tk.size(), cudaMemcpyHostToDevice, g->stream));
  GG_CUDA(cudaStreamSynchronize(g->stream));  // the host vectors go out of scope
  return GG_OK;
}

gg_status pagerank_pull_twc(gg_graph *g, int32_t iters, float damping, float *rank_out, float *contrib2) {
  GG_TRY(ensure_relabel(g));
  GG_TRY(ensure_relabel_csc(g));
  const int32_t V = g->csr.V;
  const GraphStore &t = g->symmetric ? g->rel->g : g->rel->csc;  // in-lists in new ids
  float *rank = nullptr;  // ranks in new ids
  GG_TRY(scratch_get_app(g, 4, sizeof(float) * std::max(V, 1), (void **)&rank));
  PrPlan P;
  GG_TRY(pr_plan(g, t, &P));
  cudaStream_t st = g->stream;
  const float inv_v = (float)(1.0 / V);
  note_launch();
  k_pr_init<<<g->sm_count * 8, 256, 0, st>>>(g->rel->g.off, V, inv_v, rank, contrib2);
  PrArgs a{};
  a.toff = t.off;
  a.tsrc = t.dst;
  a.off = g->rel->g.off;  // out-degrees in new ids
  a.rank = rank;
  a.beta = (float)((1.0 - (double)damping) / V);  // pr.cpp:37
  a.damp = damping;
  const int32_t nh = P.cnt[2];
  for (int32_t it = 0; it < iters; ++it) {
    a.contrib = contrib2 + (size_t)(it & 1) * V;
    a.contrib_next = contrib2 + (size_t)((it + 1) & 1) * V;
    if (P.cnt[0]) {
      note_launch();
      k_pr_small<<<g->sm_count * 8, 256, 0, st>>>(a, P.bins, P.cnt[0]);
    }
    if (P.cnt[1]) {
      note_launch();
      k_pr_mid<<<g->sm_count * 8, 256, 0, st>>>(a, P.bins + V, P.cnt[1]);
    }
    if (nh) {
      note_launch();
      k_pr_tile<<<std::min(P.ntiles, g->sm_count * 4), 512, 0, st>>>(a, P.tile_v, P.tile_k, P.ntiles, P.partial);
      note_launch();
      k_pr_hub_finish<<<std::max(1, std::min(ceil_div(nh, 128), g->sm_count)), 128, 0, st>>>(a, P.hubs, P.first,
                                                                                               nh, P.partial);
    }
  }
  note_launch();
  k_pr_unperm<<<g->sm_count * 8, 256, 0, st>>>(rank, g->rel->perm, V, rank_out);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

}  // namespace gg
