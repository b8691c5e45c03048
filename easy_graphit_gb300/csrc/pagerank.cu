// PageRank pull iteration for PULL + TWC schedules: the in-degree bins of the
// transposed graph are built once per graph (thread / warp / CTA per vertex,
// the TWC binning of graph.h:48-54 applied to the pull gather), and every
// iteration is one gather per bin that fuses pr.cpp's three steps
//   contrib[u] = old[u] / outdeg[u];   new[v] = sum contrib[u];
//   old[v] = (1-d)/V + d * new[v]
// (apps/pr.cpp:28-41).  Each vertex's sum is computed by one owner in a fixed
// order -- no atomics, deterministic results -- and the next iteration's
// contributions are written to the other half of a double buffer.
#include "engine.h"

namespace gg {

constexpr int32_t kPrSmallMax = 32;    // in-degree < 32: one thread
constexpr int32_t kPrMidMax = 4096;    // < 4096: one warp; else one CTA

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

__global__ void k_pr_small(PrArgs a, const int32_t *__restrict__ bin, int32_t n) {
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int32_t v = bin[i];
    float s = 0.f;
    for (int32_t k = a.toff[v]; k < a.toff[v + 1]; ++k) s += __ldg(a.contrib + __ldg(a.tsrc + k));
    pr_finish(a, v, s);
  }
}

__global__ void k_pr_mid(PrArgs a, const int32_t *__restrict__ bin, int32_t n) {
  const int32_t lane = threadIdx.x & 31;
  const int32_t w0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  for (int32_t i = w0; i < n; i += nw) {
    const int32_t v = bin[i];
    float s = 0.f;
    for (int32_t k = a.toff[v] + lane; k < a.toff[v + 1]; k += 32) s += __ldg(a.contrib + __ldg(a.tsrc + k));
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) s += __shfl_xor_sync(0xffffffffu, s, d);
    if (lane == 0) pr_finish(a, v, s);
  }
}

__global__ void __launch_bounds__(512) k_pr_large(PrArgs a, const int32_t *__restrict__ bin, int32_t n) {
  __shared__ float part[32];
  for (int32_t i = blockIdx.x; i < n; i += gridDim.x) {
    const int32_t v = bin[i];
    float s = 0.f;
    for (int32_t k = a.toff[v] + threadIdx.x; k < a.toff[v + 1]; k += blockDim.x)
      s += __ldg(a.contrib + __ldg(a.tsrc + k));
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) s += __shfl_xor_sync(0xffffffffu, s, d);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
      s = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0.f;
#pragma unroll
      for (int d = 16; d > 0; d >>= 1) s += __shfl_xor_sync(0xffffffffu, s, d);
      if (threadIdx.x == 0) pr_finish(a, v, s);
    }
    __syncthreads();
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

__global__ void k_pr_init(const int32_t *__restrict__ off, int32_t V, float inv_v, float *rank, float *contrib) {
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    rank[v] = inv_v;  // pr.cpp:43-46
    contrib[v] = inv_v / (float)(off[v + 1] - off[v]);
  }
}

// In-degree bins of the transposed graph, in the TWC-bin scratch slot (no
// load-balancing strategy runs during the PageRank loop).  One pass over V.
static gg_status pr_bins(gg_graph *g, int32_t **bins, int32_t cnt_host[3]) {
  const int32_t V = g->csr.V;
  const gg::GraphStore &t = g->csc ? *g->csc : g->csr;
  void *p = nullptr;
  GG_TRY(scratch_get(g, 1, sizeof(int32_t) * (3 * (size_t)V + 16), &p));
  *bins = (int32_t *)p;
  int32_t *cnt = *bins + 3 * (size_t)V + 4;
  GG_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * 3, g->stream));
  note_launch();
  k_pr_bin<<<g->sm_count * 8, 256, 0, g->stream>>>(t.off, V, *bins, cnt);
  GG_CUDA(cudaGetLastError());
  GG_CUDA(cudaMemcpyAsync(cnt_host, cnt, sizeof(int32_t) * 3, cudaMemcpyDeviceToHost, g->stream));
  GG_CUDA(cudaStreamSynchronize(g->stream));
  return GG_OK;
}

gg_status pagerank_pull_twc(gg_graph *g, int32_t iters, float damping, float *rank, float *contrib2) {
  GG_TRY(ensure_transpose(g));
  const int32_t V = g->csr.V;
  const gg::GraphStore &t = g->csc ? *g->csc : g->csr;
  int32_t *bins = nullptr;
  int32_t cnt[3];
  GG_TRY(pr_bins(g, &bins, cnt));
  cudaStream_t st = g->stream;
  const float inv_v = (float)(1.0 / V);
  note_launch();
  k_pr_init<<<g->sm_count * 8, 256, 0, st>>>(g->csr.off, V, inv_v, rank, contrib2);
  PrArgs a{};
  a.toff = t.off;
  a.tsrc = t.dst;
  a.off = g->csr.off;
  a.rank = rank;
  a.beta = (float)((1.0 - (double)damping) / V);  // pr.cpp:37
  a.damp = damping;
  for (int32_t it = 0; it < iters; ++it) {
    a.contrib = contrib2 + (size_t)(it & 1) * V;
    a.contrib_next = contrib2 + (size_t)((it + 1) & 1) * V;
    if (cnt[0]) {
      note_launch();
      k_pr_small<<<g->sm_count * 8, 256, 0, st>>>(a, bins, cnt[0]);
    }
    if (cnt[1]) {
      note_launch();
      k_pr_mid<<<g->sm_count * 8, 256, 0, st>>>(a, bins + V, cnt[1]);
    }
    if (cnt[2]) {
      note_launch();
      k_pr_large<<<std::min(cnt[2], g->sm_count * 4), 512, 0, st>>>(a, bins + 2 * (size_t)V, cnt[2]);
    }
  }
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

}  // namespace gg
