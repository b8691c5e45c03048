// Batched BFS: up to 64 sources per pass in one persistent kernel.
//
// Bit-parallel multi-source BFS: every vertex carries 64-bit masks -- `seen`
// (sources that reached it), `acc` (sources reaching it this level) and `fr`
// (sources for which it is on the current frontier).  One traversal of an edge
// (u, v) serves every source at once: acc[v] |= fr[u] & ~seen[v].  A level ends
// with a grid barrier, then the vertices touched this level publish their new
// bits (fr = acc & ~seen, seen |= fr), write depth[s][v] = level for each new
// bit, and form the next frontier.  Frontier vertices are load-balanced by the
// TWCE device function of lb.cuh, so hubs are split across a warp or the CTA.
//
// The result for each source equals an independent BFS (apps/bfs.cpp), because
// a source's bit enters seen[v] exactly at the first level that reaches v.
#include <vector>

#include "batch.h"
#include "lb.cuh"

namespace gg {

__global__ void __launch_bounds__(512) k_msbfs(DGraph g, MsBfsState st) {
  extern __shared__ int4 smem[];
  int32_t *qs[2] = {st.q0, st.q1};
  int in = 0;
  int64_t level = 1;
  const int32_t stride = gridDim.x * blockDim.x;
  LoopClock clk;
  clk.start(st.loop_limit_ns);
  for (;; ++level) {
    const int32_t n = *(volatile int32_t *)(st.cnt3 + (level - 1) % 3);
    if (n == 0 || stopped(st.stop, st.err)) break;
    if (blockIdx.x == 0 && threadIdx.x == 0) st.cnt3[(level + 1) % 3] = 0;
    // relax: acc[v] |= fr[u] & ~seen[v]
    {
      const Enum en{qs[in], nullptr, n};
      const UMsBfs f{st.seen, st.fr, st.acc, st.qstamp, (int32_t)level};
      DOut out{};
      out.mode = OUT_SPARSE;
      out.q = qs[in ^ 1];
      out.cnt = st.cnt3 + level % 3;
      out.cap = g.V;  // qstamp admits each vertex once per level
      out.err = st.err;
      const int32_t nv = ceil_div(n, blockDim.x / kStage1);
      for (int32_t v = blockIdx.x; v < nv; v += gridDim.x)
        lb_twce<UMsBfs, true>(g, en, n, f, out, v, *reinterpret_cast<TwceSmem *>(smem));
    }
    if (!grid_barrier(st.bar, gridDim.x, st.err, st.timeout_ns)) break;
    // publish: new bits become the next frontier masks
    {
      const int32_t m = *(volatile int32_t *)(st.cnt3 + level % 3);
      const int32_t *q = qs[in ^ 1];
      for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) {
        const int32_t v = q[i];
        const uint64_t a = __ldcg(st.acc + v);
        const uint64_t sv = __ldcg(st.seen + v);
        const uint64_t nb = a & ~sv;
        st.seen[v] = sv | nb;
        st.fr[v] = nb;
        st.acc[v] = 0;
        if (st.depth) {
          uint64_t b = nb;
          while (b) {
            const int s = __ffsll((long long)b) - 1;
            b &= b - 1;
            st.depth[(int64_t)s * st.depth_stride + v] = (int32_t)level;
          }
        }
      }
    }
    clk.tick(st.stop);
    if (!grid_barrier(st.bar, gridDim.x, st.err, st.timeout_ns)) break;
    in ^= 1;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) st.stats[0] = (int32_t)(level - 1);
}

// Initial state: masks cleared, depth rows -1, sources seeded.
__global__ void k_msbfs_init(MsBfsState st, int32_t V, const int32_t *__restrict__ srcs) {
  const int64_t total = (int64_t)st.nsrc * st.depth_stride;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x)
    st.depth[i] = -1;
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    st.seen[v] = 0;
    st.acc[v] = 0;
    st.fr[v] = 0;
    st.qstamp[v] = 0;
  }
}

__global__ void k_msbfs_seed(MsBfsState st, const int32_t *__restrict__ srcs) {
  // one thread: sources are few; duplicates share a vertex
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  int32_t n = 0;
  for (int32_t s = 0; s < st.nsrc; ++s) {
    const int32_t v = srcs[s];
    if (!st.seen[v]) st.q0[n++] = v;
    st.seen[v] |= 1ull << s;
    st.fr[v] |= 1ull << s;
    st.depth[(int64_t)s * st.depth_stride + v] = 0;
  }
  st.cnt3[0] = n;
  st.cnt3[1] = 0;
  st.cnt3[2] = 0;
  *st.stop = 0;
}

// ------------------------------------------------------------------ host
MsBfsBuffers::~MsBfsBuffers() {
  if (owned)
    for (void *p : {(void *)masks, (void *)ints, (void *)dsrc})
      if (p) cudaFree(p);
}

gg_status msbfs_buffers(gg_graph *g, int32_t nsrc, bool owned, MsBfsBuffers *b) {
  const int32_t V = g->csr.V;
  b->owned = owned;
  const size_t sz[3] = {sizeof(uint64_t) * 3 * (size_t)V, sizeof(int32_t) * (3 * (size_t)V + 64),
                        sizeof(int32_t) * (size_t)std::max(nsrc, kMsBfsWidth)};
  void **ptr[3] = {(void **)&b->masks, (void **)&b->ints, (void **)&b->dsrc};
  for (int i = 0; i < 3; ++i) {
    if (owned)
      GG_CUDA(cudaMalloc(ptr[i], sz[i]));
    else
      GG_TRY(scratch_get_app(g, i, sz[i], ptr[i]));
  }
  return GG_OK;
}

MsBfsState msbfs_state(gg_graph *g, const MsBfsBuffers &b, int32_t k, int32_t *depth_rows) {
  const int32_t V = g->csr.V;
  MsBfsState S{};
  S.seen = b.masks;
  S.acc = b.masks + V;
  S.fr = b.masks + 2 * (size_t)V;
  S.qstamp = b.ints;
  S.q0 = b.ints + V;
  S.q1 = b.ints + 2 * (size_t)V;
  S.cnt3 = b.ints + 3 * (size_t)V;
  S.stats = b.ints + 3 * (size_t)V + 8;
  S.stop = b.ints + 3 * (size_t)V + 12;
  S.loop_limit_ns = loop_timeout_ns();
  S.depth = depth_rows;
  S.depth_stride = V;
  S.nsrc = k;
  S.bar = g->d_bar;
  S.err = g->d_err;
  S.timeout_ns = barrier_timeout_ns();
  return S;
}

const void *msbfs_kernel() { return (const void *)k_msbfs; }

// One pass of k <= 64 sources: reset, seed, the persistent loop writing the
// depth rows.  Stream-ordered only, so it can be captured into a CUDA graph.
gg_status msbfs_enqueue(gg_graph *g, cudaStream_t st, const MsBfsState &S, const int32_t *dsrc,
                        bool timed) {
  int per_sm = 0;
  const int cta = 512;
  const size_t smem = twce_smem_bytes(cta);
  GG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_msbfs, cta, smem));
  if (per_sm < 1) return set_error(GG_ERR_UNSUPPORTED, "batched BFS kernel does not fit an SM");
  note_launch();
  k_msbfs_init<<<g->sm_count * 8, 256, 0, st>>>(S, g->csr.V, dsrc);
  note_launch();
  k_msbfs_seed<<<1, 32, 0, st>>>(S, dsrc);
  GG_CUDA(cudaMemsetAsync(S.bar, 0, sizeof(uint32_t) * 2, st));
  DGraph dg = g->csr.view();
  dg.nbuckets = 0;
  MsBfsState arg = S;
  void *args[] = {&dg, &arg};
  if (timed) GG_CUDA(cudaEventRecord(g->ev2, st));
  note_launch();
  const int bps = effective_tuning(g, GG_BATCH_BFS, per_sm).blocks_per_sm;
  GG_CUDA(cudaLaunchCooperativeKernel((const void *)k_msbfs, bps * g->sm_count, cta, args, smem, st));
  if (timed) GG_CUDA(cudaEventRecord(g->ev3, st));
  return GG_OK;
}

}  // namespace gg

using namespace gg;

// Batched BFS: depth_out[s*V + v] for nsrc sources (host or device memory).
extern "C" gg_status gg_bfs_batch(gg_graph *g, const int32_t *sources, int32_t nsrc,
                                  int32_t *depth_out, gg_stats *stats) {
  GG_CHECK_ARG(g && sources && nsrc > 0 && depth_out, "bad arguments");
  const int32_t V = g->csr.V;
  for (int32_t i = 0; i < nsrc; ++i)
    GG_CHECK_ARG(sources[i] >= 0 && sources[i] < V, "source out of range");
  if (stats) *stats = gg_stats{};
  cudaStream_t st = g->stream;
  MsBfsBuffers b;
  GG_TRY(msbfs_buffers(g, nsrc, false, &b));
  int32_t *depth = nullptr;
  GG_TRY(scratch_get_app(g, 3, sizeof(int32_t) * (size_t)std::min(nsrc, kMsBfsWidth) * V, (void **)&depth));
  const uint64_t l0 = launches();
  cudaEventRecord(g->ev0, st);
  float loop_ms = 0;
  int32_t levels = 0;
  for (int32_t base = 0; base < nsrc; base += kMsBfsWidth) {
    const int32_t k = std::min(kMsBfsWidth, nsrc - base);
    const MsBfsState S = msbfs_state(g, b, k, depth);
    GG_CUDA(cudaMemcpyAsync(b.dsrc, sources + base, sizeof(int32_t) * k, cudaMemcpyDefault, st));
    GG_TRY(msbfs_enqueue(g, st, S, b.dsrc, true));
    GG_CUDA(cudaMemcpyAsync(depth_out + (size_t)base * V, depth, sizeof(int32_t) * (size_t)k * V,
                            cudaMemcpyDefault, st));
    GG_CUDA(cudaMemcpyAsync(g->h_pinned + 30, S.stats, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    GG_CUDA(cudaStreamSynchronize(st));
    float ms = 0;
    cudaEventElapsedTime(&ms, g->ev2, g->ev3);
    loop_ms += ms;
    levels = std::max(levels, g->h_pinned[30]);
  }
  cudaEventRecord(g->ev1, st);
  GG_CUDA(cudaEventSynchronize(g->ev1));
  GG_TRY(check_device_error(g, "bfs_batch"));
  if (stats) {
    cudaEventElapsedTime(&stats->device_ms, g->ev0, g->ev1);
    stats->loop_ms = loop_ms;
    stats->iterations = levels;
    stats->fused = 1;
    stats->launches = (int32_t)(launches() - l0);
  }
  return GG_OK;
}
