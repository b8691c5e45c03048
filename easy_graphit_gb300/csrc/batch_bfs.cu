// Batched BFS: up to 64 sources per pass in one persistent kernel.
//
// Bit-parallel multi-source BFS: every vertex carries 64-bit masks -- `seen`
// (sources that reached it), `acc` (sources reaching it this level) and the
// level masks fr (sources for which it is on the level's frontier).  Levels run
// top-down or bottom-up (direction optimisation, as bfs.cpp's hybrid schedule
// does for one source, here for all sources at once):
//  * top-down: one traversal of an edge (u, v) serves every source,
//    acc[v] |= fr[u] & ~seen[v]; frontier vertices are load-balanced by the TWCE
//    device function of lb.cuh; a publish phase then turns new bits into the
//    next level's masks and depths;
//  * bottom-up (frontier larger than V / bu_div): groups of 8 lanes take the
//    vertices some still-expanding source has not reached and OR the level
//    masks of their in-neighbours, 8 at a time, stopping as soon as every such
//    source is found; no atomics.
// Level masks rotate through three arrays and queues through three buffers:
// the masks of level L-1 are cleared (from its queue) while level L publishes,
// so a bottom-up scan never reads a stale mask.
//
// The result for each source equals an independent BFS (apps/bfs.cpp), because
// a source's bit enters seen[v] exactly at the first level that reaches v.
#include <vector>

#include "batch.h"
#include "lb.cuh"
#include "selector.h"

namespace gg {

__device__ __forceinline__ uint64_t *ms_fr(const MsBfsState &st, int32_t level) {
  const int32_t i = level % 3;
  return i == 0 ? st.fr[0] : (i == 1 ? st.fr[1] : st.fr[2]);
}
__device__ __forceinline__ int32_t *ms_q(const MsBfsState &st, int32_t level) {
  const int32_t i = level % 3;
  return i == 0 ? st.q[0] : (i == 1 ? st.q[1] : st.q[2]);
}

// depth[s][v] = level for every bit s of nb, the bits split over `ways` lanes.
__device__ __forceinline__ void ms_depths(const MsBfsState &st, int32_t v, uint64_t nb, int32_t level,
                                          int32_t sub, int32_t ways) {
  if (!st.depth) return;
  for (uint64_t b = nb; b; b &= b - 1) {
    const int32_t s = __ffsll((long long)b) - 1;
    if (s % ways == sub) st.depth[(int64_t)s * st.depth_stride + v] = level;
  }
}

// Adds the out-degree of v, entering the next level's queue, to the CTA's
// statistics of that frontier.
__device__ __forceinline__ void ms_note(const MsBfsState &st, unsigned long long *s_stat, int32_t v) {
  const unsigned long long d = (unsigned long long)(__ldg(st.off + v + 1) - __ldg(st.off + v));
  atomicAdd(s_stat, d);
  atomicAdd(s_stat + 1, d * d);
  atomicMax(s_stat + 2, d);
}

__global__ void __launch_bounds__(512) k_msbfs(DGraph g, MsBfsState st) {
  extern __shared__ int4 smem[];
  __shared__ unsigned long long s_act;
  __shared__ unsigned long long s_stat[3];
  const int32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int32_t nthreads = gridDim.x * blockDim.x;
  const int32_t lane = threadIdx.x & 31;
  LoopClock clk;
  clk.start(st.loop_limit_ns);
  int32_t L = 0, bu_levels = 0;
  double vis_v = 0, vis_e = 0;  // running totals of the frontiers so far (the same in every CTA)
  for (;; ++L) {
    const int32_t n = *(volatile int32_t *)(st.cnt4 + (L & 3));
    if (n == 0 || stopped(st.stop, L)) break;
    const volatile unsigned long long *ls = st.lstat + 4 * (L % 3);
    const double sd = (double)ls[0], sd2 = (double)ls[1], mx = (double)ls[2];
    if (tid == 0) {
      st.cnt4[(L + 2) & 3] = 0;
      st.actm[(L + 2) % 3] = 0ull;
      for (int i = 0; i < 4; ++i) st.lstat[4 * ((L + 2) % 3) + i] = 0ull;
    }
    if (threadIdx.x == 0) {
      s_act = 0ull;
      s_stat[0] = s_stat[1] = s_stat[2] = 0ull;
    }
    // direction of this level: forced, the network's, or the bu_div rule
    bool bu;
    if (st.force_dir >= 0) {
      bu = st.force_dir == 1;
    } else if (st.sel || st.feat_log) {
      float *x = reinterpret_cast<float *>(smem);  // scratch until the level's TWCE bins
      if (threadIdx.x == 0)
        selector_features(x, (double)n, sd, sd2, mx, vis_v, vis_e, L, (double)st.V, (double)st.E);
      __syncthreads();
      bu = st.sel ? selector_pull(st.sel, x, x + 16) : (st.bu_div > 0 && (int64_t)n * st.bu_div > st.V);
    } else {
      bu = st.bu_div > 0 && (int64_t)n * st.bu_div > st.V;
    }
    if (st.feat_log && L <= st.max_log && blockIdx.x == 0 && threadIdx.x == 0) {
      const float *x = reinterpret_cast<const float *>(smem);
      if (!(st.force_dir >= 0) && L < st.max_log)
        for (int i = 0; i < kSelectorFeatures; ++i) st.feat_log[L * kSelectorFeatures + i] = x[i];
      st.time_log[L] = globaltimer_ns();  // the end of level L-1 (max_log + 1 entries)
    }
    if (st.force_dir >= 0 && st.feat_log && L < st.max_log && blockIdx.x == 0 && threadIdx.x == 0) {
      float x[kSelectorFeatures];
      selector_features(x, (double)n, sd, sd2, mx, vis_v, vis_e, L, (double)st.V, (double)st.E);
      for (int i = 0; i < kSelectorFeatures; ++i) st.feat_log[L * kSelectorFeatures + i] = x[i];
    }
    vis_v = fmin((double)st.V, vis_v + n);
    vis_e = fmin((double)st.E, vis_e + sd);
    __syncthreads();
    const uint64_t *frc = ms_fr(st, L);
    uint64_t *frn = ms_fr(st, L + 1);
    int32_t *qn = ms_q(st, L + 1);
    if (!bu) {
      // top-down: acc[v] |= fr[u] & ~seen[v]; the first toucher queues v
      const Enum en{ms_q(st, L), nullptr, n};
      const UMsBfs f{st.seen, frc, st.acc, st.qstamp, L + 1};
      DOut out{};
      out.mode = OUT_SPARSE;
      out.q = qn;
      out.cnt = st.cnt4 + ((L + 1) & 3);
      out.cap = st.V;  // qstamp admits each vertex once per level
      out.err = st.err;
      const int32_t nv = ceil_div(n, blockDim.x / kStage1);
      for (int32_t v = blockIdx.x; v < nv; v += gridDim.x)
        lb_twce<UMsBfs, true>(g, en, n, f, out, v, *reinterpret_cast<TwceSmem *>(smem));
    } else {
      // bottom-up: 8-lane groups over the vertices still wanted by some source
      ++bu_levels;
      const uint64_t act = *(volatile unsigned long long *)(st.actm + L % 3);
      const int32_t sub = lane & 7;
      const uint32_t gmask = 0xFFu << (lane & ~7);
      for (int32_t v = tid >> 3; v < st.V; v += nthreads >> 3) {
        const uint64_t sv = __ldcg(st.seen + v);
        const uint64_t want = act & ~sv;
        if (!want) continue;
        const int32_t kb = __ldg(st.toff + v), ke = __ldg(st.toff + v + 1);
        uint64_t found = 0;
        for (int32_t k0 = kb; k0 < ke; k0 += 8) {
          uint64_t m = 0;
          if (k0 + sub < ke) m = __ldcg(frc + __ldg(st.tsrc + k0 + sub)) & want;
          m |= __shfl_xor_sync(gmask, m, 1);
          m |= __shfl_xor_sync(gmask, m, 2);
          m |= __shfl_xor_sync(gmask, m, 4);
          found |= m;
          if (found == want) break;
        }
        if (found) {
          if (sub == 0) {
            st.seen[v] = sv | found;
            frn[v] = found;
            const int32_t pos = atomicAdd(st.cnt4 + ((L + 1) & 3), 1);
            if (pos < st.V)
              qn[pos] = v;
            else
              atomicOr(st.err, DEV_ERR_OVERFLOW);
            atomicOr(&s_act, (unsigned long long)found);
            ms_note(st, s_stat, v);
          }
          ms_depths(st, v, found, L + 1, sub, 8);
        }
      }
    }
    if (!grid_barrier(st.bar, gridDim.x, st.err, st.timeout_ns)) break;
    // publish (top-down levels): new bits become the next level's masks
    if (!bu) {
      const int32_t m = min(*(volatile int32_t *)(st.cnt4 + ((L + 1) & 3)), st.V);
      for (int32_t i = tid; i < m; i += nthreads) {
        const int32_t v = __ldcg(qn + i);
        const uint64_t a = __ldcg(st.acc + v);
        const uint64_t sv = __ldcg(st.seen + v);
        const uint64_t nb = a & ~sv;
        st.seen[v] = sv | nb;
        frn[v] = nb;
        st.acc[v] = 0;
        atomicOr(&s_act, (unsigned long long)nb);
        ms_note(st, s_stat, v);
        ms_depths(st, v, nb, L + 1, 0, 1);
      }
    }
    // the masks of level L-1 are dead: clear them for the bottom-up scans
    if (L >= 1) {
      uint64_t *old = ms_fr(st, L - 1);
      const int32_t *qo = ms_q(st, L - 1);
      const int32_t m = min(*(volatile int32_t *)(st.cnt4 + ((L - 1) & 3)), st.V);
      for (int32_t i = tid; i < m; i += nthreads) old[__ldcg(qo + i)] = 0ull;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      if (s_act) atomicOr(st.actm + (L + 1) % 3, s_act);
      unsigned long long *nx = st.lstat + 4 * ((L + 1) % 3);  // statistics of the next frontier
      if (s_stat[0]) {
        atomicAdd(nx, s_stat[0]);
        atomicAdd(nx + 1, s_stat[1]);
        atomicMax(nx + 2, s_stat[2]);
      }
    }
    clk.tick(st.stop, L, st.err);
    if (!grid_barrier(st.bar, gridDim.x, st.err, st.timeout_ns)) break;
  }
  if (tid == 0) {
    st.stats[0] = L;
    st.stats[1] = bu_levels;
    if (st.time_log && L <= st.max_log) st.time_log[L] = globaltimer_ns();
  }
}

// Initial state: masks cleared, depth rows -1.
__global__ void k_msbfs_init(MsBfsState st) {
  const int64_t total = (int64_t)st.nsrc * st.depth_stride;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x)
    st.depth[i] = -1;
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < st.V; v += gridDim.x * blockDim.x) {
    st.seen[v] = 0;
    st.acc[v] = 0;
    st.fr[0][v] = 0;
    st.fr[1][v] = 0;
    st.fr[2][v] = 0;
    st.qstamp[v] = 0;
  }
}

// Sources seeded (one thread: sources are few; duplicates share a vertex).
__global__ void k_msbfs_seed(MsBfsState st, const int32_t *__restrict__ srcs) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  int32_t n = 0;
  unsigned long long all = 0;
  for (int32_t s = 0; s < st.nsrc; ++s) {
    const int32_t v = srcs[s];
    if (!st.seen[v]) st.q[0][n++] = v;
    st.seen[v] |= 1ull << s;
    st.fr[0][v] |= 1ull << s;
    all |= 1ull << s;
    st.depth[(int64_t)s * st.depth_stride + v] = 0;
  }
  for (int i = 0; i < 4; ++i) st.cnt4[i] = 0;
  st.cnt4[0] = n;
  for (int i = 0; i < 12; ++i) st.lstat[i] = 0ull;
  for (int32_t i = 0; i < n; ++i) {  // the sources' frontier
    const unsigned long long d = (unsigned long long)(st.off[st.q[0][i] + 1] - st.off[st.q[0][i]]);
    st.lstat[0] += d;
    st.lstat[1] += d * d;
    st.lstat[2] = st.lstat[2] > d ? st.lstat[2] : d;
  }
  st.actm[0] = all;
  st.actm[1] = 0;
  st.actm[2] = 0;
  *st.stop = 0;
}

// ------------------------------------------------------------------ host
MsBfsBuffers::~MsBfsBuffers() {
  if (owned)
    for (void *p : {(void *)masks, (void *)ints, (void *)dsrc})
      if (p) cudaFree(p);
}

gg_status msbfs_buffers(gg_graph *g, int32_t nsrc, bool owned, MsBfsBuffers *b) {
  GG_TRY(ensure_transpose(g));  // in-lists for the bottom-up levels
  const int32_t V = g->csr.V;
  b->owned = owned;
  const size_t sz[3] = {sizeof(uint64_t) * (5 * (size_t)V + 24), sizeof(int32_t) * (4 * (size_t)V + 64),
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
  const GraphStore &t = g->csc ? *g->csc : g->csr;
  MsBfsState S{};
  S.seen = b.masks;
  S.acc = b.masks + V;
  for (int i = 0; i < 3; ++i) S.fr[i] = b.masks + (2 + i) * (size_t)V;
  S.actm = reinterpret_cast<unsigned long long *>(b.masks + 5 * (size_t)V);
  S.lstat = reinterpret_cast<unsigned long long *>(b.masks + 5 * (size_t)V + 8);
  S.qstamp = b.ints;
  for (int i = 0; i < 3; ++i) S.q[i] = b.ints + (1 + i) * (size_t)V;
  int32_t *hdr = b.ints + 4 * (size_t)V;
  S.cnt4 = hdr;          // 4
  S.stats = hdr + 8;     // 2
  S.stop = hdr + 12;
  S.toff = t.off;
  S.tsrc = t.dst;
  S.V = V;
  const gg_batch_tuning tn = effective_tuning(g, GG_BATCH_BFS, 1);
  S.bu_div = tn.bottom_up_div;
  S.loop_limit_ns = loop_timeout_ns();
  S.depth = depth_rows;
  S.depth_stride = V;
  S.nsrc = k;
  S.bar = g->d_bar;
  S.err = g->d_err;
  S.timeout_ns = barrier_timeout_ns();
  S.sel = g->batch_selector[GG_BATCH_BFS] ? selector_params(g->batch_selector[GG_BATCH_BFS]) : nullptr;
  S.force_dir = -1;
  S.off = g->csr.off;
  S.E = g->csr.E;
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
  k_msbfs_init<<<g->sm_count * 8, 256, 0, st>>>(S);
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

// Attaches a selector network to a graph's batched kernels (NULL detaches it).
extern "C" gg_status gg_batch_set_selector(gg_graph *g, int32_t app, const gg_selector *sel) {
  GG_CHECK_ARG(g, "graph is NULL");
  if (app != GG_BATCH_BFS)
    return set_error(GG_ERR_UNSUPPORTED, "only batched BFS takes a learned per-level choice");
  g->batch_selector[app] = sel;
  return GG_OK;
}

// Training data for the batched BFS direction: the first min(nsrc, 64) sources
// traversed with every level top-down, then with every level bottom-up (twice
// each; a level's masks after it are the same either way, so level l starts
// from the same state in every run).  feats[l][12]: the features of level l;
// times[l][2]: its best time in ms top-down and bottom-up.
extern "C" gg_status gg_batch_collect(gg_graph *g, int32_t app, const int32_t *sources, int32_t nsrc,
                                      int32_t max_rows, float *feats, float *times, int32_t *nrows) {
  GG_CHECK_ARG(g && sources && nsrc > 0 && feats && times && nrows && max_rows > 0, "bad arguments");
  if (app != GG_BATCH_BFS) return set_error(GG_ERR_UNSUPPORTED, "timings are collected for batched BFS");
  const int32_t V = g->csr.V;
  for (int32_t i = 0; i < nsrc; ++i) GG_CHECK_ARG(sources[i] >= 0 && sources[i] < V, "source out of range");
  *nrows = 0;
  cudaStream_t st = g->stream;
  const int32_t k = std::min(nsrc, kMsBfsWidth);
  MsBfsBuffers b;
  GG_TRY(msbfs_buffers(g, k, false, &b));
  int32_t *depth = nullptr;
  GG_TRY(scratch_get_app(g, 3, sizeof(int32_t) * (size_t)k * V, (void **)&depth));
  float *dfeat = nullptr;
  unsigned long long *dtime = nullptr;
  GG_CUDA(dev_alloc(&dfeat, sizeof(float) * kSelectorFeatures * (size_t)max_rows, st));
  GG_CUDA(dev_alloc(&dtime, sizeof(unsigned long long) * ((size_t)max_rows + 1), st));
  std::vector<float> best(2 * (size_t)max_rows, INFINITY);
  std::vector<unsigned long long> ht((size_t)max_rows + 1);
  int32_t levels = -1;
  gg_status status = GG_OK;
  for (int rep = 0; rep < 4 && status == GG_OK; ++rep) {
    const int dir = rep & 1;
    MsBfsState S = msbfs_state(g, b, k, depth);
    S.force_dir = dir;
    S.feat_log = dfeat;
    S.time_log = dtime;
    S.max_log = max_rows;
    if (cudaMemcpyAsync(b.dsrc, sources, sizeof(int32_t) * k, cudaMemcpyDefault, st) != cudaSuccess ||
        (status = msbfs_enqueue(g, st, S, b.dsrc, false)) != GG_OK)
      break;
    int32_t lv = 0;
    if (cudaMemcpyAsync(&lv, S.stats, sizeof(int32_t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
      status = set_error(GG_ERR_CUDA, "batched BFS timing run failed");
      break;
    }
    if ((status = check_device_error(g, "batch_collect")) != GG_OK) break;
    if (levels >= 0 && lv != levels) {
      status = set_error(GG_ERR_STATE, "level counts differ between direction runs (%d, %d)", levels, lv);
      break;
    }
    levels = lv;
    const int32_t rows = std::min(levels, max_rows);
    cudaMemcpy(ht.data(), dtime, sizeof(unsigned long long) * ((size_t)rows + 1), cudaMemcpyDeviceToHost);
    for (int32_t l = 0; l < rows; ++l)
      best[2 * l + dir] = std::min(best[2 * l + dir], (float)((double)(ht[l + 1] - ht[l]) * 1e-6));
    if (rep == 0)
      cudaMemcpy(feats, dfeat, sizeof(float) * kSelectorFeatures * (size_t)rows, cudaMemcpyDeviceToHost);
  }
  cudaFreeAsync(dfeat, st);
  cudaFreeAsync(dtime, st);
  GG_TRY(status);
  *nrows = std::min(levels, max_rows);
  for (int32_t i = 0; i < 2 * *nrows; ++i) times[i] = best[i];
  return GG_OK;
}
