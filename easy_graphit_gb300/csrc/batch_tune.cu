// Launch-shape tuning of the batched kernels: a graph keeps one gg_batch_tuning
// per batched app, and the autotuner picks it by timing candidates on the
// graph itself (coordinate descent: CTAs per SM, then the work-item chunk,
// then SSSP's edge-parallel threshold).  Candidates change only how the work
// is spread over the GPU, never a result.
#include <vector>

#include "batch.h"
#include "lb.cuh"

namespace gg {
namespace {

bool valid_tuning(const gg_batch_tuning &t) {
  if (t.blocks_per_sm < 0 || t.blocks_per_sm > 64) return false;
  if (t.chunk != 0 && (t.chunk < kMinChunk || t.chunk > kMaxChunk || (t.chunk & (t.chunk - 1)))) return false;
  if (t.edge_parallel_max < -1 || t.edge_parallel_max > 32) return false;
  if (t.bottom_up_div < -1 || t.bottom_up_div > 4096) return false;
  return true;
}

// One timed pass of the app over the first k sources (device array dsrc);
// returns the persistent kernel's time.
struct Trial {
  gg_graph *g;
  int32_t app, k, delta;
  const int32_t *dsrc;
  BsBuffers bs;
  MsBfsBuffers ms;
  BcBuffers bc;
  int32_t *rows = nullptr;
  unsigned long long *reached = nullptr;

  gg_status setup() {
    const int32_t V = g->csr.V;
    if (app == GG_BATCH_SSSP) GG_TRY(bsssp_buffers(g, k, true, &bs));
    if (app == GG_BATCH_BFS) GG_TRY(msbfs_buffers(g, k, true, &ms));
    if (app == GG_BATCH_BC) {
      GG_TRY(bcb_buffers(g, true, &bc));
      GG_CUDA(cudaMalloc(&reached, sizeof(unsigned long long)));
    }
    GG_CUDA(cudaMalloc(&rows, sizeof(int32_t) * (size_t)k * V));
    return GG_OK;
  }
  ~Trial() {
    if (rows) cudaFree(rows);
    if (reached) cudaFree(reached);
  }
  gg_status run(float *ms_out) {
    cudaStream_t st = g->stream;
    if (app == GG_BATCH_SSSP) {
      const BsState S = bsssp_state(g, bs, delta);
      GG_TRY(bsssp_enqueue(g, st, S, dsrc, k, rows, true));
    } else if (app == GG_BATCH_BFS) {
      const MsBfsState S = msbfs_state(g, ms, k, rows);
      GG_TRY(msbfs_enqueue(g, st, S, dsrc, true));
    } else {
      GG_TRY(bcb_enqueue(g, st, bc, k, dsrc, reinterpret_cast<float *>(rows), g->csr.V, reached, nullptr, true));
    }
    GG_CUDA(cudaStreamSynchronize(st));
    GG_TRY(check_device_error(g, "batch autotune"));
    GG_CUDA(cudaEventElapsedTime(ms_out, g->ev2, g->ev3));
    return GG_OK;
  }
};

}  // namespace
}  // namespace gg

using namespace gg;

extern "C" {

gg_status gg_batch_set_tuning(gg_graph *g, int32_t app, const gg_batch_tuning *t) {
  GG_CHECK_ARG(g && t, "bad arguments");
  GG_CHECK_ARG(app >= GG_BATCH_BFS && app <= GG_BATCH_BC, "unknown batched app");
  if (!valid_tuning(*t))
    return set_error(GG_ERR_INVALID,
                     "tuning out of range (blocks_per_sm %d, chunk %d, edge_parallel_max %d, bottom_up_div %d)",
                     t->blocks_per_sm, t->chunk, t->edge_parallel_max, t->bottom_up_div);
  g->tuning[app] = *t;
  return GG_OK;
}

gg_status gg_batch_get_tuning(const gg_graph *g, int32_t app, gg_batch_tuning *t) {
  GG_CHECK_ARG(g && t, "bad arguments");
  GG_CHECK_ARG(app >= GG_BATCH_BFS && app <= GG_BATCH_BC, "unknown batched app");
  *t = g->tuning[app];
  return GG_OK;
}

gg_status gg_batch_autotune(gg_graph *g, int32_t app, const int32_t *sources, int32_t nsrc, int32_t delta,
                            gg_batch_tuning *best, gg_tune_row *rows, int32_t max_rows, int32_t *nrows) {
  GG_CHECK_ARG(g && sources && nsrc > 0 && best, "bad arguments");
  GG_CHECK_ARG(app >= GG_BATCH_BFS && app <= GG_BATCH_BC, "unknown batched app");
  GG_CHECK_ARG(app != GG_BATCH_SSSP || delta >= 1, "delta must be >= 1");
  const int32_t V = g->csr.V;
  for (int32_t i = 0; i < nsrc; ++i)
    GG_CHECK_ARG(sources[i] >= 0 && sources[i] < V, "source out of range");
  const int32_t width = app == GG_BATCH_SSSP ? kBsLanes : kMsBfsWidth;
  const int32_t k = std::min(nsrc, width);
  int fit = 0;
  if (app == GG_BATCH_SSSP)
    GG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, bsssp_kernel(), 256, 0));
  else
    GG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, app == GG_BATCH_BFS ? msbfs_kernel() : bcb_kernel(),
                                                         512, twce_smem_bytes(512)));
  if (fit < 1) return set_error(GG_ERR_UNSUPPORTED, "batched kernel does not fit an SM");
  int32_t *dsrc = nullptr;
  GG_CUDA(cudaMalloc(&dsrc, sizeof(int32_t) * k));
  struct Free {
    int32_t *p;
    ~Free() { cudaFree(p); }
  } free_dsrc{dsrc};
  GG_CUDA(cudaMemcpy(dsrc, sources, sizeof(int32_t) * k, cudaMemcpyDefault));
  Trial tr{g, app, k, delta, dsrc};
  GG_TRY(tr.setup());
  const gg_batch_tuning saved = g->tuning[app];
  int32_t n = 0;
  float best_ms = INFINITY;
  gg_batch_tuning cur = effective_tuning(g, app, fit);
  gg_batch_tuning win = cur;
  auto time_one = [&](const gg_batch_tuning &t) -> gg_status {
    g->tuning[app] = t;
    float m0 = 0, m1 = 0;
    gg_status s = tr.run(&m0);                       // warm-up (and first timing)
    if (s == GG_OK) s = tr.run(&m1);
    if (s != GG_OK) {
      g->tuning[app] = saved;
      return s;
    }
    const float ms = std::min(m0, m1);
    if (rows && n < max_rows) rows[n] = gg_tune_row{t, ms};
    ++n;
    if (ms < best_ms) {
      best_ms = ms;
      win = t;
    }
    return GG_OK;
  };
  // 1. CTAs per SM
  for (int b = 1; b <= fit; ++b) {
    gg_batch_tuning t = cur;
    t.blocks_per_sm = b;
    GG_TRY(time_one(t));
  }
  cur = win;
  // 2. work-item chunk (SSSP, BC)
  if (app != GG_BATCH_BFS) {
    for (int c : {64, 128, 256, 512, 1024}) {
      if (c == cur.chunk) continue;
      gg_batch_tuning t = cur;
      t.chunk = c;
      GG_TRY(time_one(t));
    }
    cur = win;
  }
  // 3. bottom-up threshold (BFS)
  if (app == GG_BATCH_BFS) {
    for (int d : {-1, 4, 64, 256}) {
      if (d == cur.bottom_up_div) continue;
      gg_batch_tuning t = cur;
      t.bottom_up_div = d;
      GG_TRY(time_one(t));
    }
  }
  // 4. edge-parallel threshold (SSSP)
  if (app == GG_BATCH_SSSP) {
    for (int e : {-1, 2, 12, 32}) {
      if (e == cur.edge_parallel_max) continue;
      gg_batch_tuning t = cur;
      t.edge_parallel_max = e;
      GG_TRY(time_one(t));
    }
  }
  g->tuning[app] = win;
  *best = win;
  if (nrows) *nrows = n;
  return GG_OK;
}

}  // extern "C"
