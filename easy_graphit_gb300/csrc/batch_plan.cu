// Batch plans: a whole batched BFS, SSSP or BC (every pass of every group of
// sources) captured once into a CUDA graph and replayed with one
// cudaGraphLaunch per step -- no host round trips, no per-kernel launch cost.
// The plan owns its device state and its copy of the sources, and writes into
// a device buffer the caller owns.
#include <vector>

#include "batch.h"

struct gg_batch_plan {
  gg_graph *g = nullptr;
  int32_t app = 0;
  int32_t nsrc = 0;
  int32_t *dsrc = nullptr;       // device copy of the sources
  int32_t *dstats = nullptr;     // per-group stats [ngroups][2]
  int32_t ngroups = 0;
  gg::BsBuffers bs;
  gg::MsBfsBuffers ms;
  gg::BcBuffers bc;
  int32_t *parent = nullptr;              // BFS multi-source: parent scratch
  gg::BqBuffers bq;                       // SSSP multi-source: bucket-queue buffers
  gg::Scratch cta;                        // SSSP with a CTA per source
  bool per_cta = false;
  unsigned long long *reached = nullptr;  // BC: reached out-edges summed over sources
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int32_t launches_per_run = 0;
  ~gg_batch_plan() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (dsrc) cudaFree(dsrc);
    if (dstats) cudaFree(dstats);
    if (reached) cudaFree(reached);
    if (parent) cudaFree(parent);
    if (bq.base) gg::bq_free(g, &bq);
    if (cta.p) cudaFreeAsync(cta.p, g->stream);
  }
};

using namespace gg;

extern "C" {

gg_status gg_batch_plan_create(gg_graph *g, int32_t app, const int32_t *sources, int32_t nsrc,
                               int32_t delta, void *out, gg_batch_plan **plan) {
  GG_CHECK_ARG(g && sources && nsrc > 0 && out && plan, "bad arguments");
  GG_CHECK_ARG(app >= GG_BATCH_BFS && app <= GG_BATCH_SSSP_MULTI, "unknown batched app");
  GG_CHECK_ARG((app != GG_BATCH_SSSP && app != GG_BATCH_SSSP_MULTI) || delta >= 1, "delta must be >= 1");
  const bool multi = app == GG_BATCH_BFS_MULTI || app == GG_BATCH_SSSP_MULTI;
  cudaPointerAttributes pa{};
  if (cudaPointerGetAttributes(&pa, out) != cudaSuccess || pa.type != cudaMemoryTypeDevice)
    return set_error(GG_ERR_INVALID, "a batch plan writes into device memory; out is not device memory");
  const int32_t V = g->csr.V;
  for (int32_t i = 0; i < nsrc; ++i)
    GG_CHECK_ARG(sources[i] >= 0 && sources[i] < V, "source out of range");
  auto p = std::make_unique<gg_batch_plan>();
  p->g = g;
  p->app = app;
  p->nsrc = nsrc;
  int32_t width = multi ? nsrc : (app == GG_BATCH_SSSP ? kBsLanes : kMsBfsWidth);
  if (app == GG_BATCH_SSSP) {
    bool per_cta = false;
    GG_TRY(bsssp_use_cta(g, &per_cta));
    if (per_cta) width = std::min(bsssp_cta_width(g), nsrc);
  }
  p->ngroups = ceil_div(nsrc, width);
  GG_CUDA(cudaMalloc(&p->dsrc, sizeof(int32_t) * nsrc));
  GG_CUDA(cudaMemcpy(p->dsrc, sources, sizeof(int32_t) * nsrc, cudaMemcpyDefault));
  GG_CUDA(cudaMalloc(&p->dstats, sizeof(int32_t) * 2 * p->ngroups));
  if (multi) {
    if (!g->app_frontier) GG_TRY(gg_frontier_create(g, 0, &g->app_frontier));
    if (app == GG_BATCH_BFS_MULTI) GG_CUDA(cudaMalloc(&p->parent, sizeof(int32_t) * std::max(V, 1)));
    if (app == GG_BATCH_SSSP_MULTI) GG_TRY(bq_alloc(g, &p->bq));
  } else if (app == GG_BATCH_BFS) {
    GG_TRY(msbfs_buffers(g, nsrc, true, &p->ms));
  } else if (app == GG_BATCH_SSSP) {
    GG_TRY(bsssp_use_cta(g, &p->per_cta));
    if (!p->per_cta) GG_TRY(bsssp_buffers(g, nsrc, true, &p->bs));
  } else {
    GG_TRY(bcb_buffers(g, true, &p->bc));
    GG_CUDA(cudaMalloc(&p->reached, sizeof(unsigned long long)));
  }
  if (p->per_cta) {
    CtaBuffers cb;
    GG_TRY(bsssp_cta_buffers(g, width, &p->cta, &cb));
  }
  // Capture on the graph's own stream (capturable even when the graph is
  // bound to a legacy default stream).
  cudaStream_t cs = g->own_stream;
  GG_CUDA(cudaStreamSynchronize(g->stream));
  const uint64_t l0 = launches();
  GG_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
  gg_status st = GG_OK;
  if (app == GG_BATCH_BC) {
    const cudaError_t me = cudaMemsetAsync(p->reached, 0, sizeof(unsigned long long), cs);
    if (me != cudaSuccess) st = set_error(GG_ERR_CUDA, "memset in capture: %s", cudaGetErrorString(me));
  }
  if (multi) {
    const int32_t *run_stats = nullptr;
    st = fused_multi_enqueue(g, cs, app == GG_BATCH_SSSP_MULTI, p->dsrc, nsrc, delta, p->parent, (int32_t *)out,
                             &p->bq, &run_stats);
    if (st == GG_OK) {
      const cudaError_t ce2 = cudaMemcpyAsync(p->dstats, run_stats, sizeof(int32_t) * 2,
                                              cudaMemcpyDeviceToDevice, cs);
      if (ce2 != cudaSuccess) st = set_error(GG_ERR_CUDA, "stats copy in capture: %s", cudaGetErrorString(ce2));
    }
  }
  for (int32_t gi = 0; gi < p->ngroups && st == GG_OK && !multi; ++gi) {
    const int32_t base = gi * width;
    const int32_t k = std::min(width, nsrc - base);
    if (app == GG_BATCH_BFS) {
      MsBfsState S = msbfs_state(g, p->ms, k, (int32_t *)out + (size_t)base * V);
      S.stats = p->dstats + 2 * gi;
      st = msbfs_enqueue(g, cs, S, p->dsrc + base, false);
    } else if (app == GG_BATCH_SSSP && p->per_cta) {
      CtaBuffers cb;
      st = bsssp_cta_buffers(g, width, &p->cta, &cb);  // sized before the capture: no allocation here
      if (st == GG_OK) {
        const cudaError_t ce1 = cudaMemcpyAsync(cb.dsrc, p->dsrc + base, sizeof(int32_t) * k,
                                                cudaMemcpyDeviceToDevice, cs);
        if (ce1 != cudaSuccess) st = set_error(GG_ERR_CUDA, "source copy in capture: %s", cudaGetErrorString(ce1));
      }
      if (st == GG_OK) st = bsssp_cta_run(g, cs, cb, (int32_t *)out + (size_t)base * V, k, delta, false);
      if (st == GG_OK) {
        const cudaError_t ce2 = cudaMemcpyAsync(p->dstats + 2 * gi, cb.stats, sizeof(int32_t) * 2,
                                                cudaMemcpyDeviceToDevice, cs);
        if (ce2 != cudaSuccess) st = set_error(GG_ERR_CUDA, "stats copy in capture: %s", cudaGetErrorString(ce2));
      }
    } else if (app == GG_BATCH_SSSP) {
      BsState S = bsssp_state(g, p->bs, delta);
      S.stats = p->dstats + 2 * gi;
      st = bsssp_enqueue(g, cs, S, p->dsrc + base, k, (int32_t *)out + (size_t)base * V, false);
    } else {
      st = bcb_enqueue(g, cs, p->bc, k, p->dsrc + base, (float *)out + (size_t)base * V, V, p->reached,
                       p->dstats + 2 * gi, false);
    }
  }
  cudaGraph_t graph = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(cs, &graph);
  if (st != GG_OK) {
    if (graph) cudaGraphDestroy(graph);
    return st;
  }
  if (ce != cudaSuccess)
    return set_error(GG_ERR_CUDA, "stream capture of the batch failed: %s", cudaGetErrorString(ce));
  p->graph = graph;
  GG_CUDA(cudaGraphInstantiate(&p->exec, graph, 0));
  p->launches_per_run = (int32_t)(launches() - l0);
  *plan = p.release();
  return GG_OK;
}

gg_status gg_batch_plan_run(gg_batch_plan *p, gg_stats *stats) {
  GG_CHECK_ARG(p && p->exec, "plan is NULL");
  gg_graph *g = p->g;
  cudaStream_t st = g->stream;
  if (stats) *stats = gg_stats{};
  GG_CUDA(cudaEventRecord(g->ev0, st));
  GG_CUDA(cudaGraphLaunch(p->exec, st));
  GG_CUDA(cudaEventRecord(g->ev1, st));
  for (int i = 0; i < p->launches_per_run; ++i) note_launch();
  GG_CUDA(cudaEventSynchronize(g->ev1));
  GG_TRY(check_device_error(g, "batch plan"));
  if (stats) {
    std::vector<int32_t> h(2 * p->ngroups);
    GG_CUDA(cudaMemcpy(h.data(), p->dstats, sizeof(int32_t) * h.size(), cudaMemcpyDeviceToHost));
    for (int32_t gi = 0; gi < p->ngroups; ++gi) {
      stats->iterations = std::max(stats->iterations, h[2 * gi]);
      if (p->app == GG_BATCH_SSSP || p->app == GG_BATCH_SSSP_MULTI) stats->bucket_advances += h[2 * gi + 1];
    }
    if (p->app == GG_BATCH_BC) {
      unsigned long long er = 0;
      GG_CUDA(cudaMemcpy(&er, p->reached, sizeof(er), cudaMemcpyDeviceToHost));
      stats->edges_traversed = 2 * (int64_t)er;
    }
    cudaEventElapsedTime(&stats->device_ms, g->ev0, g->ev1);
    stats->loop_ms = stats->device_ms;
    stats->fused = 1;
    stats->launches = p->launches_per_run;
  }
  return GG_OK;
}

gg_status gg_batch_plan_destroy(gg_batch_plan *p) {
  delete p;
  return GG_OK;
}

}  // extern "C"
