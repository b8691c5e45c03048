// The five apps' testcase() bodies for one trial, on the device operators:
//   BFS  apps/bfs.cpp:36-62     SSSP apps/sssp.cpp:34-57    PR apps/pr.cpp:49-69
//   CC   apps/cc.cpp:53-77      BC   apps/bc.cpp:64-123
// Unfused loops read the frontier size once per iteration, as the generated
// host code does (vertex_frontier.h:109-113); fuse=1 with a simple schedule
// runs the BFS/SSSP loop in one persistent kernel (fused.cu).
#include <vector>

#include "engine.h"
#include "selector.h"

namespace gg {

namespace {

// Hybrid direction switch (operators.cpp:516-532): s1 when
// |frontier| <= threshold * V, else s2.
const gg_schedule *pick(const gg_app_schedule *s, int32_t n, int32_t V) {
  if (s->kind == GG_SCHED_HYBRID) return (float)n <= s->threshold * (float)V ? &s->s1 : &s->s2;
  return &s->s1;
}

template <class T>
gg_status app_array(gg_graph *g, int slot, size_t n, T **p) {
  void *v = nullptr;
  GG_TRY(scratch_get_app(g, slot, sizeof(T) * std::max<size_t>(n, 1), &v));
  *p = (T *)v;
  return GG_OK;
}

gg_status app_frontier(gg_graph *g, gg_frontier **f) {
  if (!g->app_frontier) GG_TRY(gg_frontier_create(g, 0, &g->app_frontier));
  *f = g->app_frontier;
  return GG_OK;
}

// Frontier = {v}.
gg_status frontier_set_single(gg_frontier *f, int32_t v) {
  gg_graph *g = f->g;
  g->h_pinned[10] = v;
  g->h_pinned[11] = 1;
  GG_CUDA(cudaMemsetAsync(f->cnt, 0, sizeof(int32_t) * 2, g->stream));
  GG_CUDA(cudaMemcpyAsync(f->q_in, g->h_pinned + 10, sizeof(int32_t), cudaMemcpyHostToDevice, g->stream));
  GG_CUDA(cudaMemcpyAsync(f->cnt_in, g->h_pinned + 11, sizeof(int32_t), cudaMemcpyHostToDevice, g->stream));
  f->fmt = GG_FMT_SPARSE;
  return GG_OK;
}

__global__ void k_reach(const int32_t *__restrict__ val, const int32_t *__restrict__ off, int32_t V,
                        unsigned long long *out) {
  unsigned long long r = 0, e = 0;
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    const int32_t x = val[v];
    if (x >= 0 && x != INT_MAX) {
      ++r;
      e += off[v + 1] - off[v];
    }
  }
  for (int d = 16; d > 0; d >>= 1) {
    r += __shfl_xor_sync(0xffffffffu, r, d);
    e += __shfl_xor_sync(0xffffffffu, e, d);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(out, r);
    atomicAdd(out + 1, e);
  }
}

__global__ void k_sigma_to_reach(const double *__restrict__ sigma, int32_t V, int32_t *__restrict__ o) {
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
    o[v] = sigma[v] != 0.0 ? 0 : -1;
}

// vertices reached (val >= 0 and != INT_MAX) and the sum of their out-degrees.
gg_status reach_stats(gg_graph *g, const int32_t *val, gg_stats *st) {
  if (!st) return GG_OK;
  unsigned long long *d = reinterpret_cast<unsigned long long *>(g->d_misc + 32);
  GG_CUDA(cudaMemsetAsync(d, 0, 16, g->stream));
  { gg::note_launch(); k_reach<<<g->sm_count * 4, 256, 0, g->stream>>>(val, g->csr.off, g->csr.V, d); }
  GG_CUDA(cudaGetLastError());
  unsigned long long h[2];
  GG_CUDA(cudaMemcpyAsync(h, d, 16, cudaMemcpyDeviceToHost, g->stream));
  GG_CUDA(cudaStreamSynchronize(g->stream));
  st->vertices_reached = (int64_t)h[0];
  st->edges_traversed = (int64_t)h[1];
  return GG_OK;
}

// The schedule of one iteration: the learned selector's choice when the app
// schedule is GG_SCHED_LEARNED with a model (fallback s1 otherwise), else the
// simple / hybrid rule.  `f` may be NULL for rounds over every vertex.
struct Chooser {
  gg_graph *g;
  const gg_app_schedule *s;
  RunTotals rt{};
  gg_schedule learned{};
  gg_status choose(gg_frontier *f, int32_t n, const gg_schedule **out) {
    if (s->kind != GG_SCHED_LEARNED || !s->selector) {
      *out = pick(s, n, g->csr.V);
      return GG_OK;
    }
    FrontierStats fs;
    if (f) {
      GG_TRY(frontier_stats(g, f, &fs));
    } else {
      fs.n = g->csr.V;
      fs.sum_deg = g->csr.E;
    }
    float x[kSelectorFeatures];
    make_features(g, fs, rt, x);
    int32_t d[3];
    GG_TRY(selector_decide(const_cast<gg_selector *>(s->selector), x, d, g->stream));
    learned = candidate_schedule(s->s1, d[0], d[1], d[2]);
    *out = &learned;
    rt.visited_v = std::min<double>(g->csr.V, rt.visited_v + fs.n);
    rt.visited_e = std::min<double>(g->csr.E, rt.visited_e + fs.sum_deg);
    rt.iteration++;
    return GG_OK;
  }
};

// CUDA events around one trial (and, when a loop recorded ev2/ev3, around its
// traversal loop), plus the number of kernels the trial launched.
struct Trial {
  gg_graph *g;
  uint64_t l0;
  explicit Trial(gg_graph *gr) : g(gr), l0(launches()) {
    g->loop_timed = false;
    cudaEventRecord(g->ev0, g->stream);
  }
  gg_status stop(gg_stats *st) {
    GG_CUDA(cudaEventRecord(g->ev1, g->stream));
    GG_CUDA(cudaEventSynchronize(g->ev1));
    if (st) {
      GG_CUDA(cudaEventElapsedTime(&st->device_ms, g->ev0, g->ev1));
      if (g->loop_timed) GG_CUDA(cudaEventElapsedTime(&st->loop_ms, g->ev2, g->ev3));
      st->launches = (int32_t)(launches() - l0);
    }
    return GG_OK;
  }
};

// Brackets an unfused traversal loop with ev2/ev3.
struct LoopTimer {
  gg_graph *g;
  explicit LoopTimer(gg_graph *gr) : g(gr) { cudaEventRecord(g->ev2, g->stream); }
  ~LoopTimer() {
    cudaEventRecord(g->ev3, g->stream);
    g->loop_timed = true;
  }
};

gg_status check_app(gg_graph *g, const gg_app_schedule *s) {
  if (!g || !s) return set_error(GG_ERR_INVALID, "graph or schedule is NULL");
  if (s->kind != GG_SCHED_SIMPLE && s->kind != GG_SCHED_HYBRID && s->kind != GG_SCHED_LEARNED)
    return set_error(GG_ERR_INVALID, "bad schedule kind %d", s->kind);
  return GG_OK;
}

void count_dir(gg_stats *st, const gg_schedule *s) {
  if (!st) return;
  if (s->direction == GG_PUSH)
    st->push_iterations++;
  else
    st->pull_iterations++;
}

}  // namespace

gg_status app_reach_stats(gg_graph *g, const int32_t *val, gg_stats *st) { return reach_stats(g, val, st); }

gg_status scratch_get_app(gg_graph *g, int slot, size_t bytes, void **p) {
  Scratch &s = g->app[slot];
  if (s.bytes < bytes) {
    if (s.p) cudaFreeAsync(s.p, g->stream);
    s.p = nullptr;
    s.bytes = 0;
    GG_CUDA(dev_alloc(&s.p, bytes, g->stream));
    s.bytes = bytes;
  }
  *p = s.p;
  return GG_OK;
}

// Multi-source start: parent[s] = s, depth[s] = 0 (BFS) or dist[s] = 0 (SSSP)
// for every source, and the frontier queue holds the sources.
__global__ void k_seed_sources(int32_t sssp, VData d, const int32_t *__restrict__ srcs, int32_t n,
                               int32_t *__restrict__ q, int32_t *__restrict__ cnt) {
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int32_t s = srcs[i];
    if (sssp) {
      d.dist[s] = 0;
    } else {
      d.parent[s] = s;
      if (d.depth) d.depth[s] = 0;
    }
    q[i] = s;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *cnt = n;
}

gg_status seed_sources(gg_graph *g, gg_frontier *f, bool sssp, const VData &vd, const int32_t *srcs,
                       int32_t n) {
  int32_t *dsrc = nullptr;
  GG_TRY(scratch_get(g, 0, sizeof(int32_t) * ((size_t)std::max(n, 1) + (size_t)g->csr.V + 32),
                     (void **)&dsrc));
  GG_CUDA(cudaMemcpyAsync(dsrc, srcs, sizeof(int32_t) * n, cudaMemcpyDefault, g->stream));
  GG_CUDA(cudaMemsetAsync(f->cnt, 0, sizeof(int32_t) * 2, g->stream));
  note_launch();
  k_seed_sources<<<std::max(1, std::min(ceil_div(n, 256), 1024)), 256, 0, g->stream>>>(
      sssp, vd, dsrc, n, f->q_in, f->cnt_in);
  GG_CUDA(cudaGetLastError());
  f->fmt = GG_FMT_SPARSE;
  GG_CUDA(cudaStreamSynchronize(g->stream));  // dsrc is reused by the next scratch user
  return GG_OK;
}

// A fused BFS whose levels change direction (fused_bfs_do): a hybrid schedule
// of one push schedule the fused loop supports and one pull schedule (the
// rule), or a learned schedule with a network (its direction head; s1 pushes).
static bool bfs_do_plan(const gg_app_schedule *s, BfsDoPlan *p) {
  if (s->kind == GG_SCHED_HYBRID) {
    const bool p1 = s->s1.direction == GG_PULL, p2 = s->s2.direction == GG_PULL;
    if (p1 == p2) return false;
    p->push = p1 ? &s->s2 : &s->s1;
    if (!fused_supported(p->push) || p->push->cta_size > kBfsDoMaxCta) return false;
    p->mode = DO_RULE;
    p->threshold = s->threshold;
    p->small_pull = p1;
    return true;
  }
  if (s->kind == GG_SCHED_LEARNED && s->selector && fused_supported(&s->s1) && s->s1.cta_size <= kBfsDoMaxCta) {
    p->push = &s->s1;
    p->mode = DO_SELECTOR;
    p->sel = s->selector;
    return true;
  }
  return false;
}

gg_status run_bfs(gg_graph *g, const gg_app_schedule *s, const int32_t *srcs, int32_t nsrc,
                  int32_t *parent, int32_t *depth, gg_stats *st) {
  const int32_t V = g->csr.V;
  gg_frontier *f = nullptr;
  GG_TRY(app_frontier(g, &f));
  VData vd{};
  vd.parent = parent;
  vd.depth = depth;
  vd.src = nsrc == 1 ? srcs[0] : -1;
  GG_TRY(vertexset_apply_impl(g, nullptr, GG_VUDF_BFS_RESET, vd));  // reset + parent[src]=src
  if (nsrc == 1)
    GG_TRY(frontier_set_single(f, srcs[0]));
  else
    GG_TRY(seed_sources(g, f, false, vd, srcs, nsrc));
  if (s->fuse && s->kind == GG_SCHED_SIMPLE && fused_supported(&s->s1)) {
    bool ran = false;
    int32_t iters = 0;
    GG_TRY(fused_bfs(g, &s->s1, nsrc, vd, f, &iters, &ran));
    if (ran) {
      if (st) {
        st->iterations = iters;
        st->push_iterations = iters;
        st->fused = 1;
      }
      return check_device_error(g, "bfs");
    }
  }
  BfsDoPlan dp;
  if (s->fuse && bfs_do_plan(s, &dp)) {
    int32_t iters = 0, pulls = 0;
    GG_TRY(fused_bfs_do(g, dp, nsrc, vd, f, &iters, &pulls));
    if (st) {
      st->iterations = iters;
      st->pull_iterations = pulls;
      st->push_iterations = iters - pulls;
      st->fused = 1;
    }
    return check_device_error(g, "bfs");
  }
  LoopTimer lt(g);
  int32_t n = 1;
  Chooser ch{g, s};
  for (int32_t level = 1;; ++level) {
    GG_TRY(frontier_size(f, &n));
    if (n == 0) break;
    const gg_schedule *sc = nullptr;
    GG_TRY(ch.choose(f, n, &sc));
    vd.level = level;
    GG_TRY(edgeset_apply_impl(g, sc, GG_UDF_BFS_PARENT, GG_FILTER_PARENT_UNSET, f, f, true, vd,
                              INT_MAX, false));
    if (st) st->iterations++;
    count_dir(st, sc);
  }
  return check_device_error(g, "bfs");
}

gg_status run_sssp(gg_graph *g, const gg_app_schedule *s, const int32_t *srcs, int32_t nsrc,
                   int32_t delta, int32_t *dist, gg_stats *st) {
  const int32_t src = nsrc == 1 ? srcs[0] : -1;
  if (!g->app_pq) {
    GG_TRY(gg_pq_create(g, dist, 0, delta, src, &g->app_pq));
  }
  gg_pq *pq = g->app_pq;
  pq->prio = dist;
  GG_TRY(pq_reset(pq, 0, delta, src));  // pq.init(edges, SP, 0, delta, src)
  VData vd{};
  vd.dist = dist;
  vd.src = src;
  GG_TRY(vertexset_apply_impl(g, nullptr, GG_VUDF_SSSP_RESET, vd));  // reset + SP[src]=0
  if (nsrc > 1) GG_TRY(seed_sources(g, pq->frontier, true, vd, srcs, nsrc));
  if (s->fuse && s->kind == GG_SCHED_SIMPLE && fused_supported(&s->s1)) {
    bool ran = false;
    int32_t iters = 0;
    int64_t adv = 0;
    GG_TRY(fused_sssp(g, &s->s1, nsrc, delta, vd, pq, &iters, &adv, &ran));
    if (ran) {
      if (st) {
        st->iterations = iters;
        st->push_iterations = iters;
        st->bucket_advances = (int32_t)adv;
        st->fused = 1;
      }
      return check_device_error(g, "sssp");
    }
  }
  LoopTimer lt(g);
  Chooser ch{g, s};
  for (;;) {
    bool fin = false;
    GG_TRY(pq_finished(pq, &fin));
    if (fin) break;
    GG_TRY(pq_dequeue(pq));
    int32_t n = 0;
    GG_TRY(frontier_size(pq->frontier, &n));
    const gg_schedule *sc = nullptr;
    GG_TRY(ch.choose(pq->frontier, n, &sc));
    vd.far = pq_far(pq);
    GG_TRY(edgeset_apply_impl(g, sc, GG_UDF_SSSP_RELAX, GG_FILTER_NONE, pq->frontier, pq->frontier,
                              true, vd, pq_cutoff(pq), false));
    if (st) st->iterations++;
    count_dir(st, sc);
  }
  if (st) st->bucket_advances = (int32_t)pq->advances;
  return check_device_error(g, "sssp");
}

}  // namespace gg

using namespace gg;

extern "C" {

gg_status gg_bfs(gg_graph *g, const gg_app_schedule *s, int32_t src, int32_t *depth_out,
                 int32_t *parent_out, gg_stats *st) {
  GG_TRY(check_app(g, s));
  GG_CHECK_ARG(src >= 0 && src < g->csr.V, "source out of range");
  const int32_t V = g->csr.V;
  if (st) *st = gg_stats{};
  int32_t *parent = nullptr, *depth = nullptr;
  GG_TRY(app_array(g, 0, V, &parent));
  GG_TRY(app_array(g, 1, V, &depth));
  Trial t(g);
  GG_TRY(run_bfs(g, s, &src, 1, parent, depth, st));
  GG_TRY(t.stop(st));
  if (depth_out) GG_CUDA(cudaMemcpyAsync(depth_out, depth, sizeof(int32_t) * V, cudaMemcpyDefault, g->stream));
  if (parent_out) GG_CUDA(cudaMemcpyAsync(parent_out, parent, sizeof(int32_t) * V, cudaMemcpyDefault, g->stream));
  GG_TRY(reach_stats(g, depth, st));
  GG_CUDA(cudaStreamSynchronize(g->stream));
  return GG_OK;
}

// Training data of the fused direction-optimising BFS: the traversal from src
// with every level pushed (bfs.cpp's PUSH TWCE schedule), then with every
// level pulled, twice each.  A level's result does not depend on its
// direction, so level l starts from the same state in every run.
gg_status gg_bfs_collect_directions(gg_graph *g, int32_t src, int32_t max_rows, float *feats,
                                    float *times, int32_t *nrows) {
  GG_CHECK_ARG(g && feats && times && nrows && max_rows > 0, "bad arguments");
  GG_CHECK_ARG(src >= 0 && src < g->csr.V, "source out of range");
  const int32_t V = g->csr.V;
  *nrows = 0;
  int32_t *parent = nullptr, *depth = nullptr;
  GG_TRY(app_array(g, 0, V, &parent));
  GG_TRY(app_array(g, 1, V, &depth));
  gg_frontier *f = nullptr;
  GG_TRY(app_frontier(g, &f));
  gg_schedule push;
  gg_schedule_init(&push);
  push.load_balancing = GG_LB_TWCE;
  cudaStream_t st = g->stream;
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
    VData vd{};
    vd.parent = parent;
    vd.depth = depth;
    vd.src = src;
    BfsDoPlan p;
    p.push = &push;
    p.mode = dir ? DO_FORCE_PULL : DO_FORCE_PUSH;
    p.feat_log = dfeat;
    p.time_log = dtime;
    p.max_log = max_rows;
    int32_t lv = 0, pulls = 0;
    if ((status = vertexset_apply_impl(g, nullptr, GG_VUDF_BFS_RESET, vd)) != GG_OK ||
        (status = frontier_set_single(f, src)) != GG_OK ||
        (status = fused_bfs_do(g, p, 1, vd, f, &lv, &pulls)) != GG_OK ||
        (status = check_device_error(g, "bfs_collect_directions")) != GG_OK)
      break;
    if (levels >= 0 && lv != levels) {
      status = set_error(GG_ERR_STATE, "level counts differ between direction runs (%d, %d)", levels, lv);
      break;
    }
    levels = lv;
    const int32_t rows = std::min(levels, max_rows);
    if (cudaMemcpy(ht.data(), dtime, sizeof(unsigned long long) * ((size_t)rows + 1), cudaMemcpyDeviceToHost) !=
            cudaSuccess ||
        (rep == 0 && cudaMemcpy(feats, dfeat, sizeof(float) * kSelectorFeatures * (size_t)rows,
                                cudaMemcpyDeviceToHost) != cudaSuccess)) {
      status = set_error(GG_ERR_CUDA, "reading the direction timings failed");
      break;
    }
    for (int32_t l = 0; l < rows; ++l)
      best[2 * l + dir] = std::min(best[2 * l + dir], (float)((double)(ht[l + 1] - ht[l]) * 1e-6));
  }
  cudaFreeAsync(dfeat, st);
  cudaFreeAsync(dtime, st);
  GG_TRY(status);
  *nrows = std::min(levels, max_rows);
  for (int32_t i = 0; i < 2 * *nrows; ++i) times[i] = best[i];
  return GG_OK;
}

gg_status gg_sssp(gg_graph *g, const gg_app_schedule *s, int32_t src, int32_t delta,
                  int32_t *dist_out, gg_stats *st) {
  GG_TRY(check_app(g, s));
  GG_CHECK_ARG(src >= 0 && src < g->csr.V, "source out of range");
  GG_CHECK_ARG(delta >= 1, "delta must be >= 1");
  const int32_t V = g->csr.V;
  if (st) *st = gg_stats{};
  int32_t *dist = nullptr;
  GG_TRY(app_array(g, 2, V, &dist));
  Trial t(g);
  GG_TRY(run_sssp(g, s, &src, 1, delta, dist, st));
  GG_TRY(t.stop(st));
  if (dist_out) GG_CUDA(cudaMemcpyAsync(dist_out, dist, sizeof(int32_t) * V, cudaMemcpyDefault, g->stream));
  GG_TRY(reach_stats(g, dist, st));
  GG_CUDA(cudaStreamSynchronize(g->stream));
  return GG_OK;
}

// Multi-source traversals: every source starts at depth / distance 0 and the
// result is the distance to the nearest source.  On a disjoint union of graphs
// with one source per graph (gg_host_graph_union) this is each graph's own
// BFS / SSSP, computed for all graphs in one traversal.
gg_status gg_bfs_multi(gg_graph *g, const gg_app_schedule *s, const int32_t *sources, int32_t n,
                       int32_t *depth_out, int32_t *parent_out, gg_stats *st) {
  GG_TRY(check_app(g, s));
  GG_CHECK_ARG(sources && n >= 1, "need at least one source");
  const int32_t V = g->csr.V;
  for (int32_t i = 0; i < n; ++i) GG_CHECK_ARG(sources[i] >= 0 && sources[i] < V, "source out of range");
  if (st) *st = gg_stats{};
  int32_t *parent = nullptr, *depth = nullptr;
  GG_TRY(app_array(g, 0, V, &parent));
  GG_TRY(app_array(g, 1, V, &depth));
  Trial t(g);
  GG_TRY(run_bfs(g, s, sources, n, parent, depth, st));
  GG_TRY(t.stop(st));
  if (depth_out) GG_CUDA(cudaMemcpyAsync(depth_out, depth, sizeof(int32_t) * V, cudaMemcpyDefault, g->stream));
  if (parent_out) GG_CUDA(cudaMemcpyAsync(parent_out, parent, sizeof(int32_t) * V, cudaMemcpyDefault, g->stream));
  GG_TRY(reach_stats(g, depth, st));
  GG_CUDA(cudaStreamSynchronize(g->stream));
  return GG_OK;
}

gg_status gg_sssp_multi(gg_graph *g, const gg_app_schedule *s, const int32_t *sources, int32_t n,
                        int32_t delta, int32_t *dist_out, gg_stats *st) {
  GG_TRY(check_app(g, s));
  GG_CHECK_ARG(sources && n >= 1, "need at least one source");
  GG_CHECK_ARG(delta >= 1, "delta must be >= 1");
  const int32_t V = g->csr.V;
  for (int32_t i = 0; i < n; ++i) GG_CHECK_ARG(sources[i] >= 0 && sources[i] < V, "source out of range");
  if (st) *st = gg_stats{};
  int32_t *dist = nullptr;
  GG_TRY(app_array(g, 2, V, &dist));
  Trial t(g);
  GG_TRY(run_sssp(g, s, sources, n, delta, dist, st));
  GG_TRY(t.stop(st));
  if (dist_out) GG_CUDA(cudaMemcpyAsync(dist_out, dist, sizeof(int32_t) * V, cudaMemcpyDefault, g->stream));
  GG_TRY(reach_stats(g, dist, st));
  GG_CUDA(cudaStreamSynchronize(g->stream));
  return GG_OK;
}

gg_status gg_pagerank(gg_graph *g, const gg_app_schedule *s, int32_t iters, float damping,
                      float *rank_out, gg_stats *st) {
  GG_TRY(check_app(g, s));
  GG_CHECK_ARG(iters >= 0, "iterations must be >= 0");
  const int32_t V = g->csr.V;
  if (st) *st = gg_stats{};
  float *old_rank = nullptr, *new_rank = nullptr, *contrib = nullptr;
  if (s->kind == GG_SCHED_SIMPLE && s->s1.direction == GG_PULL && s->s1.load_balancing == GG_LB_TWC) {
    // static pull gather: in-degree bins once, one owner per vertex, no atomics
    GG_TRY(app_array(g, 3, V, &old_rank));
    GG_TRY(app_array(g, 5, 2 * (size_t)V, &contrib));
    Trial t(g);
    GG_TRY(pagerank_pull_twc(g, iters, damping, old_rank, contrib));
    GG_TRY(t.stop(st));
    GG_TRY(check_device_error(g, "pagerank"));
    if (rank_out) GG_CUDA(cudaMemcpyAsync(rank_out, old_rank, sizeof(float) * V, cudaMemcpyDefault, g->stream));
    if (st) {
      st->iterations = iters;
      st->pull_iterations = iters;
      st->vertices_reached = V;
      st->edges_traversed = (int64_t)g->csr.E * iters;
    }
    GG_CUDA(cudaStreamSynchronize(g->stream));
    return GG_OK;
  }
  GG_TRY(app_array(g, 3, V, &old_rank));
  GG_TRY(app_array(g, 4, V, &new_rank));
  GG_TRY(app_array(g, 5, V, &contrib));
  VData vd{};
  vd.old_rank = old_rank;
  vd.new_rank = new_rank;
  vd.contrib = contrib;
  vd.damping = damping;
  Trial t(g);
  GG_TRY(vertexset_apply_impl(g, nullptr, GG_VUDF_PR_RESET, vd));
  for (int32_t i = 0; i < iters; ++i) {
    const gg_schedule *sc = pick(s, V, V);
    GG_TRY(vertexset_apply_impl(g, nullptr, GG_VUDF_PR_CONTRIB, vd));
    GG_TRY(edgeset_apply_impl(g, sc, GG_UDF_PR_ADD, GG_FILTER_NONE, nullptr, nullptr, true, vd,
                              INT_MAX, false));
    GG_TRY(vertexset_apply_impl(g, nullptr, GG_VUDF_PR_UPDATE, vd));
    if (st) st->iterations++;
    count_dir(st, sc);
  }
  GG_TRY(t.stop(st));
  GG_TRY(check_device_error(g, "pagerank"));
  if (rank_out) GG_CUDA(cudaMemcpyAsync(rank_out, old_rank, sizeof(float) * V, cudaMemcpyDefault, g->stream));
  if (st) {
    st->vertices_reached = V;
    st->edges_traversed = (int64_t)g->csr.E * iters;
  }
  GG_CUDA(cudaStreamSynchronize(g->stream));
  return GG_OK;
}

gg_status gg_cc(gg_graph *g, const gg_app_schedule *s, int32_t *labels_out, gg_stats *st) {
  GG_TRY(check_app(g, s));
  const int32_t V = g->csr.V;
  if (st) *st = gg_stats{};
  int32_t *ids = nullptr, *updates = nullptr;
  GG_TRY(app_array(g, 0, V, &ids));
  if (s->fuse && s->kind == GG_SCHED_SIMPLE) {
    // the whole computation fused into one edge pass (cc_uf.cu): same labels
    int32_t *parent = nullptr;
    GG_TRY(app_array(g, 2, V, &parent));
    Trial t(g);
    GG_TRY(cc_union_find(g, ids, parent));
    GG_TRY(t.stop(st));
    GG_TRY(check_device_error(g, "cc"));
    if (labels_out) GG_CUDA(cudaMemcpyAsync(labels_out, ids, sizeof(int32_t) * V, cudaMemcpyDefault, g->stream));
    if (st) {
      st->iterations = 1;
      st->fused = 1;
      st->vertices_reached = V;
      st->edges_traversed = (int64_t)g->csr.E;
    }
    GG_CUDA(cudaStreamSynchronize(g->stream));
    return GG_OK;
  }
  GG_TRY(app_array(g, 1, 2, &updates));
  VData vd{};
  vd.ids = ids;
  vd.updates = updates;
  int32_t *hu = g->h_pinned + 20;
  Trial t(g);
  GG_TRY(vertexset_apply_impl(g, nullptr, GG_VUDF_CC_INIT, vd));
  hu[0] = 1;
  int32_t rounds = 0;
  Chooser ch{g, s};
  while (hu[0]) {  // while (updates[0])
    GG_CUDA(cudaMemsetAsync(updates, 0, sizeof(int32_t), g->stream));
    const gg_schedule *sc = nullptr;
    GG_TRY(ch.choose(nullptr, V, &sc));
    GG_TRY(edgeset_apply_impl(g, sc, GG_UDF_CC_HOOK, GG_FILTER_NONE, nullptr, nullptr, true, vd,
                              INT_MAX, false));
    count_dir(st, sc);
    ++rounds;
    hu[1] = 1;
    while (hu[1]) {  // pointer jumping until stable
      GG_CUDA(cudaMemsetAsync(updates + 1, 0, sizeof(int32_t), g->stream));
      GG_TRY(vertexset_apply_impl(g, nullptr, GG_VUDF_CC_PJUMP, vd));
      GG_CUDA(cudaMemcpyAsync(hu, updates, sizeof(int32_t) * 2, cudaMemcpyDeviceToHost, g->stream));
      GG_CUDA(cudaStreamSynchronize(g->stream));
    }
  }
  GG_TRY(t.stop(st));
  GG_TRY(check_device_error(g, "cc"));
  if (labels_out) GG_CUDA(cudaMemcpyAsync(labels_out, ids, sizeof(int32_t) * V, cudaMemcpyDefault, g->stream));
  if (st) {
    st->iterations = rounds;
    st->vertices_reached = V;
    st->edges_traversed = (int64_t)g->csr.E;
  }
  GG_CUDA(cudaStreamSynchronize(g->stream));
  return GG_OK;
}

gg_status gg_bc(gg_graph *g, const gg_app_schedule *s, int32_t src, float *dep_out, gg_stats *st) {
  GG_TRY(check_app(g, s));
  GG_CHECK_ARG(src >= 0 && src < g->csr.V, "source out of range");
  const int32_t V = g->csr.V;
  if (st) *st = gg_stats{};
  double *sigma = nullptr;
  float *dep = nullptr;
  uint8_t *visited = nullptr;
  double *dep64 = nullptr;
  GG_TRY(app_array(g, 6, V, &sigma));
  GG_TRY(app_array(g, 5, V, &dep));
  GG_TRY(app_array(g, 3, V, &dep64));
  GG_TRY(app_array(g, 7, V, &visited));
  gg_frontier *f = nullptr;
  GG_TRY(app_frontier(g, &f));
  if (!g->app_list) GG_TRY(gg_frontier_list_create(g, &g->app_list));
  gg_frontier_list *l = g->app_list;
  l->level_start.assign(1, 0);
  VData vd{};
  vd.num_paths = sigma;
  vd.dependences = dep;
  // fp32 atomic accumulation (the reference's float dependences) drifts past
  // 1e-6 relative L1 on R-MAT hubs; accumulate in fp64, store fp32 at the end.
  vd.dep64 = dep64;
  vd.visited = visited;
  vd.src = src;
  Trial t(g);
  GG_TRY(vertexset_apply_impl(g, nullptr, GG_VUDF_BC_RESET, vd));  // + num_paths[src]=1, visited[src]=1
  GG_TRY(frontier_set_single(f, src));
  int32_t round = 0;
  GG_TRY(gg_frontier_list_insert(l, f));
  for (;;) {  // forward sweep
    int32_t n = 0;
    GG_TRY(frontier_size(f, &n));
    if (n == 0) break;
    ++round;
    const gg_schedule *sc = pick(s, n, V);
    GG_TRY(edgeset_apply_impl(g, sc, GG_UDF_BC_FORWARD, GG_FILTER_UNVISITED, f, f, false, vd,
                              INT_MAX, false));
    GG_TRY(vertexset_apply_impl(g, f, GG_VUDF_BC_MARK_VISITED, vd));
    GG_TRY(gg_frontier_list_insert(l, f));
    count_dir(st, sc);
  }
  GG_TRY(vertexset_apply_impl(g, nullptr, GG_VUDF_BC_MARK_UNVISITED, vd));
  GG_TRY(gg_frontier_list_retrieve(l, f));
  GG_TRY(gg_frontier_list_retrieve(l, f));
  GG_TRY(vertexset_apply_impl(g, f, GG_VUDF_BC_BACKWARD_VERTEX, vd));
  const int32_t levels = round;
  round = round - 1;
  while (round > 0) {  // backward sweep
    int32_t n = 0;
    GG_TRY(frontier_size(f, &n));
    const gg_schedule *sc = pick(s, n, V);
    GG_TRY(edgeset_apply_impl(g, sc, GG_UDF_BC_BACKWARD, GG_FILTER_UNVISITED, f, nullptr, true, vd,
                              INT_MAX, false));
    GG_TRY(gg_frontier_list_retrieve(l, f));
    GG_TRY(vertexset_apply_impl(g, f, GG_VUDF_BC_BACKWARD_VERTEX, vd));
    count_dir(st, sc);
    round = round - 1;
  }
  GG_TRY(vertexset_apply_impl(g, nullptr, GG_VUDF_BC_FINAL, vd));
  GG_TRY(t.stop(st));
  GG_TRY(check_device_error(g, "bc"));
  if (dep_out) GG_CUDA(cudaMemcpyAsync(dep_out, dep, sizeof(float) * V, cudaMemcpyDefault, g->stream));
  if (st) {
    st->iterations = levels;
    int32_t *tmp = nullptr;
    GG_TRY(app_array(g, 0, V, &tmp));
    { gg::note_launch(); k_sigma_to_reach<<<g->sm_count * 4, 256, 0, g->stream>>>(sigma, V, tmp); }
    GG_CUDA(cudaGetLastError());
    GG_TRY(reach_stats(g, tmp, st));
    st->edges_traversed *= 2;  // forward + backward sweeps
  }
  GG_CUDA(cudaStreamSynchronize(g->stream));
  return GG_OK;
}

}  // extern "C"
