// Data side of the learned schedule selector.
//  - frontier statistics (count, degree sum / sum of squares / max) on the GPU;
//  - the 12 features the network reads;
//  - gg_selector_collect: training data generated by the engine itself.  It
//    follows a run with the fallback schedule and, at every iteration, snapshots
//    the app state, times each of the 36 candidate schedules on that same
//    state (restoring it in between), and records features and timings.
#include <cmath>
#include <vector>

#include "selector.h"

namespace gg {

gg_schedule candidate_schedule(const gg_schedule &base, int dir, int lb, int fr) {
  gg_schedule s = base;
  s.direction = dir ? GG_PULL : GG_PUSH;
  s.load_balancing = kLbChoices[lb];
  s.frontier_creation = fr;
  s.pull_frontier_rep = fr == GG_FC_BOOLMAP ? GG_PULL_BOOLMAP : GG_PULL_BITMAP;
  s.edge_blocking = GG_UNBLOCKED;
  return s;
}

__global__ void k_frontier_stats(const int32_t *__restrict__ q, const int32_t *__restrict__ n_dev,
                                 const int32_t *__restrict__ off, unsigned long long *acc) {
  const int32_t n = *n_dev;
  unsigned long long s1 = 0, s2 = 0, mx = 0;
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int32_t v = q[i];
    const unsigned long long d = (unsigned long long)(off[v + 1] - off[v]);
    s1 += d;
    s2 += d * d;
    mx = d > mx ? d : mx;
  }
  for (int k = 16; k > 0; k >>= 1) {
    s1 += __shfl_xor_sync(0xffffffffu, s1, k);
    s2 += __shfl_xor_sync(0xffffffffu, s2, k);
    const unsigned long long o = __shfl_xor_sync(0xffffffffu, mx, k);
    mx = o > mx ? o : mx;
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(acc, s1);
    atomicAdd(acc + 1, s2);
    atomicMax(acc + 2, mx);
  }
}

gg_status frontier_stats(gg_graph *g, gg_frontier *f, FrontierStats *fs) {
  GG_TRY(frontier_prepare_sparse(f));
  unsigned long long *acc = reinterpret_cast<unsigned long long *>(g->d_misc + 56);
  GG_CUDA(cudaMemsetAsync(acc, 0, 24, g->stream));
  note_launch();
  k_frontier_stats<<<g->sm_count * 2, 256, 0, g->stream>>>(f->q_in, f->cnt_in, g->csr.off, acc);
  GG_CUDA(cudaGetLastError());
  unsigned long long h[3];
  int32_t n = 0;
  GG_CUDA(cudaMemcpyAsync(h, acc, 24, cudaMemcpyDeviceToHost, g->stream));
  GG_CUDA(cudaMemcpyAsync(&n, f->cnt_in, sizeof(int32_t), cudaMemcpyDeviceToHost, g->stream));
  GG_CUDA(cudaStreamSynchronize(g->stream));
  fs->n = n;
  fs->sum_deg = (double)h[0];
  fs->sum_deg2 = (double)h[1];
  fs->max_deg = (double)h[2];
  return GG_OK;
}

// Features: log-scaled frontier size and edges, unvisited vertices and edges,
// frontier degree mean / max / variance, iteration index, graph size, and the
// frontier's share of V and E.
void make_features(const gg_graph *g, const FrontierStats &fs, const RunTotals &rt,
                   float x[kSelectorFeatures]) {
  const double V = g->csr.V, E = std::max(1, g->csr.E);
  const double n = fs.n, mean = n > 0 ? fs.sum_deg / n : 0.0;
  const double var = n > 0 ? std::max(0.0, fs.sum_deg2 / n - mean * mean) : 0.0;
  const double uv = std::max(0.0, V - rt.visited_v), ue = std::max(0.0, E - rt.visited_e);
  x[0] = (float)(std::log2(1 + n) / 32);
  x[1] = (float)(std::log2(1 + fs.sum_deg) / 32);
  x[2] = (float)(std::log2(1 + uv) / 32);
  x[3] = (float)(std::log2(1 + ue) / 32);
  x[4] = (float)(std::log2(1 + mean) / 16);
  x[5] = (float)(std::log2(1 + fs.max_deg) / 32);
  x[6] = (float)(std::log2(1 + var) / 64);
  x[7] = (float)(std::min(rt.iteration, 256) / 256.0);
  x[8] = (float)(std::log2(V) / 32);
  x[9] = (float)(std::log2(1 + E) / 32);
  x[10] = (float)(n / V);
  x[11] = (float)(fs.sum_deg / E);
}

namespace {

// Device-side copy of an app's mutable state for snapshot/restore.
struct Snapshot {
  std::vector<std::pair<void *, size_t>> arrays;  // (live pointer, bytes)
  std::vector<void *> copies;
  gg_frontier fcopy;
  int32_t *q = nullptr;
  int32_t n = 0;
  gg_status take(gg_graph *g, gg_frontier *f, int32_t n_) {
    n = n_;
    cudaStream_t st = g->stream;
    if (copies.empty()) {
      for (auto &a : arrays) {
        void *p = nullptr;
        GG_CUDA(cudaMalloc(&p, a.second));
        copies.push_back(p);
      }
      GG_CUDA(cudaMalloc(&q, sizeof(int32_t) * (size_t)g->csr.V * 6 + 64));
    }
    for (size_t i = 0; i < arrays.size(); ++i)
      GG_CUDA(cudaMemcpyAsync(copies[i], arrays[i].first, arrays[i].second, cudaMemcpyDeviceToDevice, st));
    GG_CUDA(cudaMemcpyAsync(q, f->q_in, sizeof(int32_t) * (size_t)std::max(n, 1), cudaMemcpyDeviceToDevice, st));
    fcopy = *f;
    return GG_OK;
  }
  gg_status restore(gg_graph *g, gg_frontier *f) {
    cudaStream_t st = g->stream;
    *f = fcopy;
    for (size_t i = 0; i < arrays.size(); ++i)
      GG_CUDA(cudaMemcpyAsync(arrays[i].first, copies[i], arrays[i].second, cudaMemcpyDeviceToDevice, st));
    GG_CUDA(cudaMemcpyAsync(f->q_in, q, sizeof(int32_t) * (size_t)std::max(n, 1), cudaMemcpyDeviceToDevice, st));
    g->h_pinned[12] = n;
    GG_CUDA(cudaMemcpyAsync(f->cnt_in, g->h_pinned + 12, sizeof(int32_t), cudaMemcpyHostToDevice, st));
    f->fmt = GG_FMT_SPARSE;
    GG_CUDA(cudaStreamSynchronize(st));
    return GG_OK;
  }
  ~Snapshot() {
    for (void *p : copies) cudaFree(p);
    if (q) cudaFree(q);
  }
};

template <class Apply>
gg_status time_candidates(gg_graph *g, gg_frontier *f, Snapshot &snap, const gg_schedule &base, bool any_frontier,
                          Apply apply, float *times) {
  for (int c = 0; c < kCandidates; ++c) {
    const int dir = c / (3 * kNumLb), lb = (c / 3) % kNumLb, fr = c % 3;
    if (!any_frontier && fr != 0) {
      times[c] = times[c - fr];  // the frontier type does not matter here
      continue;
    }
    const gg_schedule sc = candidate_schedule(base, dir, lb, fr);
    float best = INFINITY;
    for (int rep = 0; rep < 2; ++rep) {  // the first run pays one-off scratch growth
      GG_TRY(snap.restore(g, f));
      GG_CUDA(cudaEventRecord(g->ev2, g->stream));
      const gg_status s = apply(sc);
      GG_CUDA(cudaEventRecord(g->ev3, g->stream));
      GG_CUDA(cudaEventSynchronize(g->ev3));
      float ms = 0;
      cudaEventElapsedTime(&ms, g->ev2, g->ev3);
      if (s != GG_OK) {
        clear_error();
        ms = INFINITY;
      }
      best = std::min(best, ms);
    }
    times[c] = best;
  }
  return snap.restore(g, f);
}

}  // namespace
}  // namespace gg

using namespace gg;

extern "C" gg_status gg_selector_collect(gg_graph *g, int32_t app, int32_t src, int32_t delta,
                                         int32_t max_rows, float *feats, float *times, int32_t *nrows) {
  GG_CHECK_ARG(g && feats && times && nrows && max_rows > 0, "bad arguments");
  GG_CHECK_ARG(app >= GG_SEL_BFS && app <= GG_SEL_CC, "unknown app");
  GG_CHECK_ARG(app == GG_SEL_CC || (src >= 0 && src < g->csr.V), "source out of range");
  const int32_t V = g->csr.V;
  *nrows = 0;
  GG_TRY(ensure_transpose(g));  // pull candidates must not pay it inside the timed region
  gg_schedule base;
  gg_schedule_init(&base);
  base.load_balancing = GG_LB_TWCE;
  RunTotals rt;
  VData vd{};
  Snapshot snap;
  gg_frontier *f = nullptr;
  if (app == GG_SEL_BFS) {
    int32_t *parent = nullptr, *depth = nullptr;
    GG_TRY(scratch_get_app(g, 0, sizeof(int32_t) * V, (void **)&parent));
    GG_TRY(scratch_get_app(g, 1, sizeof(int32_t) * V, (void **)&depth));
    if (!g->app_frontier) GG_TRY(gg_frontier_create(g, 0, &g->app_frontier));
    f = g->app_frontier;
    vd.parent = parent;
    vd.depth = depth;
    vd.src = src;
    GG_TRY(vertexset_apply_impl(g, nullptr, GG_VUDF_BFS_RESET, vd));
    GG_CUDA(cudaMemsetAsync(f->cnt, 0, sizeof(int32_t) * 2, g->stream));
    g->h_pinned[13] = src;
    g->h_pinned[14] = 1;
    GG_CUDA(cudaMemcpyAsync(f->q_in, g->h_pinned + 13, 4, cudaMemcpyHostToDevice, g->stream));
    GG_CUDA(cudaMemcpyAsync(f->cnt_in, g->h_pinned + 14, 4, cudaMemcpyHostToDevice, g->stream));
    f->fmt = GG_FMT_SPARSE;
    snap.arrays = {{parent, sizeof(int32_t) * (size_t)V}, {depth, sizeof(int32_t) * (size_t)V}};
    for (int32_t level = 1; *nrows < max_rows; ++level) {
      FrontierStats fs;
      GG_TRY(frontier_stats(g, f, &fs));
      if (fs.n == 0) break;
      make_features(g, fs, rt, feats + (size_t)*nrows * kSelectorFeatures);
      GG_TRY(snap.take(g, f, (int32_t)fs.n));
      vd.level = level;
      auto apply = [&](const gg_schedule &sc) {
        return edgeset_apply_impl(g, &sc, GG_UDF_BFS_PARENT, GG_FILTER_PARENT_UNSET, f, f, true, vd,
                                  INT_MAX, false);
      };
      GG_TRY(time_candidates(g, f, snap, base, true, apply, times + (size_t)*nrows * kCandidates));
      GG_TRY(apply(base));
      rt.visited_v += fs.n;
      rt.visited_e += fs.sum_deg;
      rt.iteration++;
      ++*nrows;
    }
  } else if (app == GG_SEL_SSSP) {
    GG_CHECK_ARG(delta >= 1, "delta must be >= 1");
    int32_t *dist = nullptr;
    GG_TRY(scratch_get_app(g, 2, sizeof(int32_t) * V, (void **)&dist));
    if (!g->app_pq) GG_TRY(gg_pq_create(g, dist, 0, delta, src, &g->app_pq));
    gg_pq *pq = g->app_pq;
    pq->prio = dist;
    GG_TRY(pq_reset(pq, 0, delta, src));
    vd.dist = dist;
    vd.src = src;
    GG_TRY(vertexset_apply_impl(g, nullptr, GG_VUDF_SSSP_RESET, vd));
    f = pq->frontier;
    snap.arrays = {{dist, sizeof(int32_t) * (size_t)V}};
    while (*nrows < max_rows) {
      bool fin = false;
      GG_TRY(pq_finished(pq, &fin));
      if (fin) break;
      GG_TRY(pq_dequeue(pq));
      FrontierStats fs;
      GG_TRY(frontier_stats(g, f, &fs));
      make_features(g, fs, rt, feats + (size_t)*nrows * kSelectorFeatures);
      GG_TRY(snap.take(g, f, (int32_t)fs.n));
      const int32_t cutoff = pq_cutoff(pq);
      auto apply = [&](const gg_schedule &sc) {
        return edgeset_apply_impl(g, &sc, GG_UDF_SSSP_RELAX, GG_FILTER_NONE, f, f, true, vd, cutoff, false);
      };
      GG_TRY(time_candidates(g, f, snap, base, true, apply, times + (size_t)*nrows * kCandidates));
      // candidates are timed without parking far improvements (the same for
      // all of them, and nothing to restore); the step that moves the run on
      // parks them so the queue's next advance finds them
      VData vf = vd;
      vf.far = pq_far(pq);
      GG_TRY(edgeset_apply_impl(g, &base, GG_UDF_SSSP_RELAX, GG_FILTER_NONE, f, f, true, vf, cutoff, false));
      rt.visited_v = std::min<double>(V, rt.visited_v + fs.n);
      rt.visited_e = std::min<double>(g->csr.E, rt.visited_e + fs.sum_deg);
      rt.iteration++;
      ++*nrows;
    }
  } else {  // CC hook rounds over every vertex
    int32_t *ids = nullptr, *updates = nullptr;
    GG_TRY(scratch_get_app(g, 0, sizeof(int32_t) * V, (void **)&ids));
    GG_TRY(scratch_get_app(g, 1, sizeof(int32_t) * 2, (void **)&updates));
    if (!g->app_frontier) GG_TRY(gg_frontier_create(g, 0, &g->app_frontier));
    f = g->app_frontier;
    vd.ids = ids;
    vd.updates = updates;
    GG_TRY(vertexset_apply_impl(g, nullptr, GG_VUDF_CC_INIT, vd));
    snap.arrays = {{ids, sizeof(int32_t) * (size_t)V}, {updates, sizeof(int32_t) * 2}};
    FrontierStats fs;
    fs.n = V;
    fs.sum_deg = g->csr.E;
    fs.max_deg = 0;
    int32_t *hu = g->h_pinned + 20;
    hu[0] = 1;
    while (hu[0] && *nrows < max_rows) {
      GG_CUDA(cudaMemsetAsync(updates, 0, sizeof(int32_t) * 2, g->stream));
      make_features(g, fs, rt, feats + (size_t)*nrows * kSelectorFeatures);
      GG_TRY(snap.take(g, f, 0));
      auto apply = [&](const gg_schedule &sc) {
        return edgeset_apply_impl(g, &sc, GG_UDF_CC_HOOK, GG_FILTER_NONE, nullptr, nullptr, true, vd, INT_MAX,
                                  false);
      };
      GG_TRY(time_candidates(g, f, snap, base, false, apply, times + (size_t)*nrows * kCandidates));
      gg_schedule eo = base;
      eo.load_balancing = GG_LB_EDGE_ONLY;
      GG_TRY(apply(eo));
      rt.iteration++;
      ++*nrows;
      hu[1] = 1;
      while (hu[1]) {
        GG_CUDA(cudaMemsetAsync(updates + 1, 0, sizeof(int32_t), g->stream));
        GG_TRY(vertexset_apply_impl(g, nullptr, GG_VUDF_CC_PJUMP, vd));
        GG_CUDA(cudaMemcpyAsync(hu, updates, sizeof(int32_t) * 2, cudaMemcpyDeviceToHost, g->stream));
        GG_CUDA(cudaStreamSynchronize(g->stream));
      }
    }
  }
  return check_device_error(g, "selector_collect");
}
