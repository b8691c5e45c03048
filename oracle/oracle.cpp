// ORACLE -- test infrastructure only.
//
// CPU restatement of the easy_graphit apps (apps/bfs.cpp, sssp.cpp, pr.cpp,
// cc.cpp, bc.cpp) and of the runtime algorithms they drive, used to check the
// GPU engine.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
// legs load this library; the engine (libgg.so) never does.
//
// Pinning: the reference ships no tests or golden vectors.  tests/golden holds
// fixtures produced by the reference's own code compiled here (oracle/_ref,
// built from runtime/infra_gapbs by oracle/Makefile): GAPBS-built graphs and
// GAPBS's OrderedProcessingOperatorNoMerge SSSP distances, weighted and with
// unit weights (= BFS depths), and the outputs of the reference's five apps
// themselves (apps/*.cpp compiled against oracle/app_shim, a host-execution
// stand-in for the absent BuildIt staging library, by `make -C oracle apps`).
// Every function below is checked against those (tests/test_oracle.py), besides
// hand-computed known answers on tiny graphs.
#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <queue>
#include <random>
#include <utility>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct Csr {
  int32_t V;
  const int32_t *off, *dst, *w;
};

// In-neighbour CSR (CSC) of a CSR graph.
void transpose(int32_t V, const int32_t *off, const int32_t *dst,
               std::vector<int32_t> &toff, std::vector<int32_t> &tsrc) {
  const int64_t E = off[V];
  toff.assign(V + 1, 0);
  for (int64_t e = 0; e < E; ++e) toff[dst[e] + 1]++;
  for (int32_t v = 0; v < V; ++v) toff[v + 1] += toff[v];
  std::vector<int32_t> pos(toff.begin(), toff.end() - 1);
  tsrc.resize(E);
  for (int32_t u = 0; u < V; ++u)
    for (int32_t k = off[u]; k < off[u + 1]; ++k) tsrc[pos[dst[k]]++] = u;
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------- BFS
// apps/bfs.cpp:36-62 with the push operator of operators.cpp:550-576:
// the frontier starts as {src}; every edge (u,v) with parent[v] == -1 sets
// parent[v] = u and enqueues v.  The level at which v is first reached is its
// depth; depths are schedule-invariant, parents are not.
void orc_bfs(int32_t V, const int32_t *off, const int32_t *dst, int32_t src,
             int32_t *depth) {
  for (int32_t v = 0; v < V; ++v) depth[v] = -1;
  if (src < 0 || src >= V) return;
  std::vector<int32_t> cur{src}, next;
  depth[src] = 0;
  for (int32_t level = 1; !cur.empty(); ++level) {
    next.clear();
    for (int32_t u : cur)
      for (int32_t k = off[u]; k < off[u + 1]; ++k)
        if (depth[dst[k]] == -1) {
          depth[dst[k]] = level;
          next.push_back(dst[k]);
        }
    cur.swap(next);
  }
}

// Counts vertices whose parent entry is inconsistent with a BFS tree of the
// given depths: parent[src] == src; a reached v != src needs an edge
// (parent[v], v) with depth[parent[v]] == depth[v]-1; unreached v needs -1.
int64_t orc_bfs_check_parent(int32_t V, const int32_t *off, const int32_t *dst,
                             int32_t src, const int32_t *depth,
                             const int32_t *parent) {
  int64_t bad = 0;
  for (int32_t v = 0; v < V; ++v) {
    if (depth[v] < 0) {
      bad += parent[v] != -1;
      continue;
    }
    if (v == src) {
      bad += parent[v] != src;
      continue;
    }
    const int32_t p = parent[v];
    if (p < 0 || p >= V || depth[p] != depth[v] - 1) {
      ++bad;
      continue;
    }
    bool edge = std::binary_search(dst + off[p], dst + off[p + 1], v);
    if (!edge)
      for (int32_t k = off[p]; k < off[p + 1] && !edge; ++k) edge = dst[k] == v;
    bad += !edge;
  }
  return bad;
}

// Level-synchronous OpenMP BFS (CPU baseline; no reference CPU BFS exists).
void orc_bfs_omp(int32_t V, const int32_t *off, const int32_t *dst, int32_t src,
                 int32_t *depth, int32_t nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  std::vector<std::atomic<int32_t>> d(V);
#pragma omp parallel for schedule(static)
  for (int32_t v = 0; v < V; ++v) d[v].store(-1, std::memory_order_relaxed);
  std::vector<int32_t> cur{src}, next(V);
  d[src].store(0);
  std::atomic<int64_t> tail{0};
  for (int32_t level = 1; !cur.empty(); ++level) {
    tail.store(0);
#pragma omp parallel
    {
      std::vector<int32_t> local;
#pragma omp for schedule(dynamic, 64) nowait
      for (int64_t i = 0; i < (int64_t)cur.size(); ++i) {
        const int32_t u = cur[i];
        for (int32_t k = off[u]; k < off[u + 1]; ++k) {
          int32_t expect = -1;
          if (d[dst[k]].load(std::memory_order_relaxed) == -1 &&
              d[dst[k]].compare_exchange_strong(expect, level))
            local.push_back(dst[k]);
        }
      }
      const int64_t at = tail.fetch_add((int64_t)local.size());
      std::copy(local.begin(), local.end(), next.begin() + at);
    }
    cur.assign(next.begin(), next.begin() + tail.load());
  }
#pragma omp parallel for schedule(static)
  for (int32_t v = 0; v < V; ++v) depth[v] = d[v].load(std::memory_order_relaxed);
}

// --------------------------------------------------------------- SSSP
// Dijkstra with a binary heap: exact int32 distances, INT_MAX if unreached.
void orc_sssp_dijkstra(int32_t V, const int32_t *off, const int32_t *dst,
                       const int32_t *w, int32_t src, int32_t *dist) {
  for (int32_t v = 0; v < V; ++v) dist[v] = INT_MAX;
  if (src < 0 || src >= V) return;
  typedef std::pair<int64_t, int32_t> Item;
  std::priority_queue<Item, std::vector<Item>, std::greater<Item>> pq;
  dist[src] = 0;
  pq.push({0, src});
  while (!pq.empty()) {
    const Item it = pq.top();
    pq.pop();
    if (it.first != dist[it.second]) continue;
    const int32_t u = it.second;
    for (int32_t k = off[u]; k < off[u + 1]; ++k) {
      const int64_t nd = it.first + w[k];
      if (nd < dist[dst[k]]) {
        dist[dst[k]] = (int32_t)nd;
        pq.push({nd, dst[k]});
      }
    }
  }
}

// Sequential restatement of the GPU delta-stepping loop (apps/sssp.cpp:47-52,
// GPUPriorityQueue::finished/dequeueReadySet gpu_priority_queue.h:63-153,
// update_nodes_identify_min / update_nodes_special :250-288, and
// PriorityQueue::updatePriorityMin graphit_types.h:426-430).
// Returns the number of bucket advances.
int64_t orc_sssp_delta_gpu(int32_t V, const int32_t *off, const int32_t *dst,
                           const int32_t *w, int32_t src, int32_t delta,
                           int32_t *dist) {
  for (int32_t v = 0; v < V; ++v) dist[v] = INT_MAX;
  if (src < 0 || src >= V || delta < 1) return 0;
  dist[src] = 0;
  int64_t cur = 0;
  int64_t cutoff = cur + delta;
  bool ready_set_dequeued = false;
  std::vector<int32_t> frontier{src}, next;
  int64_t advances = 0;
  auto dequeue_ready_set = [&]() {
    const int64_t window_upper = cur + delta;
    int64_t m = INT_MAX;
    for (int32_t v = 0; v < V; ++v)
      if (dist[v] >= window_upper && dist[v] != INT_MAX && dist[v] < m) m = dist[v];
    cur = m;
    frontier.clear();
    if (cur != INT_MAX)
      for (int32_t v = 0; v < V; ++v)
        if (dist[v] >= cur && dist[v] < cur + delta) frontier.push_back(v);
    cutoff = cur + delta;
    ++advances;
  };
  for (;;) {
    // finished()
    if (cur == INT_MAX) break;
    if (!ready_set_dequeued && frontier.empty()) {
      dequeue_ready_set();
      ready_set_dequeued = true;
      if (cur == INT_MAX) break;
    }
    // dequeue()
    if (ready_set_dequeued)
      ready_set_dequeued = false;
    else if (frontier.empty())
      dequeue_ready_set();
    // edgeset_apply(...).apply_priority(edges, updateEdge, pq)
    next.clear();
    for (int32_t u : frontier)
      for (int32_t k = off[u]; k < off[u + 1]; ++k) {
        const int64_t np = (int64_t)dist[u] + w[k];
        if (np < dist[dst[k]]) {
          dist[dst[k]] = (int32_t)np;
          if (np < cutoff) next.push_back(dst[k]);
        }
      }
    frontier.swap(next);
  }
  return advances;
}

// OpenMP port of GAPBS's OrderedProcessingOperatorNoMerge with the
// updatePriorityMin edge function (infra_gapbs/ordered_processing.h:15-143,
// eager_priority_queue.h:17-62): thread-local bins indexed by dist/delta, a
// shared frontier, and a per-round minimum-bin election.  This is the
// reference's CPU SSSP; used as the timed CPU baseline.
void orc_sssp_ordered(int32_t V, const int32_t *off, const int32_t *dst,
                      const int32_t *w, int32_t src, int32_t delta,
                      int32_t *dist_out, int32_t nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  const size_t kMaxBin = std::numeric_limits<size_t>::max() / 2;
  std::vector<std::atomic<int32_t>> P(V);
#pragma omp parallel for schedule(static)
  for (int32_t v = 0; v < V; ++v) P[v].store(INT_MAX, std::memory_order_relaxed);
  P[src].store(0);
  // Bins persist across rounds, so a round's frontier can exceed E; size for
  // E + V entries twice over.
  std::vector<int32_t> frontier(2 * ((size_t)off[V] + (size_t)V) + 1);
  size_t shared_indexes[2] = {0, kMaxBin};
  std::atomic<size_t> frontier_tails[2];
  frontier_tails[0] = 1;
  frontier_tails[1] = 0;
  frontier[0] = src;
  size_t iter_global = 0;
#pragma omp parallel
  {
    std::vector<std::vector<int32_t>> local_bins;
    size_t iter = 0;
    while (shared_indexes[iter & 1] != kMaxBin) {
      size_t &curr_bin_index = shared_indexes[iter & 1];
      size_t &next_bin_index = shared_indexes[(iter + 1) & 1];
      std::atomic<size_t> &curr_tail = frontier_tails[iter & 1];
      std::atomic<size_t> &next_tail = frontier_tails[(iter + 1) & 1];
      const size_t cur_prio = curr_bin_index;
      const size_t ntail = curr_tail.load();
#pragma omp for nowait schedule(dynamic, 64)
      for (size_t i = 0; i < ntail; i++) {
        const int32_t u = frontier[i];
        const int32_t pu = P[u].load(std::memory_order_relaxed);
        if ((int64_t)pu >= (int64_t)delta * (int64_t)cur_prio) {
          for (int32_t k = off[u]; k < off[u + 1]; ++k) {
            const int32_t v = dst[k];
            const int64_t nv = (int64_t)pu + w[k];
            int32_t old = P[v].load(std::memory_order_relaxed);
            bool changed = false;
            while (nv < old) {
              if (P[v].compare_exchange_weak(old, (int32_t)nv)) {
                changed = true;
                break;
              }
            }
            if (changed) {
              const size_t bin = (size_t)(nv / delta);
              if (bin >= local_bins.size()) local_bins.resize(bin + 1);
              local_bins[bin].push_back(v);
            }
          }
        }
      }
      for (size_t i = cur_prio; i < local_bins.size(); i++) {
        if (!local_bins[i].empty()) {
#pragma omp critical
          next_bin_index = std::min(next_bin_index, i);
          break;
        }
      }
#pragma omp barrier
#pragma omp single nowait
      {
        curr_bin_index = kMaxBin;
        curr_tail.store(0);
        ++iter_global;
      }
      if (next_bin_index < local_bins.size()) {
        const size_t n = local_bins[next_bin_index].size();
        const size_t at = next_tail.fetch_add(n);
        std::copy(local_bins[next_bin_index].begin(), local_bins[next_bin_index].end(),
                  frontier.begin() + at);
        local_bins[next_bin_index].resize(0);
      }
      iter++;
#pragma omp barrier
    }
  }
#pragma omp parallel for schedule(static)
  for (int32_t v = 0; v < V; ++v) dist_out[v] = P[v].load(std::memory_order_relaxed);
}

// ----------------------------------------------------------- PageRank
// apps/pr.cpp:36-69 in FP64: old = 1/V; `iters` times {contrib = old/outdeg;
// new[v] += contrib[u] over edges (u,v); new = (1-d)/V + d*new; old = new;
// new = 0}.  No dangling redistribution, as in the reference.
void orc_pagerank(int32_t V, const int32_t *off, const int32_t *dst,
                  int32_t iters, double damp, double *rank) {
  std::vector<int32_t> toff, tsrc;
  transpose(V, off, dst, toff, tsrc);
  std::vector<double> contrib(V), next(V);
  for (int32_t v = 0; v < V; ++v) rank[v] = 1.0 / V;
  const double beta = (1.0 - damp) / V;
  for (int32_t it = 0; it < iters; ++it) {
    for (int32_t v = 0; v < V; ++v) {
      const int32_t d = off[v + 1] - off[v];
      contrib[v] = d ? rank[v] / d : 0.0;
    }
    for (int32_t v = 0; v < V; ++v) {
      double s = 0;
      for (int32_t k = toff[v]; k < toff[v + 1]; ++k) s += contrib[tsrc[k]];
      next[v] = s;
    }
    for (int32_t v = 0; v < V; ++v) rank[v] = beta + damp * next[v];
  }
}

// OpenMP pull PageRank in fp32, the reference's value type (CPU baseline).
void orc_pagerank_omp(int32_t V, const int32_t *toff, const int32_t *tsrc,
                      const int32_t *outdeg, int32_t iters, float damp,
                      float *rank, int32_t nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  std::vector<float> contrib(V);
  const float beta = (1.0f - damp) / V;
#pragma omp parallel for schedule(static)
  for (int32_t v = 0; v < V; ++v) rank[v] = 1.0f / V;
  for (int32_t it = 0; it < iters; ++it) {
#pragma omp parallel for schedule(static)
    for (int32_t v = 0; v < V; ++v) contrib[v] = outdeg[v] ? rank[v] / outdeg[v] : 0.f;
#pragma omp parallel for schedule(dynamic, 1024)
    for (int32_t v = 0; v < V; ++v) {
      float s = 0;
      for (int32_t k = toff[v]; k < toff[v + 1]; ++k) s += contrib[tsrc[k]];
      rank[v] = beta + damp * s;
    }
  }
}

// ----------------------------------------------------------------- CC
// Weakly connected components by union-find; label = minimum vertex id of the
// component.  apps/cc.cpp's hook + pointer-jump iteration converges to the same
// labels (ID[m] == m stays fixed for the component minimum m).
void orc_cc(int32_t V, const int32_t *off, const int32_t *dst, int32_t *labels) {
  std::vector<int32_t> p(V);
  for (int32_t v = 0; v < V; ++v) p[v] = v;
  auto find = [&](int32_t x) {
    while (p[x] != x) {
      p[x] = p[p[x]];
      x = p[x];
    }
    return x;
  };
  for (int32_t u = 0; u < V; ++u)
    for (int32_t k = off[u]; k < off[u + 1]; ++k) {
      int32_t a = find(u), b = find(dst[k]);
      if (a != b) {
        if (a < b) std::swap(a, b);
        p[a] = b;  // keep the smaller id as root
      }
    }
  for (int32_t v = 0; v < V; ++v) labels[v] = find(v);
}

// Literal sequential restatement of apps/cc.cpp:53-77 (hook over all edges,
// then pointer jumping until stable, until no hook changed anything).
// Returns the number of outer rounds.
int32_t orc_cc_labelprop(int32_t V, const int32_t *off, const int32_t *dst,
                         int32_t *ID) {
  for (int32_t v = 0; v < V; ++v) ID[v] = v;
  int32_t rounds = 0;
  int32_t upd0 = 1;
  while (upd0) {
    upd0 = 0;
    ++rounds;
    for (int32_t s = 0; s < V; ++s)
      for (int32_t k = off[s]; k < off[s + 1]; ++k) {
        const int32_t d = dst[k];
        const int32_t src_id = ID[s], dst_id = ID[d];
        const int32_t p_src = ID[src_id], p_dst = ID[dst_id];
        ID[src_id] = std::min(ID[src_id], p_dst);
        ID[dst_id] = std::min(ID[dst_id], p_src);
        if (p_dst != ID[dst_id] || p_src != ID[src_id]) upd0 = 1;
      }
    int32_t upd1 = 1;
    while (upd1) {
      upd1 = 0;
      for (int32_t v = 0; v < V; ++v) {
        const int32_t y = ID[v], x = ID[y];
        if (x != y) {
          ID[v] = x;
          upd1 = 1;
        }
      }
    }
  }
  return rounds;
}

// OpenMP port of cc.cpp's hook/jump loop (CPU baseline).
void orc_cc_omp(int32_t V, const int32_t *off, const int32_t *dst, int32_t *labels,
                int32_t nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  std::vector<std::atomic<int32_t>> ID(V);
#pragma omp parallel for schedule(static)
  for (int32_t v = 0; v < V; ++v) ID[v].store(v, std::memory_order_relaxed);
  auto wmin = [&](int32_t i, int32_t val) {
    int32_t old = ID[i].load(std::memory_order_relaxed);
    while (val < old && !ID[i].compare_exchange_weak(old, val)) {
    }
  };
  int upd0 = 1;
  while (upd0) {
    upd0 = 0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(| : upd0)
    for (int32_t s = 0; s < V; ++s)
      for (int32_t k = off[s]; k < off[s + 1]; ++k) {
        const int32_t d = dst[k];
        const int32_t si = ID[s].load(std::memory_order_relaxed), di = ID[d].load(std::memory_order_relaxed);
        const int32_t ps = ID[si].load(std::memory_order_relaxed), pd = ID[di].load(std::memory_order_relaxed);
        wmin(si, pd);
        wmin(di, ps);
        if (ps != pd) upd0 = 1;
      }
    int upd1 = 1;
    while (upd1) {
      upd1 = 0;
#pragma omp parallel for schedule(static) reduction(| : upd1)
      for (int32_t v = 0; v < V; ++v) {
        const int32_t y = ID[v].load(std::memory_order_relaxed), x = ID[y].load(std::memory_order_relaxed);
        if (x != y) {
          ID[v].store(x, std::memory_order_relaxed);
          upd1 = 1;
        }
      }
    }
  }
#pragma omp parallel for schedule(static)
  for (int32_t v = 0; v < V; ++v) labels[v] = ID[v].load(std::memory_order_relaxed);
}

// ----------------------------------------------------------------- BC
// apps/bc.cpp:64-123 in FP64, level by level: forward sigma accumulation over
// unvisited neighbours with a deduplicated frontier, a level stack, then the
// backward sweep (dep[v] += 1/sigma[v]; push dep along out-edges to unvisited
// vertices) and final dep = (dep - 1/sigma) * sigma (0 where sigma == 0).
// Correct Brandes dependencies on symmetric graphs, like the reference.
void orc_bc(int32_t V, const int32_t *off, const int32_t *dst, int32_t src,
            double *dep) {
  std::vector<double> sigma(V, 0.0);
  std::vector<uint8_t> visited(V, 0);
  for (int32_t v = 0; v < V; ++v) dep[v] = 0.0;
  if (src < 0 || src >= V) return;
  sigma[src] = 1;
  visited[src] = 1;
  std::vector<std::vector<int32_t>> levels;
  std::vector<int32_t> frontier{src};
  levels.push_back(frontier);
  int32_t round = 0;
  std::vector<int32_t> stamp(V, -1);
  while (!frontier.empty()) {
    ++round;
    std::vector<int32_t> next;
    for (int32_t u : frontier)
      for (int32_t k = off[u]; k < off[u + 1]; ++k) {
        const int32_t v = dst[k];
        if (visited[v]) continue;
        sigma[v] += sigma[u];
        if (stamp[v] != round) {
          stamp[v] = round;
          next.push_back(v);
        }
      }
    for (int32_t v : next) visited[v] = 1;
    frontier.swap(next);
    levels.push_back(frontier);
  }
  std::fill(visited.begin(), visited.end(), 0);
  levels.pop_back();  // the empty last level
  frontier = levels.back();
  levels.pop_back();
  for (int32_t v : frontier) {
    visited[v] = 1;
    dep[v] += 1.0 / sigma[v];
  }
  --round;
  while (round > 0) {
    for (int32_t u : frontier)
      for (int32_t k = off[u]; k < off[u + 1]; ++k)
        if (!visited[dst[k]]) dep[dst[k]] += dep[u];
    frontier = levels.back();
    levels.pop_back();
    for (int32_t v : frontier) {
      visited[v] = 1;
      dep[v] += 1.0 / sigma[v];
    }
    --round;
  }
  for (int32_t v = 0; v < V; ++v)
    dep[v] = sigma[v] != 0 ? (dep[v] - 1.0 / sigma[v]) * sigma[v] : 0.0;
}

// ------------------------------------------------------------- helpers
// Sum of out-degrees of vertices with depth/dist marked reached (>= 0 and
// != INT_MAX): the algorithmic edge count E_r used for TEPS.
int64_t orc_reached_edges(int32_t V, const int32_t *off, const int32_t *val) {
  int64_t s = 0;
  for (int32_t v = 0; v < V; ++v)
    if (val[v] >= 0 && val[v] != INT_MAX) s += off[v + 1] - off[v];
  return s;
}

// ------------------------------------------------------------ input graphs
// R-MAT input of the benchmarks, restated from GAPBS's generator and builder
// (runtime/infra_gapbs/generator.h:45-55, 74-107, 125-139; builder.h:134-163,
// 188-226), so the CPU legs build their graphs without the engine.  Edges come
// in blocks of 2^18, each drawn by a std::mt19937 seeded with seed + block
// index: `scale` float draws per edge pick a quadrant at every level.  Ids are
// then permuted by one std::shuffle driven by std::mt19937(seed), and weights
// U[wmin, wmax] are drawn per block with the same reseeding.  The CSR has V =
// largest id + 1, neighbour lists sorted by (id, weight), repeated neighbours
// merged into the first (lightest) copy, and self-loops dropped; symmetrize
// adds every edge in both directions with its weight.  Pinned by the CSR
// digests of tests/golden (made by the reference's own builder).
struct OrcGraph {
  int32_t V = 0;
  std::vector<int32_t> off, dst, w;
};

void *orc_rmat(int32_t scale, int32_t degree, float a, float b, float c, int64_t seed,
               int32_t symmetrize, int32_t wmin, int32_t wmax) {
  const int64_t M = (int64_t(1) << scale) * degree;
  const int64_t kEdgeBlock = int64_t(1) << 18;
  const int64_t nblocks = (M + kEdgeBlock - 1) / kEdgeBlock;
  std::vector<int32_t> eu(M), ev(M), ew(M);
  const float ab = a + b, abc = a + b + c;
#pragma omp parallel for schedule(static)
  for (int64_t blk = 0; blk < nblocks; ++blk) {
    std::mt19937 gen((std::mt19937::result_type)(seed + blk));
    std::uniform_real_distribution<float> unit(0.0f, 1.0f);
    const int64_t end = std::min(M, (blk + 1) * kEdgeBlock);
    for (int64_t e = blk * kEdgeBlock; e < end; ++e) {
      int32_t x = 0, y = 0;
      for (int32_t lvl = 0; lvl < scale; ++lvl) {
        const float r = unit(gen);
        x = 2 * x + (r < ab ? 0 : 1);
        y = 2 * y + (r < ab ? (r > a ? 1 : 0) : (r > abc ? 1 : 0));
      }
      eu[e] = x;
      ev[e] = y;
    }
  }
  std::vector<int32_t> relabel(size_t(1) << scale);
  std::iota(relabel.begin(), relabel.end(), 0);
  std::mt19937 perm_gen((std::mt19937::result_type)seed);
  std::shuffle(relabel.begin(), relabel.end(), perm_gen);
  int32_t top = 0;
#pragma omp parallel for schedule(static) reduction(max : top)
  for (int64_t blk = 0; blk < nblocks; ++blk) {
    std::mt19937 gen((std::mt19937::result_type)(seed + blk));
    std::uniform_int_distribution<int> draw(wmin, wmax);
    const int64_t end = std::min(M, (blk + 1) * kEdgeBlock);
    for (int64_t e = blk * kEdgeBlock; e < end; ++e) {
      eu[e] = relabel[eu[e]];
      ev[e] = relabel[ev[e]];
      ew[e] = draw(gen);
      top = std::max(top, std::max(eu[e], ev[e]));
    }
  }
  auto *g = new OrcGraph();
  const int32_t V = top + 1;
  g->V = V;
  // bucket (neighbour, weight) pairs by source, then sort and merge per vertex
  std::vector<int64_t> start(V + 1, 0);
  for (int64_t e = 0; e < M; ++e) {
    start[eu[e] + 1]++;
    if (symmetrize) start[ev[e] + 1]++;
  }
  for (int32_t v = 0; v < V; ++v) start[v + 1] += start[v];
  std::vector<std::pair<int32_t, int32_t>> adj(start[V]);
  {
    std::vector<int64_t> fillp(start.begin(), start.end() - 1);
    for (int64_t e = 0; e < M; ++e) {
      adj[fillp[eu[e]]++] = {ev[e], ew[e]};
      if (symmetrize) adj[fillp[ev[e]]++] = {eu[e], ew[e]};
    }
  }
  std::vector<int32_t> keep(V, 0);
#pragma omp parallel for schedule(dynamic, 256)
  for (int32_t v = 0; v < V; ++v) {
    auto *lo = adj.data() + start[v], *hi = adj.data() + start[v + 1];
    std::sort(lo, hi);
    int32_t k = 0;
    for (auto *p = lo; p < hi; ++p) {
      if (p->first == v) continue;
      if (k > 0 && lo[k - 1].first == p->first) continue;
      lo[k++] = *p;
    }
    keep[v] = k;
  }
  g->off.assign(V + 1, 0);
  for (int32_t v = 0; v < V; ++v) g->off[v + 1] = g->off[v] + keep[v];
  g->dst.resize(g->off[V]);
  g->w.resize(g->off[V]);
#pragma omp parallel for schedule(dynamic, 256)
  for (int32_t v = 0; v < V; ++v)
    for (int32_t k = 0; k < keep[v]; ++k) {
      g->dst[g->off[v] + k] = adj[start[v] + k].first;
      g->w[g->off[v] + k] = adj[start[v] + k].second;
    }
  return g;
}

int32_t orc_graph_vertices(const void *h) { return static_cast<const OrcGraph *>(h)->V; }
int64_t orc_graph_edges(const void *h) { return (int64_t) static_cast<const OrcGraph *>(h)->dst.size(); }
void orc_graph_copy(const void *h, int32_t *off, int32_t *dst, int32_t *w) {
  const OrcGraph *g = static_cast<const OrcGraph *>(h);
  std::copy(g->off.begin(), g->off.end(), off);
  std::copy(g->dst.begin(), g->dst.end(), dst);
  std::copy(g->w.begin(), g->w.end(), w);
}
void orc_graph_free(void *h) { delete static_cast<OrcGraph *>(h); }

// GAPBS SourcePicker (runtime/infra_gapbs/benchmark.h:50-71): uniform ids
// from one std::mt19937(seed), skipping vertices without out-edges.
void orc_pick_sources(int32_t V, const int32_t *off, int32_t n, int64_t seed, int32_t *out) {
  std::mt19937 gen((std::mt19937::result_type)seed);
  std::uniform_int_distribution<int32_t> pick(0, V - 1);
  for (int32_t i = 0; i < n; ++i) {
    int32_t v = pick(gen);
    while (off[v + 1] == off[v]) v = pick(gen);
    out[i] = v;
  }
}

}  // extern "C"
