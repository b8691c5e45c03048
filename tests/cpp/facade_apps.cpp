// Drives libgg.so through the C++ facade (include/graphit/{schedule,operators}.h)
// the way the reference's apps drive their operators: the testcase() loops of
// apps/bfs.cpp:36-62, apps/sssp.cpp:34-57 and apps/bc.cpp:64-123, written
// against graphit::edgeset_apply / vertexset_apply / PriorityQueue /
// FrontierList, plus the whole-app entry point through app_schedule().
//
//   facade_apps <out_dir>
//
// Graphs: the symmetrized R-MAT 12 (edge factor 16) and the directed R-MAT 12,
// from gg_host_graph_rmat with GAPBS's seed.  Writes raw int32 / float32 arrays
// to <out_dir>/<name>.bin; tests/test_gpu_facade.py checks them with the oracle.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "graphit/operators.h"
#include "graphit/schedule.h"

using graphit::edgeset_apply;
using graphit::Filter;
using graphit::GraphT;
using graphit::SimpleGPUSchedule;
using graphit::Udf;
using graphit::VertexData;
using graphit::VertexSubset;
using graphit::VertexUdf;
using graphit::vertexset_apply;

namespace {

std::string out_dir;

template <class T>
struct DeviceArray {
  T *p = nullptr;
  size_t n = 0;
  explicit DeviceArray(size_t count) : n(count) {
    if (cudaMalloc(&p, sizeof(T) * count) != cudaSuccess) throw std::runtime_error("cudaMalloc failed");
  }
  ~DeviceArray() { cudaFree(p); }
  std::vector<T> host() const {
    std::vector<T> h(n);
    cudaMemcpy(h.data(), p, sizeof(T) * n, cudaMemcpyDeviceToHost);
    return h;
  }
};

template <class T>
void save(const std::string &name, const std::vector<T> &v) {
  const std::string path = out_dir + "/" + name + ".bin";
  FILE *f = fopen(path.c_str(), "wb");
  if (!f || fwrite(v.data(), sizeof(T), v.size(), f) != v.size()) throw std::runtime_error("cannot write " + path);
  fclose(f);
}

struct Host {
  gg_host_graph *h = nullptr;
  int32_t V = 0;
  int64_t E = 0;
  Host(int scale, bool sym) {
    graphit::check(gg_host_graph_rmat(scale, 16, 0.57f, 0.19f, 0.19f, 27491095, sym ? 1 : 0, 1, 255, &h));
    graphit::check(gg_host_graph_info(h, &V, &E));
  }
  ~Host() { gg_host_graph_destroy(h); }
  int32_t hub() const {
    const int32_t *off = gg_host_graph_offsets(h);
    int32_t best = 0;
    for (int32_t v = 0; v < V; ++v)
      if (off[v + 1] - off[v] > off[best + 1] - off[best]) best = v;
    return best;
  }
};

// apps/bfs.cpp:36-62, one trial; returns the parent array.
std::vector<int32_t> bfs_testcase(GraphT &edges, int32_t src, graphit::Schedule &s1) {
  DeviceArray<int32_t> parent(edges.num_vertices());
  VertexData vd{};
  vd.parent = parent.p;
  vd.src = src;
  vertexset_apply(edges, VertexUdf::BFS_RESET, vd);  // reset; parent[src] = src
  VertexSubset frontier(edges);
  frontier.addVertex(src);
  while (frontier.size() != 0)
    edgeset_apply(s1).from(frontier).to(Filter::PARENT_UNSET).apply_modified(edges, frontier, vd, Udf::BFS_PARENT);
  return parent.host();
}

// apps/sssp.cpp:34-57, one trial.
std::vector<int32_t> sssp_testcase(GraphT &edges, int32_t src, int32_t delta, graphit::Schedule &s1) {
  DeviceArray<int32_t> SP(edges.num_vertices());
  graphit::PriorityQueue pq(edges, SP.p, 0, delta, src);
  VertexData vd{};
  vd.dist = SP.p;
  vd.src = src;
  vertexset_apply(edges, VertexUdf::SSSP_RESET, vd);  // reset; SP[src] = 0
  while (!pq.finished()) {
    VertexSubset &frontier = pq.dequeue();
    edgeset_apply(s1).from(frontier).apply_priority(edges, Udf::SSSP_RELAX, pq, vd);
  }
  return SP.host();
}

// apps/bc.cpp:64-123, one trial (fp32 dependences).
std::vector<float> bc_testcase(GraphT &edges, int32_t src, graphit::Schedule &s1) {
  const int32_t V = edges.num_vertices();
  DeviceArray<double> num_paths(V);
  DeviceArray<float> dependences(V);
  DeviceArray<uint8_t> visited(V);
  VertexData vd{};
  vd.num_paths = num_paths.p;
  vd.dependences = dependences.p;
  vd.visited = visited.p;
  vd.src = src;
  vertexset_apply(edges, VertexUdf::BC_RESET, vd);  // reset; num_paths[src] = 1; visited[src] = 1
  VertexSubset frontier(edges);
  frontier.addVertex(src);
  int round = 0;
  graphit::FrontierList frontier_list(edges);
  frontier_list.insert(frontier);
  while (frontier.size() != 0) {
    round = round + 1;
    edgeset_apply(s1).from(frontier).to(Filter::UNVISITED).apply_modified(edges, frontier, vd, Udf::BC_FORWARD,
                                                                           false);
    graphit::vertexset_apply(frontier, VertexUdf::BC_MARK_VISITED, edges, vd);
    frontier_list.insert(frontier);
  }
  vertexset_apply(edges, VertexUdf::BC_MARK_UNVISITED, vd);
  frontier_list.retrieve(frontier);
  frontier_list.retrieve(frontier);
  graphit::vertexset_apply(frontier, VertexUdf::BC_BACKWARD_VERTEX, edges, vd);
  round = round - 1;
  while (round > 0) {
    edgeset_apply(s1).from(frontier).to(Filter::UNVISITED).apply(edges, Udf::BC_BACKWARD, vd);
    frontier_list.retrieve(frontier);
    graphit::vertexset_apply(frontier, VertexUdf::BC_BACKWARD_VERTEX, edges, vd);
    round = round - 1;
  }
  vertexset_apply(edges, VertexUdf::BC_FINAL, vd);
  return dependences.host();
}

}  // namespace

int main(int argc, char **argv) {
  if (argc != 2) {
    fprintf(stderr, "usage: %s <out_dir>\n", argv[0]);
    return 2;
  }
  out_dir = argv[1];
  try {
    Host hs(12, true), hd(12, false);
    GraphT sym(gg_host_graph_offsets(hs.h), gg_host_graph_dst(hs.h), gg_host_graph_weights(hs.h), hs.V, hs.E, true);
    GraphT dir(gg_host_graph_offsets(hd.h), gg_host_graph_dst(hd.h), gg_host_graph_weights(hd.h), hd.V, hd.E);
    using LB = SimpleGPUSchedule::load_balancing_type;
    using Dir = SimpleGPUSchedule::direction_type;
    using FC = SimpleGPUSchedule::frontier_creation_type;
    using Rep = SimpleGPUSchedule::pull_frontier_rep_type;

    // bfs.cpp's two schedules: PUSH TWCE, and the "power" hybrid
    SimpleGPUSchedule push_twce;
    push_twce.configDirection(Dir::PUSH);
    push_twce.configLoadBalancing(LB::TWCE);
    SimpleGPUSchedule pull_vb;
    pull_vb.configDirection(Dir::PULL, Rep::BITMAP);
    pull_vb.configLoadBalancing(LB::VERTEX_BASED);
    pull_vb.configFrontierCreation(FC::BITMAP);
    graphit::HybridGPUSchedule power(push_twce, pull_vb);
    float t = 0.12f;
    power.bindThreshold(t);
    const int32_t s_sym = hs.hub(), s_dir = hd.hub();
    save("bfs_push_twce", bfs_testcase(sym, s_sym, push_twce));
    save("bfs_power", bfs_testcase(sym, s_sym, power));
    t = 0.0f;  // the bound threshold is read at every call
    save("bfs_power_t0", bfs_testcase(sym, s_sym, power));

    // sssp.cpp's default (PUSH SPARSE VERTEX_BASED) and power (TWCE, BOOLMAP)
    SimpleGPUSchedule vb;
    vb.configDirection(Dir::PUSH);
    vb.configFrontierCreation(FC::SPARSE);
    SimpleGPUSchedule twce_boolmap;
    twce_boolmap.configDirection(Dir::PUSH);
    twce_boolmap.configLoadBalancing(LB::TWCE);
    twce_boolmap.configFrontierCreation(FC::BOOLMAP);
    save("sssp_vertex_d8", sssp_testcase(dir, s_dir, 8, vb));
    save("sssp_twce_boolmap_d32", sssp_testcase(dir, s_dir, 32, twce_boolmap));

    // bc.cpp's default, and with the unfused dedup pass
    save("bc_push_twce", bc_testcase(sym, s_sym, push_twce));
    SimpleGPUSchedule twce_unfused = push_twce;
    twce_unfused.configDeduplication(SimpleGPUSchedule::deduplication_type::ENABLED,
                                     SimpleGPUSchedule::deduplication_strategy_type::UNFUSED);
    save("bc_push_twce_unfused_dedup", bc_testcase(sym, s_sym, twce_unfused));

    // the whole-app entry point with the same schedule objects (fused, as bfs.cpp's main)
    std::vector<int32_t> depth(hs.V);
    gg_app_schedule a = graphit::app_schedule(push_twce, true);
    graphit::check(gg_bfs(sym.handle(), &a, s_sym, depth.data(), nullptr, nullptr));
    save("bfs_app_depth", depth);
    std::vector<int32_t> meta{s_sym, s_dir, hs.V, hd.V};
    save("meta", meta);
  } catch (const graphit::error &e) {
    fprintf(stderr, "graphit error %d: %s\n", (int)e.status, e.what());
    return 1;
  } catch (const std::exception &e) {
    fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
  printf("facade_apps ok\n");
  return 0;
}
