/*
 * graphit/operators.h -- the GraphIt GPU operators in C++ over libgg.so.
 *
 * The reference's operator chain (easy_graphit include/graphit/operators.h:
 * 38-178, src/graphit/operators.cpp:10-65, 513-672) and the runtime objects
 * its generated code calls (runtime/infra_gpu/: GraphT, VertexFrontier,
 * GPUPriorityQueue, VertexFrontierList), as RAII wrappers that call the C ABI:
 *
 *   edgeset_apply(s).from(frontier).to(Filter::PARENT_UNSET)
 *       .apply_modified(edges, frontier, parent_data, Udf::BFS_PARENT);
 *   edgeset_apply(s).from(pq.dequeue()).apply_priority(edges, Udf::SSSP_RELAX, pq, data);
 *   vertexset_apply(edges, VertexUdf::BFS_RESET, data);
 *
 * The reference stages UDFs written as C++ lambdas into CUDA; here the five
 * apps' UDFs ship compiled in libgg.so and are named by Udf / VertexUdf /
 * Filter, and VertexData is gg_vertex_data: the device arrays they touch.
 * Errors throw graphit::error (status + message) where the reference calls
 * exit(-1) or asserts.
 */
#ifndef GRAPHIT_GB300_OPERATORS_H
#define GRAPHIT_GB300_OPERATORS_H

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../gg.h"
#include "schedule.h"

namespace graphit {

struct error : std::runtime_error {
  gg_status status;
  error(gg_status s, const std::string &m) : std::runtime_error(m), status(s) {}
};

inline void check(gg_status s) {
  if (s == GG_OK) return;
  char buf[2048];
  gg_last_error(buf, sizeof buf);
  throw error(s, buf);
}

enum class Udf : int32_t {
  BFS_PARENT = GG_UDF_BFS_PARENT,   // bfs.cpp:23-25
  SSSP_RELAX = GG_UDF_SSSP_RELAX,   // sssp.cpp:24-27
  PR_ADD = GG_UDF_PR_ADD,           // pr.cpp:32-34
  CC_HOOK = GG_UDF_CC_HOOK,         // cc.cpp:23-36
  BC_FORWARD = GG_UDF_BC_FORWARD,   // bc.cpp:34-36
  BC_BACKWARD = GG_UDF_BC_BACKWARD  // bc.cpp:52-54
};
enum class Filter : int32_t {
  NONE = GG_FILTER_NONE,
  PARENT_UNSET = GG_FILTER_PARENT_UNSET,  // bfs.cpp:27-29
  UNVISITED = GG_FILTER_UNVISITED         // bc.cpp:38-40
};
enum class VertexUdf : int32_t {
  BFS_RESET = GG_VUDF_BFS_RESET,
  SSSP_RESET = GG_VUDF_SSSP_RESET,
  PR_RESET = GG_VUDF_PR_RESET,
  PR_CONTRIB = GG_VUDF_PR_CONTRIB,
  PR_UPDATE = GG_VUDF_PR_UPDATE,
  CC_INIT = GG_VUDF_CC_INIT,
  CC_PJUMP = GG_VUDF_CC_PJUMP,
  BC_RESET = GG_VUDF_BC_RESET,
  BC_MARK_VISITED = GG_VUDF_BC_MARK_VISITED,
  BC_MARK_UNVISITED = GG_VUDF_BC_MARK_UNVISITED,
  BC_BACKWARD_VERTEX = GG_VUDF_BC_BACKWARD_VERTEX,
  BC_FINAL = GG_VUDF_BC_FINAL
};
using VertexData = gg_vertex_data;

// graphit_runtime::GraphT (graph.h:17-88): a CSR resident in HBM.
class GraphT {
 public:
  GraphT(const int32_t *offsets, const int32_t *dst, const int32_t *weights, int32_t num_vertices,
         int64_t num_edges, bool symmetric = false)
      : V_(num_vertices), E_(num_edges) {
    check(gg_graph_create(offsets, dst, weights, num_vertices, num_edges, symmetric ? GG_GRAPH_SYMMETRIC : 0, &g_));
  }
  ~GraphT() {
    if (g_) gg_graph_destroy(g_);
  }
  GraphT(const GraphT &) = delete;
  GraphT &operator=(const GraphT &) = delete;
  gg_graph *handle() const { return g_; }
  int32_t num_vertices() const { return V_; }
  int64_t num_edges() const { return E_; }
  GraphT &get_transposed_graph() {
    check(gg_graph_transpose(g_));
    return *this;
  }
  void sync() { check(gg_graph_sync(g_)); }

 private:
  gg_graph *g_ = nullptr;
  int32_t V_;
  int64_t E_;
};

// graphit_runtime::VertexFrontier (vertex_frontier.h:26-166).
class VertexSubset {
 public:
  explicit VertexSubset(GraphT &g, bool init_all = false) { check(gg_frontier_create(g.handle(), init_all, &f_)); }
  ~VertexSubset() {
    if (f_ && owned_) gg_frontier_destroy(f_);
  }
  VertexSubset(const VertexSubset &) = delete;
  VertexSubset &operator=(const VertexSubset &) = delete;
  VertexSubset(VertexSubset &&o) noexcept : f_(std::exchange(o.f_, nullptr)), owned_(o.owned_) {}
  gg_frontier *handle() const { return f_; }
  void addVertex(int32_t v) { check(gg_frontier_add(f_, v)); }
  int32_t size() {
    int32_t n = 0;
    check(gg_frontier_size(f_, &n));
    return n;
  }
  void to_sparse() { check(gg_frontier_to_sparse(f_)); }
  void to_bitmap() { check(gg_frontier_to_bitmap(f_)); }
  void to_boolmap() { check(gg_frontier_to_boolmap(f_)); }
  void dedup() { check(gg_frontier_dedup(f_)); }  // dedup_frontier_perfect
  std::vector<int32_t> read() {
    int32_t n = 0;
    check(gg_frontier_read(f_, nullptr, 0, &n));
    std::vector<int32_t> out(n);
    if (n) check(gg_frontier_read(f_, out.data(), n, &n));
    return out;
  }

 private:
  friend class PriorityQueue;
  VertexSubset() = default;  // a view of a frontier owned elsewhere
  gg_frontier *f_ = nullptr;
  bool owned_ = true;
};

// graphit_runtime::GPUPriorityQueue (gpu_priority_queue.h:21-247) with
// pq.init(edges, SP, init, delta, src) of sssp.cpp:39.
class PriorityQueue {
 public:
  PriorityQueue(GraphT &g, int32_t *priorities, int32_t init_priority, int32_t delta, int32_t src) {
    check(gg_pq_create(g.handle(), priorities, init_priority, delta, src, &pq_));
    view_.owned_ = false;
  }
  ~PriorityQueue() {
    if (pq_) gg_pq_destroy(pq_);
  }
  PriorityQueue(const PriorityQueue &) = delete;
  PriorityQueue &operator=(const PriorityQueue &) = delete;
  gg_pq *handle() const { return pq_; }
  bool finished() {
    int32_t f = 0;
    check(gg_pq_finished(pq_, &f));
    return f != 0;
  }
  VertexSubset &dequeue() {
    check(gg_pq_dequeue(pq_, &view_.f_));
    return view_;
  }

 private:
  gg_pq *pq_ = nullptr;
  VertexSubset view_;
};

// graphit_runtime::VertexFrontierList (list.h:18-116), bc.cpp's level stack.
class FrontierList {
 public:
  explicit FrontierList(GraphT &g) { check(gg_frontier_list_create(g.handle(), &l_)); }
  ~FrontierList() {
    if (l_) gg_frontier_list_destroy(l_);
  }
  FrontierList(const FrontierList &) = delete;
  FrontierList &operator=(const FrontierList &) = delete;
  void insert(VertexSubset &f) { check(gg_frontier_list_insert(l_, f.handle())); }
  void retrieve(VertexSubset &f) { check(gg_frontier_list_retrieve(l_, f.handle())); }

 private:
  gg_frontier_list *l_ = nullptr;
};

// operators.h:38-178.
struct edgeset_apply {
  SimpleGPUSchedule _default_schedule;
  Schedule *current_schedule;
  VertexSubset *from_set = nullptr;
  Filter to_filter = Filter::NONE;

  edgeset_apply() : current_schedule(&_default_schedule) {}
  explicit edgeset_apply(Schedule &s) : current_schedule(&s) {}

  edgeset_apply &from(VertexSubset &f) {
    from_set = &f;
    return *this;
  }
  edgeset_apply &to(Filter f) {
    to_filter = f;
    return *this;
  }

  void apply(GraphT &graph, Udf udf, const VertexData &vd) { run(graph, udf, vd, nullptr, true); }
  // The output frontier is `to`; allow_dupes = false deduplicates it, fused
  // into the apply or, with deduplication_strategy UNFUSED, by a pass after it.
  void apply_modified(GraphT &graph, VertexSubset &to, const VertexData &vd, Udf udf, bool allow_dupes = true) {
    run(graph, udf, vd, &to, allow_dupes);
  }
  void apply_priority(GraphT &graph, Udf udf, PriorityQueue &pq, const VertexData &vd) {
    if (udf != Udf::SSSP_RELAX) throw error(GG_ERR_INVALID, "apply_priority takes the SSSP relax UDF");
    const gg_schedule s = pick(graph).to_c();
    check(gg_edgeset_apply_priority(graph.handle(), &s, pq.handle(), &vd));
  }

 private:
  // A hybrid schedule decides on |from| at every call (operators.h:116-132).
  const SimpleGPUSchedule &pick(GraphT &graph) {
    Schedule *s = current_schedule;
    if (auto *h = s_to<HybridGPUSchedule>(s)) {
      const double n = from_set ? from_set->size() : graph.num_vertices();
      s = n <= (double)h->current_threshold() * graph.num_vertices() ? h->s1 : h->s2;
    } else if (auto *l = s_to<LearnedGPUSchedule>(s)) {
      return l->fallback;
    }
    if (auto *simple = s_to<SimpleGPUSchedule>(s)) return *simple;
    throw error(GG_ERR_UNSUPPORTED, "edgeset_apply needs a simple, hybrid or learned schedule");
  }
  void run(GraphT &graph, Udf udf, const VertexData &vd, VertexSubset *out, bool allow_dupes) {
    const gg_schedule s = pick(graph).to_c();
    check(gg_edgeset_apply(graph.handle(), &s, static_cast<int32_t>(udf), static_cast<int32_t>(to_filter),
                           from_set ? from_set->handle() : nullptr, out ? out->handle() : nullptr,
                           allow_dupes ? 1 : 0, &vd));
  }
};

// vertexset_apply(set | graph, udf) (operators.cpp:10-65).
inline void vertexset_apply(VertexSubset &set, VertexUdf udf, GraphT &graph, const VertexData &vd) {
  check(gg_vertexset_apply(graph.handle(), set.handle(), static_cast<int32_t>(udf), &vd));
}
inline void vertexset_apply(GraphT &graph, VertexUdf udf, const VertexData &vd) {
  check(gg_vertexset_apply(graph.handle(), nullptr, static_cast<int32_t>(udf), &vd));
}

}  // namespace graphit

#endif  // GRAPHIT_GB300_OPERATORS_H
