// Test infrastructure, not product code: a host-execution stand-in for the
// BuildIt-staged GraphIt API, so that the reference's own application sources
// (apps/{bfs,sssp,pr,cc,bc}.cpp of easy_graphit) compile with g++ and RUN on
// the CPU.  The reference stages these apps with BuildIt (builder::dyn_var and
// friends) to generate CUDA; BuildIt is an empty submodule in the reference
// tree, so its staging cannot be built.  This header gives the same names
// (dyn_var, Vertex, VertexData, GraphT, VertexSubset, FrontierList,
// PriorityQueue, edgeset_apply / vertexset_apply, the schedules, the runtime
// calls, builder_context / run_graphit_pipeline) plain sequential meaning:
//
//  * dyn_var<T> is T itself (a value, not a staged expression), except that
//    dyn_var<float> and VertexData<float> hold double: the apps' arithmetic
//    runs in FP64, which makes the run an FP64 oracle of the reference's code;
//  * edgeset_apply(s).from(f).to(filter).apply(...) visits, for every source
//    in f (every vertex without from()), its out-edges in CSR order and calls
//    the UDF on each edge whose destination passes the filter; schedules
//    (direction, load balancing, blocking, fusion) change only the order and
//    parallelism of these calls on the GPU, so they are accepted and ignored;
//  * apply_modified(g, to, var, udf, allow_dupes) tracks writes to `var`
//    during the apply (assignment, +=, and a min() that lowers the value) and
//    makes `to` the list of written destinations, once each unless
//    allow_dupes (operators.h:108-176); apply_priority / PriorityQueue follow
//    runtime/infra_gpu/gpu_priority_queue.h:33-153,250-297 (next window =
//    smallest priority >= cur + delta, frontier = [cur, cur + delta));
//  * builder_context().extract_function_ast(testcase, name, static args...)
//    returns the call itself: the testcase's leading dynamic parameters come
//    from the environment (GG_SHIM_ARG0 = graph file, GG_SHIM_ARG1 ... =
//    source, threshold or delta), and run_graphit_pipeline runs it, then
//    writes every VertexData to $GG_SHIM_OUT/<name>.<i32|u8|f64>.
//
// Graph files are the .graphit_bin layout load_graph reads
// (runtime/infra_gpu/graph.h:255-270): V, E, src[E], dst[E], weight[E],
// offsets[V+1], all int32.
#pragma once

#include <algorithm>
#include <chrono>
#include <climits>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <iostream>
#include <memory>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

namespace shim {
template <class T>
struct host {
  using type = T;
};
template <>
struct host<float> {
  using type = double;
};
}  // namespace shim
template <class T>
using dyn_var = typename shim::host<T>::type;

namespace graphit {

enum class context_type { HOST = 0, DEVICE = 1 };
inline context_type current_context = context_type::HOST;

// ---------------------------------------------------------------- schedules
struct Schedule {
  virtual ~Schedule() = default;
};
template <typename T>
bool s_isa(Schedule *s) {
  return dynamic_cast<T *>(s) != nullptr;
}
template <typename T>
T *s_to(Schedule *s) {
  return dynamic_cast<T *>(s);
}
struct SimpleGPUSchedule : public Schedule {
  static inline int default_max_cta = 60;
  static inline int default_cta_size = 512;
  enum class direction_type { PUSH, PULL };
  enum class pull_frontier_rep_type { BITMAP, BOOLMAP };
  enum class frontier_creation_type { SPARSE, BITMAP, BOOLMAP };
  enum class deduplication_type { DISABLED, ENABLED };
  enum class deduplication_strategy_type { FUSED, UNFUSED };
  enum class load_balancing_type { VERTEX_BASED, TWC, TWCE, WM, CM, STRICT, EDGE_ONLY };
  enum class edge_blocking_type { BLOCKED, UNBLOCKED };
  enum class kernel_fusion_type { DISABLED, ENABLED };
  void configDirection(direction_type, pull_frontier_rep_type = pull_frontier_rep_type::BOOLMAP) {}
  void configFrontierCreation(frontier_creation_type) {}
  void configDeduplication(deduplication_type) {}
  void configDeduplication(deduplication_type, deduplication_strategy_type) {}
  void configLoadBalancing(load_balancing_type, edge_blocking_type = edge_blocking_type::UNBLOCKED, int = -1) {}
  void configDelta(int) {}
};
struct HybridGPUSchedule : public Schedule {
  Schedule *s1, *s2;
  double threshold = 0;
  HybridGPUSchedule(Schedule &a, Schedule &b) : s1(&a), s2(&b) {}
  void configThreshold(float t) { threshold = t; }
  void bindThreshold(double t) { threshold = t; }
};

// -------------------------------------------------------------------- types
struct Vertex {
  int vid;
  Vertex(int v) : vid(v) {}
  operator int() const { return vid; }
};

struct GraphT;
struct GraphData {
  int V = 0, E = 0;
  std::vector<int> off, src, dst, w, outdeg;
  std::shared_ptr<GraphData> transposed;
};

struct GraphT {
  std::shared_ptr<GraphData> d;
  int num_vertices = 0, num_edges = 0;
  int *out_degrees = nullptr;
  std::shared_ptr<GraphT> t;
  GraphT() = default;
  explicit GraphT(const char *) {}
  explicit GraphT(std::shared_ptr<GraphData> g) : d(std::move(g)) {
    num_vertices = d->V;
    num_edges = d->E;
    out_degrees = d->outdeg.data();
  }
  // get_transposed_graph()[0]: the transpose, in-lists in source order.
  GraphT *get_transposed_graph() {
    if (!t) {
      auto g = std::make_shared<GraphData>();
      g->V = d->V;
      g->E = d->E;
      g->off.assign(d->V + 1, 0);
      for (int e = 0; e < d->E; ++e) g->off[d->dst[e] + 1]++;
      for (int v = 0; v < d->V; ++v) g->off[v + 1] += g->off[v];
      std::vector<int> pos(g->off.begin(), g->off.end() - 1);
      g->src.resize(d->E);
      g->dst.resize(d->E);
      g->w.resize(d->E);
      for (int v = 0; v < d->V; ++v)
        for (int e = d->off[v]; e < d->off[v + 1]; ++e) {
          const int p = pos[d->dst[e]]++;
          g->src[p] = d->dst[e];
          g->dst[p] = v;
          g->w[p] = d->w[e];
        }
      g->outdeg.resize(d->V);
      for (int v = 0; v < d->V; ++v) g->outdeg[v] = g->off[v + 1] - g->off[v];
      t = std::make_shared<GraphT>(g);
    }
    return t.get();
  }
};

struct VertexSubset {
  std::vector<int> v;
  int max_elems = 0;
  void addVertex(int x) { v.push_back(x); }
  int size() const { return (int)v.size(); }
  VertexSubset *addr() { return this; }
};

struct FrontierList {
  std::vector<std::vector<int>> levels;
  void insert(VertexSubset &s) { levels.push_back(s.v); }
  void retrieve(VertexSubset &s) {
    s.v = levels.empty() ? std::vector<int>{} : levels.back();
    if (!levels.empty()) levels.pop_back();
  }
};

// Every VertexData registers itself (name, dump function) so that the run's
// results can be written out by name.
struct Dumpable {
  std::string name;
  std::function<void(const std::string &)> dump;
};
inline std::vector<Dumpable> &registry() {
  static std::vector<Dumpable> r;
  return r;
}

template <typename T>
struct VertexData {
  using H = dyn_var<T>;
  std::string name;
  std::vector<H> data;
  // apply_modified tracking
  std::vector<int> *out = nullptr;
  std::vector<char> mark;
  bool dupes = true;

  explicit VertexData(std::string n) : name(std::move(n)) {
    registry().push_back({name, [this](const std::string &dir) { write(dir); }});
  }
  VertexData(const VertexData &) = delete;
  void allocate(int n) { data.assign((size_t)std::max(n, 0), H()); }
  void touch(int i) {
    if (!out) return;
    if (dupes) {
      out->push_back(i);
    } else if (!mark[i]) {
      mark[i] = 1;
      out->push_back(i);
    }
  }
  struct Ref {
    VertexData *vd;
    int i;
    operator H() const { return vd->data[i]; }
    Ref &operator=(H x) {
      vd->data[i] = x;
      vd->touch(i);
      return *this;
    }
    Ref &operator=(const Ref &o) { return *this = (H)o; }
    void operator+=(H x) {
      vd->data[i] += x;
      vd->touch(i);
    }
    void min(H x) {
      if (vd->data[i] > x) {
        vd->data[i] = x;
        vd->touch(i);
      }
    }
  };
  Ref operator[](int i) { return Ref{this, i}; }
  void write(const std::string &dir) const {
    if (data.empty()) return;
    const char *ext = std::is_same<H, double>::value ? "f64"
                      : std::is_same<H, unsigned char>::value ? "u8"
                      : std::is_same<H, int>::value ? "i32" : "raw";
    const std::string path = dir + "/" + name + "." + ext;
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) {
      std::fprintf(stderr, "cannot write %s\n", path.c_str());
      std::exit(1);
    }
    std::fwrite(data.data(), sizeof(H), data.size(), f);
    std::fclose(f);
  }
};

// gpu_priority_queue.h:33-153 and 250-297 run sequentially.  The number of
// window moves of the last run (each a scan for the next priority, the last
// one finding none) is written out as <name>_advances.
struct PriorityQueue {
  VertexData<int> *p = nullptr;
  long long current = 0, window_upper = 0, cutoff = 0;
  int delta = 1;
  bool ready = false;
  int advances = 0;
  std::vector<int> frontier, out;
  explicit PriorityQueue(std::string name) {
    registry().push_back({name, [this, name](const std::string &dir) {
                            const std::string path = dir + "/" + name + "_advances.i32";
                            FILE *f = std::fopen(path.c_str(), "wb");
                            if (!f) std::exit(1);
                            std::fwrite(&advances, sizeof(int), 1, f);
                            std::fclose(f);
                          }});
  }
  void init(GraphT &, VertexData<int> &p_, int init_p, int delta_, int src = -1) {
    p = &p_;
    current = init_p;
    delta = delta_;
    ready = false;
    advances = 0;
    frontier.clear();
    if (src != -1) frontier.push_back(src);
    cutoff = current + delta;
  }
  void updatePriorityMin(Vertex v, int np) {
    int &x = p->data[v.vid];
    if (np < x) {
      x = np;
      if (np < cutoff) out.push_back(v.vid);
    }
  }
  void advance() {
    ++advances;
    window_upper = current + delta;
    long long m = INT_MAX;
    for (int x : p->data)
      if (x >= window_upper && x != INT_MAX && x < m) m = x;
    current = m;
    frontier.clear();
    for (int v = 0; v < (int)p->data.size(); ++v) {
      const long long x = p->data[v];
      if (x >= current && x < current + delta) frontier.push_back(v);
    }
    cutoff = current + delta;
  }
  int finished() {
    if (current == INT_MAX) return 1;
    if (!ready && frontier.empty()) {
      advance();
      ready = true;
      return current == INT_MAX;
    }
    return 0;
  }
  VertexSubset dequeue() {
    if (ready) {
      ready = false;
    } else if (frontier.empty()) {
      advance();
      ready = false;
    }
    VertexSubset s;
    s.v = frontier;
    return s;
  }
};

// ---------------------------------------------------------------- operators
inline void vertexset_apply(GraphT &g, const std::function<void(Vertex)> &f) {
  for (int v = 0; v < g.num_vertices; ++v) f(Vertex(v));
}
inline void vertexset_apply(VertexSubset &s, const std::function<void(Vertex)> &f) {
  const std::vector<int> members = s.v;
  for (int v : members) f(Vertex(v));
}

struct edgeset_apply {
  VertexSubset *from_set = nullptr;
  std::function<int(Vertex)> to_filter;
  edgeset_apply() = default;
  explicit edgeset_apply(Schedule &) {}
  edgeset_apply &from(VertexSubset &f) {
    from_set = &f;
    return *this;
  }
  edgeset_apply &to(std::function<int(Vertex)> f) {
    to_filter = std::move(f);
    return *this;
  }
  void apply(GraphT &g, const std::function<void(Vertex, Vertex, int)> &udf) {
    const GraphData &d = *g.d;
    auto visit = [&](int s) {
      for (int e = d.off[s]; e < d.off[s + 1]; ++e) {
        const int t = d.dst[e];
        if (to_filter && !to_filter(Vertex(t))) continue;
        udf(Vertex(s), Vertex(t), d.w[e]);
      }
    };
    if (from_set) {
      const std::vector<int> members = from_set->v;
      for (int s : members) visit(s);
    } else {
      for (int s = 0; s < d.V; ++s) visit(s);
    }
  }
  void apply(GraphT &g, const std::function<void(Vertex, Vertex)> &udf) {
    apply(g, std::function<void(Vertex, Vertex, int)>([&](Vertex s, Vertex t, int) { udf(s, t); }));
  }
  template <typename T>
  void apply_modified(GraphT &g, VertexSubset &to, VertexData<T> &var,
                      const std::function<void(Vertex, Vertex, int)> &udf, bool allow_dupes = true) {
    std::vector<int> out;
    var.out = &out;
    var.dupes = allow_dupes;
    if (!allow_dupes) var.mark.assign((size_t)g.num_vertices, 0);
    apply(g, udf);
    var.out = nullptr;
    to.v = std::move(out);
  }
  template <typename T>
  void apply_modified(GraphT &g, VertexSubset &to, VertexData<T> &var, const std::function<void(Vertex, Vertex)> &udf,
                      bool allow_dupes = true) {
    apply_modified(g, to, var,
                   std::function<void(Vertex, Vertex, int)>([&](Vertex s, Vertex t, int) { udf(s, t); }),
                   allow_dupes);
  }
  void apply_priority(GraphT &g, const std::function<void(Vertex, Vertex, int)> &udf, PriorityQueue &pq) {
    pq.out.clear();
    apply(g, udf);
    pq.frontier = std::move(pq.out);
    pq.out.clear();
  }
};

inline void fuse_kernel(bool, const std::function<void(void)> &body) { body(); }

// ------------------------------------------------------------------ runtime
namespace runtime {
inline GraphT load_graph(const char *path) {
  FILE *f = std::fopen(path, "rb");
  if (!f) {
    std::fprintf(stderr, "cannot open %s\n", path);
    std::exit(1);
  }
  auto g = std::make_shared<GraphData>();
  bool ok = std::fread(&g->V, 4, 1, f) == 1 && std::fread(&g->E, 4, 1, f) == 1 && g->V >= 0 && g->E >= 0;
  if (ok) {
    g->src.resize(g->E);
    g->dst.resize(g->E);
    g->w.resize(g->E);
    g->off.resize((size_t)g->V + 1);
    ok = std::fread(g->src.data(), 4, g->E, f) == (size_t)g->E && std::fread(g->dst.data(), 4, g->E, f) == (size_t)g->E &&
         std::fread(g->w.data(), 4, g->E, f) == (size_t)g->E &&
         std::fread(g->off.data(), 4, (size_t)g->V + 1, f) == (size_t)g->V + 1;
  }
  std::fclose(f);
  if (!ok) {
    std::fprintf(stderr, "truncated graph file %s\n", path);
    std::exit(1);
  }
  g->outdeg.resize(g->V);
  for (int v = 0; v < g->V; ++v) g->outdeg[v] = g->off[v + 1] - g->off[v];
  return GraphT(g);
}
inline VertexSubset new_vertex_subset(int n, int = 0) {
  VertexSubset s;
  s.max_elems = n;
  return s;
}
inline FrontierList new_frontier_list(int) { return FrontierList{}; }
inline std::chrono::steady_clock::time_point &timer_start() {
  static std::chrono::steady_clock::time_point t;
  return t;
}
inline void start_timer() { timer_start() = std::chrono::steady_clock::now(); }
inline double stop_timer() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - timer_start()).count();
}
inline void print_time(double) {}
}  // namespace runtime
}  // namespace graphit

// ------------------------------------------------- builder / pipeline entry
namespace shim {
template <class T>
T arg_from_env(size_t i) {
  const char *e = std::getenv(("GG_SHIM_ARG" + std::to_string(i)).c_str());
  if constexpr (std::is_same<T, char *>::value) {
    static std::string keep[8];
    keep[i % 8] = e ? e : "";
    return const_cast<char *>(keep[i % 8].c_str());
  } else if constexpr (std::is_floating_point<T>::value) {
    return e ? (T)std::atof(e) : T(0);
  } else {
    return e ? (T)std::atoll(e) : T(0);
  }
}
template <class... P, class... S, size_t... I>
void run_with(void (*f)(P...), std::index_sequence<I...>, S &...s) {
  using Tup = std::tuple<std::decay_t<P>...>;
  f(arg_from_env<std::tuple_element_t<I, Tup>>(I)..., s...);
}
}  // namespace shim

namespace builder {
struct builder_context {
  template <class... P, class... S>
  std::function<void()> extract_function_ast(void (*f)(P...), const char *, S... s) {
    static_assert(sizeof...(P) >= sizeof...(S), "more static arguments than parameters");
    return [f, s...]() mutable {
      shim::run_with(f, std::make_index_sequence<sizeof...(P) - sizeof...(S)>{}, s...);
    };
  }
};
}  // namespace builder

namespace pipeline {
inline void run_graphit_pipeline(const std::function<void()> &ast, std::ostream &) {
  ast();
  const char *dir = std::getenv("GG_SHIM_OUT");
  if (!dir) return;
  for (auto &d : graphit::registry()) d.dump(dir);
}
}  // namespace pipeline
