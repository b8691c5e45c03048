/*
 * graphit/schedule.h -- the GraphIt GPU scheduling API in C++ over libgg.so.
 *
 * Same names, enumerators (in the same order) and defaults as easy_graphit's
 * include/graphit/schedule.h:26-139 and src/graphit/schedule.cpp:5-12, so
 * code written against the reference's schedules compiles against this one.
 * Differences: load_balancing_type gains ETWC (appended); the threshold of a
 * HybridGPUSchedule binds to a plain float the caller keeps changing
 * (bindThreshold(float&), read at every decision) where the reference binds a
 * staged dyn_var<float>; LearnedGPUSchedule is new.
 */
#ifndef GRAPHIT_GB300_SCHEDULE_H
#define GRAPHIT_GB300_SCHEDULE_H

#include "../gg.h"

namespace graphit {

// Abstract schedule (schedule.h:11-14).
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

// schedule.h:26-118.  Enumerator values equal gg.h's GG_* constants.
struct SimpleGPUSchedule : public Schedule {
  static inline int default_max_cta = 60;    // schedule.cpp:6
  static inline int default_cta_size = 512;  // schedule.cpp:5

  enum class direction_type { PUSH, PULL };
  enum class pull_frontier_rep_type { BITMAP, BOOLMAP };
  enum class frontier_creation_type { SPARSE, BITMAP, BOOLMAP };
  enum class deduplication_type { DISABLED, ENABLED };
  enum class deduplication_strategy_type { FUSED, UNFUSED };
  enum class load_balancing_type { VERTEX_BASED, TWC, TWCE, WM, CM, STRICT, EDGE_ONLY, ETWC };
  enum class edge_blocking_type { BLOCKED, UNBLOCKED };
  enum class kernel_fusion_type { DISABLED, ENABLED };

  direction_type direction;
  pull_frontier_rep_type pull_frontier_rep;
  frontier_creation_type frontier_creation;
  deduplication_type deduplication = deduplication_type::DISABLED;
  deduplication_strategy_type deduplication_stategy = deduplication_strategy_type::FUSED;  // (sic) the reference's member name
  load_balancing_type load_balancing;
  edge_blocking_type edge_blocking;
  int block_size;
  kernel_fusion_type kernel_fusion = kernel_fusion_type::DISABLED;
  int max_cta;
  int cta_size;

  SimpleGPUSchedule() {
    direction = direction_type::PUSH;
    load_balancing = load_balancing_type::VERTEX_BASED;
    edge_blocking = edge_blocking_type::UNBLOCKED;
    frontier_creation = frontier_creation_type::SPARSE;
    pull_frontier_rep = pull_frontier_rep_type::BOOLMAP;
    block_size = -1;
    max_cta = default_max_cta;
    cta_size = default_cta_size;
  }

  void configDirection(direction_type dir, pull_frontier_rep_type pf = pull_frontier_rep_type::BOOLMAP) {
    direction = dir;
    if (direction == direction_type::PULL) pull_frontier_rep = pf;
  }
  void configFrontierCreation(frontier_creation_type fc) { frontier_creation = fc; }
  // The strategy argument is new: the reference picks fused dedup on the
  // device and the unfused dedup_frontier_perfect pass on the host
  // (operators.h:144-145,171-172).
  void configDeduplication(deduplication_type dedup,
                           deduplication_strategy_type strategy = deduplication_strategy_type::FUSED) {
    deduplication = dedup;
    deduplication_stategy = strategy;
  }
  void configLoadBalancing(load_balancing_type lb, edge_blocking_type eb = edge_blocking_type::UNBLOCKED,
                           int bs = -1) {
    load_balancing = lb;
    if (lb == load_balancing_type::EDGE_ONLY) {
      edge_blocking = eb;
      block_size = bs;
    }
  }
  void configKernelFusion(kernel_fusion_type kf) { kernel_fusion = kf; }

  // The C ABI's POD mirror.
  gg_schedule to_c() const {
    gg_schedule s;
    s.direction = static_cast<int32_t>(direction);
    s.pull_frontier_rep = static_cast<int32_t>(pull_frontier_rep);
    s.frontier_creation = static_cast<int32_t>(frontier_creation);
    s.deduplication = static_cast<int32_t>(deduplication);
    s.deduplication_strategy = static_cast<int32_t>(deduplication_stategy);
    s.load_balancing = static_cast<int32_t>(load_balancing);
    s.edge_blocking = static_cast<int32_t>(edge_blocking);
    s.block_size = block_size;
    s.kernel_fusion = static_cast<int32_t>(kernel_fusion);
    s.max_cta = max_cta;
    s.cta_size = cta_size;
    return s;
  }
};

// schedule.h:122-139: s1 while |frontier| <= threshold * V, else s2
// (operators.cpp:516-532, operators.h:116-132).
struct HybridGPUSchedule : public Schedule {
  Schedule *s1;
  Schedule *s2;
  const float *threshold = nullptr;  // bound by bindThreshold
  float static_threshold = 0.0f;

  HybridGPUSchedule(Schedule &_s1, Schedule &_s2) : s1(&_s1), s2(&_s2) {}
  void configThreshold(float t) {
    threshold = nullptr;
    static_threshold = t;
  }
  // The caller keeps t alive and may change it between runs.
  void bindThreshold(float &t) { threshold = &t; }
  float current_threshold() const { return threshold ? *threshold : static_threshold; }
};

// No reference counterpart: the learned per-iteration selector (gg.h
// gg_selector_*) with the hand-written schedule as its fallback.
struct LearnedGPUSchedule : public Schedule {
  const gg_selector *selector;
  SimpleGPUSchedule fallback;
  explicit LearnedGPUSchedule(const gg_selector *sel, const SimpleGPUSchedule &fb = SimpleGPUSchedule())
      : selector(sel), fallback(fb) {}
};

// The C form of a simple schedule (a default one for anything else).
inline gg_schedule simple_schedule_c(Schedule *s) {
  const SimpleGPUSchedule *p = s_to<SimpleGPUSchedule>(s);
  return p ? p->to_c() : SimpleGPUSchedule().to_c();
}

// The app-level schedule the whole-app entry points (gg_bfs ... gg_bc) take;
// `fuse` is the app's fuse_kernel(to_fuse, ...) flag (operators.cpp:652-672).
// A hybrid schedule's bound threshold is read here, at the call.
inline gg_app_schedule app_schedule(Schedule &s, bool fuse) {
  gg_app_schedule a{};
  a.fuse = fuse ? 1 : 0;
  if (auto *h = s_to<HybridGPUSchedule>(&s)) {
    a.kind = GG_SCHED_HYBRID;
    a.threshold = h->current_threshold();
    a.s1 = simple_schedule_c(h->s1);
    a.s2 = simple_schedule_c(h->s2);
  } else if (auto *l = s_to<LearnedGPUSchedule>(&s)) {
    a.kind = GG_SCHED_LEARNED;
    a.fuse = 0;
    a.s1 = a.s2 = l->fallback.to_c();
    a.selector = l->selector;
  } else {
    a.kind = GG_SCHED_SIMPLE;
    a.s1 = a.s2 = simple_schedule_c(&s);
  }
  return a;
}

}  // namespace graphit

#endif  // GRAPHIT_GB300_SCHEDULE_H
