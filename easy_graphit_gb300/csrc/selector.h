// The learned schedule selector: shared constants and internal interfaces.
#pragma once

#include "engine.h"

namespace gg {

constexpr int kSelectorFeatures = 12;
constexpr int kNumLb = 6;
constexpr int kSelectorOutputs = 2 + kNumLb + 3;  // direction, load balancing, frontier type heads
constexpr int kSelectorParams = 16 * 64 + 64 + 64 * 64 + 64 + 64 * 16 + 16;
constexpr int kCandidates = 2 * kNumLb * 3;      // direction x load balancing x frontier type
constexpr int kHeadLoHost[3] = {0, 2, 2 + kNumLb};
constexpr int kHeadHiHost[3] = {2, 2 + kNumLb, kSelectorOutputs};

// Load-balancing head order.
constexpr int kLbChoices[kNumLb] = {GG_LB_TWCE, GG_LB_ETWC, GG_LB_CM, GG_LB_WM, GG_LB_VERTEX_BASED, GG_LB_EDGE_ONLY};

// Candidate c = direction*(3*kNumLb) + lb*3 + frontier -> a schedule derived from `base`.
gg_schedule candidate_schedule(const gg_schedule &base, int dir, int lb, int fr);

// Per-iteration frontier statistics and the running totals the features use.
struct FrontierStats {
  double n = 0, sum_deg = 0, sum_deg2 = 0, max_deg = 0;
};
struct RunTotals {
  double visited_v = 0, visited_e = 0;
  int32_t iteration = 0;
};
gg_status frontier_stats(gg_graph *g, gg_frontier *f, FrontierStats *fs);
void make_features(const gg_graph *g, const FrontierStats &fs, const RunTotals &rt, float x[kSelectorFeatures]);

gg_status selector_decide(gg_selector *s, const float *x_host, int32_t decision[3], cudaStream_t st);

}  // namespace gg
