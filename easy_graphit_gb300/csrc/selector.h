// The learned schedule selector: shared constants and internal interfaces.
#pragma once

#include <cuda_bf16.h>

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
// The network's fp32 master parameters on the device (layout below).
const float *selector_params(const gg_selector *s);

// Parameter layout (fp32): W1[16][64] b1[64] W2[64][64] b2[64] W3[64][16] b3[16]
// (inputs and outputs padded to 16; the padding is zero).
constexpr int kSelIn = 16, kSelHidden = 64, kSelOut = 16;
constexpr int kSelW1 = 0, kSelB1 = kSelW1 + kSelIn * kSelHidden, kSelW2 = kSelB1 + kSelHidden,
              kSelB2 = kSelW2 + kSelHidden * kSelHidden, kSelW3 = kSelB2 + kSelHidden,
              kSelB3 = kSelW3 + kSelHidden * kSelOut;

// The 12 selector features of one frontier (make_features of selector_data.cu,
// on the device): frontier size n, its out-degree sum sd, sum of squares sd2
// and maximum mx, the vertices and edges visited before it, and its level.
__device__ __forceinline__ void selector_features(float *x, double n, double sd, double sd2, double mx,
                                                  double vis_v, double vis_e, int32_t level, double V,
                                                  double E) {
  E = E > 1 ? E : 1;
  const double mean = n > 0 ? sd / n : 0.0;
  const double var = n > 0 ? fmax(0.0, sd2 / n - mean * mean) : 0.0;
  x[0] = (float)(log2(1 + n) / 32);
  x[1] = (float)(log2(1 + sd) / 32);
  x[2] = (float)(log2(1 + fmax(0.0, V - vis_v)) / 32);
  x[3] = (float)(log2(1 + fmax(0.0, E - vis_e)) / 32);
  x[4] = (float)(log2(1 + mean) / 16);
  x[5] = (float)(log2(1 + mx) / 32);
  x[6] = (float)(log2(1 + var) / 64);
  x[7] = (float)(min(level, 256) / 256.0);
  x[8] = (float)(log2(V) / 32);
  x[9] = (float)(log2(1 + E) / 32);
  x[10] = (float)(n / V);
  x[11] = (float)(sd / E);
}

// Direction head of the network on one feature vector x (12 floats), computed
// by the calling CTA inside a persistent kernel: fp32 accumulation over
// bf16-rounded operands, as the tensor-core forward pass computes it.  h is
// 2*64 floats of shared memory.  Every thread of the CTA calls it and gets the
// same answer: true when the network picks PULL.
static __device__ __noinline__ bool selector_pull(const float *__restrict__ p, const float *x, float *h) {
  auto bf = [](float v) { return __bfloat162float(__float2bfloat16_rn(v)); };
  const int j = threadIdx.x;
  if (j < kSelHidden) {
    float a = 0.f;
    for (int k = 0; k < kSelectorFeatures; ++k) a += bf(x[k]) * bf(__ldg(p + kSelW1 + k * kSelHidden + j));
    h[j] = fmaxf(a + __ldg(p + kSelB1 + j), 0.f);
  }
  __syncthreads();
  if (j < kSelHidden) {
    float a = 0.f;
    for (int k = 0; k < kSelHidden; ++k) a += bf(h[k]) * bf(__ldg(p + kSelW2 + k * kSelHidden + j));
    h[kSelHidden + j] = fmaxf(a + __ldg(p + kSelB2 + j), 0.f);
  }
  __syncthreads();
  float z = 0.f;
  if (j < 2) {
    for (int k = 0; k < kSelHidden; ++k) z += bf(h[kSelHidden + k]) * bf(__ldg(p + kSelW3 + k * kSelOut + j));
    z += __ldg(p + kSelB3 + j);
  }
  __syncthreads();
  if (j < 2) h[j] = z;  // the two direction logits (push, pull)
  __syncthreads();
  const bool pull = h[1] > h[0];
  __syncthreads();
  return pull;
}

}  // namespace gg
