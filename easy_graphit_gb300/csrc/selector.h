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

// Feature i (0..11) of selector_features, in single precision: the per-level
// form used inside persistent loops, where twelve threads compute one each.
__device__ __forceinline__ float selector_feature(int i, float n, float sd, float sd2, float mx, float vis_v,
                                                  float vis_e, int32_t level, float V, float E) {
  E = E > 1.f ? E : 1.f;
  const float mean = n > 0.f ? sd / n : 0.f;
  switch (i) {
    case 0: return log2f(1.f + n) / 32.f;
    case 1: return log2f(1.f + sd) / 32.f;
    case 2: return log2f(1.f + fmaxf(0.f, V - vis_v)) / 32.f;
    case 3: return log2f(1.f + fmaxf(0.f, E - vis_e)) / 32.f;
    case 4: return log2f(1.f + mean) / 16.f;
    case 5: return log2f(1.f + mx) / 32.f;
    case 6: return log2f(1.f + (n > 0.f ? fmaxf(0.f, sd2 / n - mean * mean) : 0.f)) / 64.f;
    case 7: return (float)min(level, 256) / 256.f;
    case 8: return log2f(V) / 32.f;
    case 9: return log2f(1.f + E) / 32.f;
    case 10: return n / V;
    default: return sd / E;
  }
}

// The network's parameters staged in shared memory once per persistent CTA:
// weights rounded to bf16 (as the tensor-core forward pass reads them), biases
// as they are.  kSelectorParams floats.
__device__ __forceinline__ void selector_stage(const float *__restrict__ p, float *w) {
  for (int i = threadIdx.x; i < kSelectorParams; i += blockDim.x) {
    const bool bias = (i >= kSelB1 && i < kSelW2) || (i >= kSelB2 && i < kSelW3) || i >= kSelB3;
    const float v = __ldg(p + i);
    w[i] = bias ? v : __bfloat162float(__float2bfloat16_rn(v));
  }
}

// Direction head on staged parameters w (selector_stage), computed by one
// warp (the calling one; all 32 lanes call it) with warp-level
// synchronisation only: lane l owns hidden units l and l+32 of both layers,
// layer 2 accumulates its 64 inputs in order, layer 3's two logits are
// reduced across the lanes in a fixed tree.  x: 12 features; h1: 64 floats of
// shared memory.  Returns the same answer in every lane (true = PULL), and in
// every CTA that computes it from the same x.
__device__ __forceinline__ bool selector_pull_warp(const float *w, const float *x, float *h1) {
  auto bf = [](float v) { return __bfloat162float(__float2bfloat16_rn(v)); };
  const int l = threadIdx.x & 31;
  float a0 = 0.f, a1 = 0.f;
#pragma unroll
  for (int k = 0; k < kSelectorFeatures; ++k) {
    const float xk = bf(x[k]);
    a0 += xk * w[kSelW1 + k * kSelHidden + l];
    a1 += xk * w[kSelW1 + k * kSelHidden + l + 32];
  }
  h1[l] = bf(fmaxf(a0 + w[kSelB1 + l], 0.f));
  h1[l + 32] = bf(fmaxf(a1 + w[kSelB1 + l + 32], 0.f));
  __syncwarp();
  a0 = 0.f;
  a1 = 0.f;
#pragma unroll 8
  for (int k = 0; k < kSelHidden; ++k) {
    const float hk = h1[k];
    a0 += hk * w[kSelW2 + k * kSelHidden + l];
    a1 += hk * w[kSelW2 + k * kSelHidden + l + 32];
  }
  __syncwarp();
  const float g0 = bf(fmaxf(a0 + w[kSelB2 + l], 0.f)), g1 = bf(fmaxf(a1 + w[kSelB2 + l + 32], 0.f));
  float z0 = g0 * w[kSelW3 + l * kSelOut] + g1 * w[kSelW3 + (l + 32) * kSelOut];
  float z1 = g0 * w[kSelW3 + l * kSelOut + 1] + g1 * w[kSelW3 + (l + 32) * kSelOut + 1];
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    z0 += __shfl_xor_sync(0xffffffffu, z0, d);
    z1 += __shfl_xor_sync(0xffffffffu, z1, d);
  }
  return z1 + w[kSelB3 + 1] > z0 + w[kSelB3];
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
