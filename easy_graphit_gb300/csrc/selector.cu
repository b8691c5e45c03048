// The learned schedule selector: a bf16 MLP (12 -> 64 -> 64 -> 10) whose three
// heads pick, per iteration, the direction (push/pull), the load-balancing
// strategy (TWCE/ETWC/CM/WM/VERTEX_BASED) and the output frontier type
// (queue/bitmap/boolmap) from frontier statistics.  No reference counterpart.
//
// Forward and backward run on the tensor cores with mma.sync m16n8k16 (bf16
// operands, fp32 accumulation); parameters are fp32 master copies updated by
// Adam.  A block handles 64 samples; gradients are block partial sums added
// atomically.  The layers are padded to multiples of 16 (inputs 12 -> 16,
// outputs 10 -> 16) with zero rows/columns that never change.
#include <cuda_bf16.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "engine.h"
#include "selector.h"

namespace gg {

// Parameter layout (fp32): W1[16][64] b1[64] W2[64][64] b2[64] W3[64][16] b3[16]
constexpr int kIn = 16, kH = 64, kOut = 16;
constexpr int oW1 = 0, oB1 = oW1 + kIn * kH, oW2 = oB1 + kH, oB2 = oW2 + kH * kH, oW3 = oB2 + kH,
              oB3 = oW3 + kH * kOut, kParams = oB3 + kOut;
constexpr int kTileS = 64;  // samples per block

static_assert(kParams == kSelectorParams, "parameter count");

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
  const __nv_bfloat16 l = __float2bfloat16_rn(lo), h = __float2bfloat16_rn(hi);
  return (uint32_t)__bfloat16_as_ushort(l) | ((uint32_t)__bfloat16_as_ushort(h) << 16);
}

__device__ __forceinline__ void mma16816(float c[4], const uint32_t a[4], const uint32_t b[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// C[M][N] (+)= A[M][K] * B[K][N] over fp32 shared-memory operands read through
// accessors (so transposes are free); operands are rounded to bf16 for the
// tensor cores.  M, N multiples of 16 / 8, K a multiple of 16.  Every warp of
// the block takes output tiles round-robin; `store(i, j, v)` receives results.
template <class FA, class FB, class FS>
__device__ __forceinline__ void block_gemm(int M, int N, int K, FA A, FB B, FS store) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  const int tn = N / 8;
  for (int tile = warp; tile < (M / 16) * tn; tile += nwarps) {
    const int m0 = (tile / tn) * 16, n0 = (tile % tn) * 8;
    float c[4] = {0.f, 0.f, 0.f, 0.f};
    for (int k0 = 0; k0 < K; k0 += 16) {
      uint32_t a[4], b[2];
      a[0] = pack2(A(m0 + g, k0 + 2 * t), A(m0 + g, k0 + 2 * t + 1));
      a[1] = pack2(A(m0 + g + 8, k0 + 2 * t), A(m0 + g + 8, k0 + 2 * t + 1));
      a[2] = pack2(A(m0 + g, k0 + 2 * t + 8), A(m0 + g, k0 + 2 * t + 9));
      a[3] = pack2(A(m0 + g + 8, k0 + 2 * t + 8), A(m0 + g + 8, k0 + 2 * t + 9));
      b[0] = pack2(B(k0 + 2 * t, n0 + g), B(k0 + 2 * t + 1, n0 + g));
      b[1] = pack2(B(k0 + 2 * t + 8, n0 + g), B(k0 + 2 * t + 9, n0 + g));
      mma16816(c, a, b);
    }
    store(m0 + g, n0 + 2 * t, c[0]);
    store(m0 + g, n0 + 2 * t + 1, c[1]);
    store(m0 + g + 8, n0 + 2 * t, c[2]);
    store(m0 + g + 8, n0 + 2 * t + 1, c[3]);
  }
}

struct MlpSmem {
  float w1[kIn * kH], w2[kH * kH], w3[kH * kOut];
  float b1[kH], b2[kH], b3[kOut];
  float x[kTileS * kIn];
  float h1[kTileS * kH], h2[kTileS * kH];
  float z[kTileS * kOut];
  float d2[kTileS * kH], d1[kTileS * kH];
};

__device__ void load_params(MlpSmem &s, const float *__restrict__ p) {
  for (int i = threadIdx.x; i < kIn * kH; i += blockDim.x) s.w1[i] = p[oW1 + i];
  for (int i = threadIdx.x; i < kH * kH; i += blockDim.x) s.w2[i] = p[oW2 + i];
  for (int i = threadIdx.x; i < kH * kOut; i += blockDim.x) s.w3[i] = p[oW3 + i];
  for (int i = threadIdx.x; i < kH; i += blockDim.x) {
    s.b1[i] = p[oB1 + i];
    s.b2[i] = p[oB2 + i];
  }
  for (int i = threadIdx.x; i < kOut; i += blockDim.x) s.b3[i] = p[oB3 + i];
}

// Forward pass of a 64-sample tile; x (N x 12 fp32) rows beyond n are zero.
__device__ void forward_tile(MlpSmem &s, const float *__restrict__ x, int row0, int n) {
  for (int i = threadIdx.x; i < kTileS * kIn; i += blockDim.x) {
    const int r = i / kIn, c = i % kIn;
    s.x[i] = (row0 + r < n && c < kSelectorFeatures) ? x[(int64_t)(row0 + r) * kSelectorFeatures + c] : 0.f;
  }
  __syncthreads();
  block_gemm(kTileS, kH, kIn, [&](int i, int k) { return s.x[i * kIn + k]; },
             [&](int k, int j) { return s.w1[k * kH + j]; },
             [&](int i, int j, float v) { s.h1[i * kH + j] = fmaxf(v + s.b1[j], 0.f); });
  __syncthreads();
  block_gemm(kTileS, kH, kH, [&](int i, int k) { return s.h1[i * kH + k]; },
             [&](int k, int j) { return s.w2[k * kH + j]; },
             [&](int i, int j, float v) { s.h2[i * kH + j] = fmaxf(v + s.b2[j], 0.f); });
  __syncthreads();
  block_gemm(kTileS, kOut, kH, [&](int i, int k) { return s.h2[i * kH + k]; },
             [&](int k, int j) { return s.w3[k * kOut + j]; },
             [&](int i, int j, float v) { s.z[i * kOut + j] = v + s.b3[j]; });
  __syncthreads();
}

__global__ void __launch_bounds__(128) k_mlp_forward(const float *__restrict__ p, const float *__restrict__ x,
                                                     int n, float *__restrict__ logits) {
  extern __shared__ float4 smraw[];
  MlpSmem &s = *reinterpret_cast<MlpSmem *>(smraw);
  load_params(s, p);
  const int row0 = blockIdx.x * kTileS;
  forward_tile(s, x, row0, n);
  for (int i = threadIdx.x; i < kTileS * kSelectorOutputs; i += blockDim.x) {
    const int r = i / kSelectorOutputs, c = i % kSelectorOutputs;
    if (row0 + r < n) logits[(int64_t)(row0 + r) * kSelectorOutputs + c] = s.z[r * kOut + c];
  }
}

// Heads: [0,2) direction, [2,7) load balancing, [7,10) frontier type.
__device__ __constant__ int kHeadLo[3] = {kHeadLoHost[0], kHeadLoHost[1], kHeadLoHost[2]};
__device__ __constant__ int kHeadHi[3] = {kHeadHiHost[0], kHeadHiHost[1], kHeadHiHost[2]};

// Forward + backward of the summed softmax cross-entropy of the three heads
// (mean over n samples).  Gradients are added into grad[kParams]; the loss
// into loss[0].
__global__ void __launch_bounds__(128) k_mlp_backward(const float *__restrict__ p, const float *__restrict__ x,
                                                      const int32_t *__restrict__ labels, int n,
                                                      float *__restrict__ grad, float *__restrict__ loss) {
  extern __shared__ float4 smraw[];
  MlpSmem &s = *reinterpret_cast<MlpSmem *>(smraw);
  load_params(s, p);
  const int row0 = blockIdx.x * kTileS;
  forward_tile(s, x, row0, n);
  const float inv_n = 1.f / (float)n;
  // dZ = (softmax - onehot) / n per head, in place in s.z; padded outputs 0.
  float lsum = 0.f;
  for (int i = threadIdx.x; i < kTileS * 3; i += blockDim.x) {
    const int r = i / 3, h = i % 3;
    float *zr = s.z + r * kOut;
    const int lo = kHeadLo[h], hi = kHeadHi[h];
    if (row0 + r >= n) {
      for (int c = lo; c < hi; ++c) zr[c] = 0.f;
      continue;
    }
    const int lab = labels[(int64_t)(row0 + r) * 3 + h];
    float m = -INFINITY;
    for (int c = lo; c < hi; ++c) m = fmaxf(m, zr[c]);
    float se = 0.f;
    for (int c = lo; c < hi; ++c) se += __expf(zr[c] - m);
    lsum += (logf(se) + m - zr[lo + lab]) * inv_n;
    for (int c = lo; c < hi; ++c) zr[c] = (__expf(zr[c] - m) / se - (c == lo + lab ? 1.f : 0.f)) * inv_n;
  }
  for (int i = threadIdx.x; i < kTileS; i += blockDim.x)
    for (int c = kSelectorOutputs; c < kOut; ++c) s.z[i * kOut + c] = 0.f;
  if (lsum != 0.f) atomicAdd(loss, lsum);
  __syncthreads();
  // dW3 = H2^T dZ ; db3 = sum dZ
  block_gemm(kH, kOut, kTileS, [&](int i, int k) { return s.h2[k * kH + i]; },
             [&](int k, int j) { return s.z[k * kOut + j]; },
             [&](int i, int j, float v) { atomicAdd(grad + oW3 + i * kOut + j, v); });
  for (int j = threadIdx.x; j < kOut; j += blockDim.x) {
    float a = 0.f;
    for (int r = 0; r < kTileS; ++r) a += s.z[r * kOut + j];
    atomicAdd(grad + oB3 + j, a);
  }
  // dH2 = dZ W3^T masked by relu'(H2)
  block_gemm(kTileS, kH, kOut, [&](int i, int k) { return s.z[i * kOut + k]; },
             [&](int k, int j) { return s.w3[j * kOut + k]; },
             [&](int i, int j, float v) { s.d2[i * kH + j] = s.h2[i * kH + j] > 0.f ? v : 0.f; });
  __syncthreads();
  block_gemm(kH, kH, kTileS, [&](int i, int k) { return s.h1[k * kH + i]; },
             [&](int k, int j) { return s.d2[k * kH + j]; },
             [&](int i, int j, float v) { atomicAdd(grad + oW2 + i * kH + j, v); });
  for (int j = threadIdx.x; j < kH; j += blockDim.x) {
    float a = 0.f;
    for (int r = 0; r < kTileS; ++r) a += s.d2[r * kH + j];
    atomicAdd(grad + oB2 + j, a);
  }
  // dH1 = dH2 W2^T masked by relu'(H1)
  block_gemm(kTileS, kH, kH, [&](int i, int k) { return s.d2[i * kH + k]; },
             [&](int k, int j) { return s.w2[j * kH + k]; },
             [&](int i, int j, float v) { s.d1[i * kH + j] = s.h1[i * kH + j] > 0.f ? v : 0.f; });
  __syncthreads();
  block_gemm(kIn, kH, kTileS, [&](int i, int k) { return s.x[k * kIn + i]; },
             [&](int k, int j) { return s.d1[k * kH + j]; },
             [&](int i, int j, float v) { atomicAdd(grad + oW1 + i * kH + j, v); });
  for (int j = threadIdx.x; j < kH; j += blockDim.x) {
    float a = 0.f;
    for (int r = 0; r < kTileS; ++r) a += s.d1[r * kH + j];
    atomicAdd(grad + oB1 + j, a);
  }
}

// Adam on the fp32 master parameters; padded rows/columns stay zero.
__global__ void k_adam(float *__restrict__ p, const float *__restrict__ grad, float *__restrict__ m,
                       float *__restrict__ v, float lr, float b1t, float b2t) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kParams; i += gridDim.x * blockDim.x) {
    bool pad = false;
    if (i >= oW1 && i < oB1) pad = (i - oW1) / kH >= kSelectorFeatures;
    if (i >= oW3 && i < oB3) pad = (i - oW3) % kOut >= kSelectorOutputs;
    if (i >= oB3) pad = (i - oB3) >= kSelectorOutputs;
    if (pad) {
      p[i] = 0.f;
      continue;
    }
    const float gi = grad[i];
    m[i] = b1 * m[i] + (1 - b1) * gi;
    v[i] = b2 * v[i] + (1 - b2) * gi * gi;
    const float mh = m[i] / (1 - b1t), vh = v[i] / (1 - b2t);
    p[i] -= lr * mh / (sqrtf(vh) + eps);
  }
}

}  // namespace gg

using namespace gg;

struct gg_selector {
  float *p = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr, *loss = nullptr;
  int64_t steps = 0;
  float *x = nullptr, *logits = nullptr;  // device staging for single-sample inference
  int32_t *labels = nullptr;
  size_t cap = 0;  // rows of x / labels / logits
  ~gg_selector() {
    for (void *q : {(void *)p, (void *)grad, (void *)m, (void *)v, (void *)loss, (void *)x,
                    (void *)logits, (void *)labels})
      if (q) cudaFree(q);
  }
};

namespace gg {

static size_t mlp_smem() { return sizeof(MlpSmem); }

static gg_status ensure_rows(gg_selector *s, size_t n) {
  if (s->cap >= n) return GG_OK;
  for (void *q : {(void *)s->x, (void *)s->logits, (void *)s->labels})
    if (q) cudaFree(q);
  const size_t c = std::max<size_t>(n, 64);
  GG_CUDA(cudaMalloc(&s->x, sizeof(float) * kSelectorFeatures * c));
  GG_CUDA(cudaMalloc(&s->logits, sizeof(float) * kSelectorOutputs * c));
  GG_CUDA(cudaMalloc(&s->labels, sizeof(int32_t) * 3 * c));
  s->cap = c;
  return GG_OK;
}

static gg_status set_smem_attr() {
  static bool done = false;
  if (!done) {
    GG_CUDA(cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mlp_smem()));
    GG_CUDA(cudaFuncSetAttribute(k_mlp_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mlp_smem()));
    done = true;
  }
  return GG_OK;
}

// Logits of n samples already in device memory.
gg_status selector_forward_device(const gg_selector *s, const float *x_dev, int32_t n, float *logits_dev,
                                  cudaStream_t st) {
  GG_TRY(set_smem_attr());
  note_launch();
  k_mlp_forward<<<ceil_div(n, kTileS), 128, mlp_smem(), st>>>(s->p, x_dev, n, logits_dev);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

// Decision for one feature vector on the device: argmax of each head.
gg_status selector_decide(gg_selector *s, const float *x_host, int32_t decision[3], cudaStream_t st) {
  GG_TRY(ensure_rows(s, 1));
  GG_CUDA(cudaMemcpyAsync(s->x, x_host, sizeof(float) * kSelectorFeatures, cudaMemcpyHostToDevice, st));
  GG_TRY(selector_forward_device(s, s->x, 1, s->logits, st));
  float z[kSelectorOutputs];
  GG_CUDA(cudaMemcpyAsync(z, s->logits, sizeof(z), cudaMemcpyDeviceToHost, st));
  GG_CUDA(cudaStreamSynchronize(st));
  for (int h = 0; h < 3; ++h) {
    int best = kHeadLoHost[h];
    for (int c = kHeadLoHost[h]; c < kHeadHiHost[h]; ++c)
      if (z[c] > z[best]) best = c;
    decision[h] = best - kHeadLoHost[h];
  }
  return GG_OK;
}

}  // namespace gg

extern "C" {

gg_status gg_selector_create(int64_t seed, gg_selector **out) {
  GG_CHECK_ARG(out, "out is NULL");
  auto s = std::make_unique<gg_selector>();
  GG_CUDA(cudaMalloc(&s->p, sizeof(float) * kParams));
  GG_CUDA(cudaMalloc(&s->grad, sizeof(float) * kParams));
  GG_CUDA(cudaMalloc(&s->m, sizeof(float) * kParams));
  GG_CUDA(cudaMalloc(&s->v, sizeof(float) * kParams));
  GG_CUDA(cudaMalloc(&s->loss, sizeof(float)));
  // He-uniform initialisation on the live rows/columns, zero padding.
  std::vector<float> h(kParams, 0.f);
  std::mt19937 rng((uint32_t)seed);
  auto fill = [&](int off, int rows, int cols, int live_rows, int live_cols, int fan_in) {
    std::uniform_real_distribution<float> u(-std::sqrt(6.f / fan_in), std::sqrt(6.f / fan_in));
    for (int r = 0; r < rows; ++r)
      for (int c = 0; c < cols; ++c) h[off + r * cols + c] = (r < live_rows && c < live_cols) ? u(rng) : 0.f;
  };
  fill(oW1, kIn, kH, kSelectorFeatures, kH, kSelectorFeatures);
  fill(oW2, kH, kH, kH, kH, kH);
  fill(oW3, kH, kOut, kH, kSelectorOutputs, kH);
  GG_CUDA(cudaMemcpy(s->p, h.data(), sizeof(float) * kParams, cudaMemcpyHostToDevice));
  GG_CUDA(cudaMemset(s->m, 0, sizeof(float) * kParams));
  GG_CUDA(cudaMemset(s->v, 0, sizeof(float) * kParams));
  *out = s.release();
  return GG_OK;
}

gg_status gg_selector_destroy(gg_selector *s) {
  delete s;
  return GG_OK;
}

gg_status gg_selector_get_params(const gg_selector *s, float *out, int32_t n) {
  GG_CHECK_ARG(s && out && n == kParams, "parameter buffer must hold gg_selector_num_params() floats");
  GG_CUDA(cudaMemcpy(out, s->p, sizeof(float) * kParams, cudaMemcpyDeviceToHost));
  return GG_OK;
}

gg_status gg_selector_set_params(gg_selector *s, const float *in, int32_t n) {
  GG_CHECK_ARG(s && in && n == kParams, "parameter buffer must hold gg_selector_num_params() floats");
  GG_CUDA(cudaMemcpy(s->p, in, sizeof(float) * kParams, cudaMemcpyHostToDevice));
  return GG_OK;
}

int32_t gg_selector_num_params(void) { return kParams; }

gg_status gg_selector_forward(gg_selector *s, const float *x, int32_t n, float *logits) {
  GG_CHECK_ARG(s && x && logits && n >= 1, "bad arguments");
  GG_TRY(ensure_rows(s, n));
  GG_CUDA(cudaMemcpy(s->x, x, sizeof(float) * kSelectorFeatures * n, cudaMemcpyDefault));
  GG_TRY(selector_forward_device(s, s->x, n, s->logits, nullptr));
  GG_CUDA(cudaMemcpy(logits, s->logits, sizeof(float) * kSelectorOutputs * n, cudaMemcpyDefault));
  return GG_OK;
}

// Gradient of the mean loss at the current parameters (for checking).
// Labels index the heads' logits inside the kernels: every one must lie in
// its head (host or device memory).
static gg_status check_labels(const int32_t *labels, int32_t n) {
  std::vector<int32_t> h((size_t)n * 3);
  GG_CUDA(cudaMemcpy(h.data(), labels, sizeof(int32_t) * h.size(), cudaMemcpyDefault));
  for (size_t i = 0; i < h.size(); ++i) {
    const int hd = (int)(i % 3);
    if (h[i] < 0 || h[i] >= kHeadHiHost[hd] - kHeadLoHost[hd])
      return set_error(GG_ERR_INVALID, "label %d of head %d out of range", h[i], hd);
  }
  return GG_OK;
}

gg_status gg_selector_grad(gg_selector *s, const float *x, const int32_t *labels, int32_t n, float *grad,
                           float *loss) {
  GG_CHECK_ARG(s && x && labels && grad && n >= 1, "bad arguments");
  GG_TRY(check_labels(labels, n));
  GG_TRY(ensure_rows(s, n));
  GG_TRY(set_smem_attr());
  GG_CUDA(cudaMemcpy(s->x, x, sizeof(float) * kSelectorFeatures * n, cudaMemcpyDefault));
  GG_CUDA(cudaMemcpy(s->labels, labels, sizeof(int32_t) * 3 * n, cudaMemcpyDefault));
  GG_CUDA(cudaMemset(s->grad, 0, sizeof(float) * kParams));
  GG_CUDA(cudaMemset(s->loss, 0, sizeof(float)));
  note_launch();
  k_mlp_backward<<<ceil_div(n, kTileS), 128, mlp_smem()>>>(s->p, s->x, s->labels, n, s->grad, s->loss);
  GG_CUDA(cudaGetLastError());
  GG_CUDA(cudaMemcpy(grad, s->grad, sizeof(float) * kParams, cudaMemcpyDeviceToHost));
  if (loss) GG_CUDA(cudaMemcpy(loss, s->loss, sizeof(float), cudaMemcpyDeviceToHost));
  return GG_OK;
}

// Full-batch Adam for `epochs` steps; *final_loss = loss of the last step.
gg_status gg_selector_train(gg_selector *s, const float *x, const int32_t *labels, int32_t n,
                            int32_t epochs, float lr, float *final_loss) {
  GG_CHECK_ARG(s && x && labels && n >= 1 && epochs >= 1, "bad arguments");
  GG_TRY(check_labels(labels, n));
  GG_TRY(ensure_rows(s, n));
  GG_TRY(set_smem_attr());
  GG_CUDA(cudaMemcpy(s->x, x, sizeof(float) * kSelectorFeatures * n, cudaMemcpyDefault));
  GG_CUDA(cudaMemcpy(s->labels, labels, sizeof(int32_t) * 3 * n, cudaMemcpyDefault));
  for (int32_t e = 0; e < epochs; ++e) {
    GG_CUDA(cudaMemsetAsync(s->grad, 0, sizeof(float) * kParams));
    GG_CUDA(cudaMemsetAsync(s->loss, 0, sizeof(float)));
    note_launch();
    k_mlp_backward<<<ceil_div(n, kTileS), 128, mlp_smem()>>>(s->p, s->x, s->labels, n, s->grad, s->loss);
    ++s->steps;
    const float b1t = (float)std::pow(0.9, (double)s->steps), b2t = (float)std::pow(0.999, (double)s->steps);
    note_launch();
    k_adam<<<ceil_div(kParams, 256), 256>>>(s->p, s->grad, s->m, s->v, lr, b1t, b2t);
  }
  GG_CUDA(cudaGetLastError());
  if (final_loss) GG_CUDA(cudaMemcpy(final_loss, s->loss, sizeof(float), cudaMemcpyDeviceToHost));
  GG_CUDA(cudaDeviceSynchronize());
  return GG_OK;
}

// File format: "GGSEL1\0\0" magic, int32 count, count fp32 parameters.
gg_status gg_selector_save(const gg_selector *s, const char *path) {
  GG_CHECK_ARG(s && path, "bad arguments");
  std::vector<float> h(kParams);
  GG_CUDA(cudaMemcpy(h.data(), s->p, sizeof(float) * kParams, cudaMemcpyDeviceToHost));
  FILE *f = fopen(path, "wb");
  if (!f) return set_error(GG_ERR_IO, "cannot create %s", path);
  const char magic[8] = {'G', 'G', 'S', 'E', 'L', '1', 0, 0};
  const int32_t n = kParams;
  bool ok = fwrite(magic, 1, 8, f) == 8 && fwrite(&n, 4, 1, f) == 1 &&
            fwrite(h.data(), 4, kParams, f) == (size_t)kParams;
  ok = (fclose(f) == 0) && ok;
  if (!ok) return set_error(GG_ERR_IO, "short write to %s", path);
  return GG_OK;
}

gg_status gg_selector_load(const char *path, gg_selector **out) {
  GG_CHECK_ARG(path && out, "bad arguments");
  FILE *f = fopen(path, "rb");
  if (!f) return set_error(GG_ERR_IO, "cannot open %s", path);
  char magic[8];
  int32_t n = 0;
  std::vector<float> h(kParams);
  bool ok = fread(magic, 1, 8, f) == 8 && memcmp(magic, "GGSEL1", 6) == 0 && fread(&n, 4, 1, f) == 1 &&
            n == kParams && fread(h.data(), 4, kParams, f) == (size_t)kParams;
  fclose(f);
  if (!ok) return set_error(GG_ERR_IO, "%s is not a selector parameter file", path);
  gg_selector *s = nullptr;
  GG_TRY(gg_selector_create(0, &s));
  const cudaError_t e = cudaMemcpy(s->p, h.data(), sizeof(float) * kParams, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    delete s;
    return set_error(GG_ERR_CUDA, "%s", cudaGetErrorString(e));
  }
  *out = s;
  return GG_OK;
}

}  // extern "C"
