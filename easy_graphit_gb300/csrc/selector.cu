// The learned schedule selector: a bf16 MLP (12 -> 64 -> 64 -> 11) whose three
// heads pick, per iteration, the direction (push/pull), the load-balancing
// strategy (TWCE/ETWC/CM/WM/VERTEX_BASED/EDGE_ONLY) and the output frontier
// type (queue/bitmap/boolmap) from frontier statistics.  No reference
// counterpart.
//
// Every matrix product of the forward and backward passes runs on the 5th-gen
// tensor cores: operands are staged in shared memory as bf16 in the canonical
// no-swizzle K-major layout (8-row x 16-byte core matrices), one thread issues
// tcgen05.mma (kind::f16, bf16 x bf16 -> fp32, M = 128) into a TMEM accumulator,
// tcgen05.commit signals an mbarrier, and each warp reads its 32 accumulator
// lanes back with tcgen05.ld for the epilogue (bias, ReLU, gradient atomics).
// Parameters are fp32 master copies updated by Adam.  A block handles 64
// samples; gradients are block partial sums added atomically.  The layers are
// padded to multiples of 16 (inputs 12 -> 16, outputs 11 -> 16) with zero
// rows/columns that never change.
#include <cuda_bf16.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "engine.h"
#include "selector.h"

namespace gg {

// Parameter layout: selector.h (W1[16][64] b1[64] W2[64][64] b2[64] W3[64][16] b3[16]).
constexpr int kIn = kSelIn, kH = kSelHidden, kOut = kSelOut;
constexpr int oW1 = kSelW1, oB1 = kSelB1, oW2 = kSelW2, oB2 = kSelB2, oW3 = kSelW3, oB3 = kSelB3,
              kParams = oB3 + kOut;
constexpr int kTileS = 64;  // samples per block

static_assert(kParams == kSelectorParams, "parameter count");

constexpr int kTcCols = 64;         // TMEM columns per block (N <= 64)
constexpr int kStageRows = 128;     // the MMA's M: rows beyond a product's M are zero
constexpr int kStageK = 64;         // largest K of the network's products
constexpr uint64_t kTcWaitNs = 1000000000ull;  // 1 s bound on an MMA completion wait

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Element offset of (row r, k) in the canonical K-major no-swizzle layout:
// 8 x 8 bf16 core matrices (128 contiguous bytes), consecutive along K
// (leading byte offset 128), 8-row groups K/8 cores apart (stride byte offset).
__device__ __forceinline__ int canon(int r, int k, int K) {
  return (((r >> 3) * (K >> 3) + (k >> 3)) << 6) + ((r & 7) << 3) + (k & 7);
}

// tcgen05 shared-memory matrix descriptor: start, leading / stride byte
// offsets (>> 4), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t tc_sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: fp32 accumulator, bf16 A and B, both
// K-major, N >> 3 and M >> 4.
__host__ __device__ constexpr uint32_t tc_idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ uint64_t gtime_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Waits for the completion of the mbarrier phase with the given parity; false
// after kTcWaitNs.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
  const uint64_t t0 = gtime_ns();
  for (uint32_t spin = 0;; ++spin) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.b32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
    if ((spin & 63u) == 63u && gtime_ns() - t0 > kTcWaitNs) return false;
  }
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 lanes x 16 columns of fp32 accumulator: this thread's row, 16 values.
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t u[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(u[0]), "=r"(u[1]), "=r"(u[2]), "=r"(u[3]), "=r"(u[4]), "=r"(u[5]), "=r"(u[6]), "=r"(u[7]),
        "=r"(u[8]), "=r"(u[9]), "=r"(u[10]), "=r"(u[11]), "=r"(u[12]), "=r"(u[13]), "=r"(u[14]), "=r"(u[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(u[i]);
}

// Tensor-core state of one block: operand staging, the accumulator's TMEM
// address, the completion mbarrier and its phase.
struct TcState {
  __nv_bfloat16 a[kStageRows * kStageK];
  __nv_bfloat16 b[kH * kStageK];
  uint64_t mbar;
  uint32_t tmem;
  uint32_t phase;
  int32_t failed;
};

// Block-wide: allocate the TMEM accumulator (warp 0) and set up the mbarrier.
__device__ void tc_begin(TcState &t) {
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&t.tmem)),
                 "r"(kTcCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&t.mbar)), "r"(1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    t.phase = 0;
    t.failed = 0;
  }
  for (int i = threadIdx.x; i < kStageRows * kStageK; i += blockDim.x) t.a[i] = __float2bfloat16_rn(0.f);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
}

// Block-wide: if an MMA wait timed out, wait once more (bounded) for it, then
// free the TMEM columns (warp 0).
__device__ void tc_end(TcState &t, int32_t *err) {
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (t.failed) {
    if (threadIdx.x == 0) {
      atomicOr(err, 1);
      mbar_wait(smem_u32(&t.mbar), t.phase);
    }
    __syncthreads();
  }
  if (threadIdx.x < 32)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(t.tmem), "r"(kTcCols) : "memory");
}

// C[M][N] = A[M][K] * B[K][N] on the tensor cores, operands read through
// accessors from fp32 shared memory (so transposes are free) and rounded to
// bf16; M <= 128, N in {16, 32, 48, 64}, K a multiple of 16 up to 64.
// `store(i, j, v)` receives every result with i < M.  Block of 128 threads.
template <class FA, class FB, class FS>
__device__ __forceinline__ void tc_gemm(TcState &t, int M, int N, int K, FA A, FB B, FS store) {
  __syncthreads();  // operands written; the staging buffers are free
  if (t.failed) return;
  for (int idx = threadIdx.x; idx < M * K; idx += blockDim.x) {
    const int i = idx / K, k = idx % K;
    t.a[canon(i, k, K)] = __float2bfloat16_rn(A(i, k));
  }
  for (int idx = threadIdx.x; idx < N * K; idx += blockDim.x) {
    const int j = idx / K, k = idx % K;
    t.b[canon(j, k, K)] = __float2bfloat16_rn(B(k, j));
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // staging visible to the tensor cores
  __syncthreads();
  const uint32_t mbar = smem_u32(&t.mbar);
  if (threadIdx.x == 0) {
    tc_fence_after();
    const uint32_t sbo = (uint32_t)(K / 8) * 128u, abase = smem_u32(t.a), bbase = smem_u32(t.b);
    const uint32_t idesc = tc_idesc(kStageRows, N);
    for (int kk = 0; kk < K / 16; ++kk) {
      const uint64_t ad = tc_sdesc(abase + 256u * kk, 128u, sbo), bd = tc_sdesc(bbase + 256u * kk, 128u, sbo);
      asm volatile(
          "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
              t.tmem),
          "l"(ad), "l"(bd), "r"(idesc), "r"((uint32_t)(kk > 0))
          : "memory");
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
  }
  const bool ok = mbar_wait(mbar, t.phase);
  __syncthreads();
  if (threadIdx.x == 0) {
    if (ok)
      t.phase ^= 1u;
    else
      t.failed = 1;
  }
  __syncthreads();
  if (t.failed) return;
  tc_fence_after();
  const int warp = threadIdx.x >> 5, row = warp * 32 + (threadIdx.x & 31);
  for (int c0 = 0; c0 < N; c0 += 16) {
    float v[16];
    tc_ld16(t.tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
    if (row < M) {
#pragma unroll
      for (int j = 0; j < 16; ++j) store(row, c0 + j, v[j]);
    }
  }
  tc_fence_before();
}

struct MlpSmem {
  TcState tc;
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
  tc_gemm(s.tc, kTileS, kH, kIn, [&](int i, int k) { return s.x[i * kIn + k]; },
             [&](int k, int j) { return s.w1[k * kH + j]; },
             [&](int i, int j, float v) { s.h1[i * kH + j] = fmaxf(v + s.b1[j], 0.f); });
  __syncthreads();
  tc_gemm(s.tc, kTileS, kH, kH, [&](int i, int k) { return s.h1[i * kH + k]; },
             [&](int k, int j) { return s.w2[k * kH + j]; },
             [&](int i, int j, float v) { s.h2[i * kH + j] = fmaxf(v + s.b2[j], 0.f); });
  __syncthreads();
  tc_gemm(s.tc, kTileS, kOut, kH, [&](int i, int k) { return s.h2[i * kH + k]; },
             [&](int k, int j) { return s.w3[k * kOut + j]; },
             [&](int i, int j, float v) { s.z[i * kOut + j] = v + s.b3[j]; });
  __syncthreads();
}

__global__ void __launch_bounds__(128) k_mlp_forward(const float *__restrict__ p, const float *__restrict__ x,
                                                     int n, float *__restrict__ logits, int32_t *err) {
  extern __shared__ float4 smraw[];
  MlpSmem &s = *reinterpret_cast<MlpSmem *>(smraw);
  tc_begin(s.tc);
  load_params(s, p);
  const int row0 = blockIdx.x * kTileS;
  forward_tile(s, x, row0, n);
  for (int i = threadIdx.x; i < kTileS * kSelectorOutputs; i += blockDim.x) {
    const int r = i / kSelectorOutputs, c = i % kSelectorOutputs;
    if (row0 + r < n) logits[(int64_t)(row0 + r) * kSelectorOutputs + c] = s.z[r * kOut + c];
  }
  tc_end(s.tc, err);
}

// Heads: [0,2) direction, [2,7) load balancing, [7,10) frontier type.
__device__ __constant__ int kHeadLo[3] = {kHeadLoHost[0], kHeadLoHost[1], kHeadLoHost[2]};
__device__ __constant__ int kHeadHi[3] = {kHeadHiHost[0], kHeadHiHost[1], kHeadHiHost[2]};

// Forward + backward of the summed softmax cross-entropy of the three heads
// (mean over n samples).  Gradients are added into grad[kParams]; the loss
// into loss[0].
__global__ void __launch_bounds__(128) k_mlp_backward(const float *__restrict__ p, const float *__restrict__ x,
                                                      const int32_t *__restrict__ labels, int n,
                                                      float *__restrict__ grad, float *__restrict__ loss,
                                                      int32_t *err) {
  extern __shared__ float4 smraw[];
  MlpSmem &s = *reinterpret_cast<MlpSmem *>(smraw);
  tc_begin(s.tc);
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
  tc_gemm(s.tc, kH, kOut, kTileS, [&](int i, int k) { return s.h2[k * kH + i]; },
             [&](int k, int j) { return s.z[k * kOut + j]; },
             [&](int i, int j, float v) { atomicAdd(grad + oW3 + i * kOut + j, v); });
  for (int j = threadIdx.x; j < kOut; j += blockDim.x) {
    float a = 0.f;
    for (int r = 0; r < kTileS; ++r) a += s.z[r * kOut + j];
    atomicAdd(grad + oB3 + j, a);
  }
  // dH2 = dZ W3^T masked by relu'(H2)
  tc_gemm(s.tc, kTileS, kH, kOut, [&](int i, int k) { return s.z[i * kOut + k]; },
             [&](int k, int j) { return s.w3[j * kOut + k]; },
             [&](int i, int j, float v) { s.d2[i * kH + j] = s.h2[i * kH + j] > 0.f ? v : 0.f; });
  __syncthreads();
  tc_gemm(s.tc, kH, kH, kTileS, [&](int i, int k) { return s.h1[k * kH + i]; },
             [&](int k, int j) { return s.d2[k * kH + j]; },
             [&](int i, int j, float v) { atomicAdd(grad + oW2 + i * kH + j, v); });
  for (int j = threadIdx.x; j < kH; j += blockDim.x) {
    float a = 0.f;
    for (int r = 0; r < kTileS; ++r) a += s.d2[r * kH + j];
    atomicAdd(grad + oB2 + j, a);
  }
  // dH1 = dH2 W2^T masked by relu'(H1)
  tc_gemm(s.tc, kTileS, kH, kH, [&](int i, int k) { return s.d2[i * kH + k]; },
             [&](int k, int j) { return s.w2[j * kH + k]; },
             [&](int i, int j, float v) { s.d1[i * kH + j] = s.h1[i * kH + j] > 0.f ? v : 0.f; });
  __syncthreads();
  tc_gemm(s.tc, kIn, kH, kTileS, [&](int i, int k) { return s.x[k * kIn + i]; },
             [&](int k, int j) { return s.d1[k * kH + j]; },
             [&](int i, int j, float v) { atomicAdd(grad + oW1 + i * kH + j, v); });
  for (int j = threadIdx.x; j < kH; j += blockDim.x) {
    float a = 0.f;
    for (int r = 0; r < kTileS; ++r) a += s.d1[r * kH + j];
    atomicAdd(grad + oB1 + j, a);
  }
  tc_end(s.tc, err);
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
  int32_t *err = nullptr;  // device: non-zero after a tensor-core wait timed out
  size_t cap = 0;  // rows of x / labels / logits
  ~gg_selector() {
    for (void *q : {(void *)p, (void *)grad, (void *)m, (void *)v, (void *)loss, (void *)x,
                    (void *)logits, (void *)labels, (void *)err})
      if (q) cudaFree(q);
  }
};

namespace gg {

static size_t mlp_smem() { return sizeof(MlpSmem); }

// A tensor-core completion wait that gave up leaves its mark in s->err.
static gg_status check_tc(const gg_selector *s) {
  int32_t e = 0;
  GG_CUDA(cudaMemcpy(&e, s->err, sizeof(e), cudaMemcpyDeviceToHost));
  if (e) return set_error(GG_ERR_TIMEOUT, "selector: a tensor-core MMA did not complete within its time limit");
  return GG_OK;
}

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
  k_mlp_forward<<<ceil_div(n, kTileS), 128, mlp_smem(), st>>>(s->p, x_dev, n, logits_dev, s->err);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

const float *selector_params(const gg_selector *s) { return s->p; }

// Decision for one feature vector on the device: argmax of each head.
gg_status selector_decide(gg_selector *s, const float *x_host, int32_t decision[3], cudaStream_t st) {
  GG_TRY(ensure_rows(s, 1));
  GG_CUDA(cudaMemcpyAsync(s->x, x_host, sizeof(float) * kSelectorFeatures, cudaMemcpyHostToDevice, st));
  GG_TRY(selector_forward_device(s, s->x, 1, s->logits, st));
  float z[kSelectorOutputs];
  GG_CUDA(cudaMemcpyAsync(z, s->logits, sizeof(z), cudaMemcpyDeviceToHost, st));
  GG_CUDA(cudaStreamSynchronize(st));
  GG_TRY(check_tc(s));
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
  GG_CUDA(cudaMalloc(&s->err, sizeof(int32_t)));
  GG_CUDA(cudaMemset(s->err, 0, sizeof(int32_t)));
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
  return check_tc(s);
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
  k_mlp_backward<<<ceil_div(n, kTileS), 128, mlp_smem()>>>(s->p, s->x, s->labels, n, s->grad, s->loss, s->err);
  GG_CUDA(cudaGetLastError());
  GG_TRY(check_tc(s));
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
    k_mlp_backward<<<ceil_div(n, kTileS), 128, mlp_smem()>>>(s->p, s->x, s->labels, n, s->grad, s->loss,
                                                              s->err);
    ++s->steps;
    const float b1t = (float)std::pow(0.9, (double)s->steps), b2t = (float)std::pow(0.999, (double)s->steps);
    note_launch();
    k_adam<<<ceil_div(kParams, 256), 256>>>(s->p, s->grad, s->m, s->v, lr, b1t, b2t);
  }
  GG_CUDA(cudaGetLastError());
  if (final_loss) GG_CUDA(cudaMemcpy(final_loss, s->loss, sizeof(float), cudaMemcpyDeviceToHost));
  GG_CUDA(cudaDeviceSynchronize());
  return check_tc(s);
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
