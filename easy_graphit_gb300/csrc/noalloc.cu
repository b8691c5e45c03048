// Allocation-free BFS: a variant of the fused BFS kernel (fused.cu) whose
// scratch -- two frontier queues, the rotating queue counts, the grid-barrier
// state and the status word -- lives in one file-scope __device__ array instead
// of memory the library allocates.
//
// Who needs it: callers that must not allocate device memory at call time --
// code running inside a pre-sized memory pool or arena owned by someone else,
// real-time loops where an allocation could stall or fail mid-run, and hosts
// whose allocator is off limits to plug-ins.  They pass the CSR and the output
// array (device pointers they own) and get BFS depths back; the library itself
// calls no cudaMalloc/cudaFree and no allocating library routine here.
//
// Limits and sharing:
//  - at most kNoAllocMaxVertices vertices (larger graphs are rejected);
//  - the array occupies (2 * kNoAllocMaxVertices + 64) * 4 bytes (about 8 MiB)
//    on every GPU that loads libgg.so, for the life of the process;
//  - every call shares the one array and it keeps the previous call's contents:
//    each call re-initialises the parts that must start at zero, and calls that
//    overlap on the GPU (different streams, or another thread) race on it.
#include <cuda.h>

#include <mutex>

#include "engine.h"
#include "lb.cuh"

namespace gg {

constexpr int32_t kNoAllocMaxVertices = 1 << 20;
constexpr int32_t kNoAllocHeader = 64;  // ints: counts[3], barrier[2], err, iterations
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) int32_t g_noalloc_scratch[kNoAllocHeader + 2 * kNoAllocMaxVertices];

// Host copies of the array's device address, one per device, each tagged with
// the unique id of the context it was looked up in: the array lives in the
// module loaded into that context, so after cudaDeviceReset, or under another
// context made current by the caller, the address is looked up again.
struct NoAllocSlot {
  unsigned long long ctx_id = 0;
  int32_t *ptr = nullptr;
};
static NoAllocSlot g_noalloc_slot[kNoAllocMaxDevices];
static std::mutex g_noalloc_mu;

// BFS UDF on the output array itself: depth[v] == -1 marks unvisited, and the
// winning CAS writes the level (the parent write of bfs.cpp:23-25 becomes the
// depth write).
struct UDepth {
  static constexpr bool kWeight = false;
  int32_t *depth;
  int32_t level;
  __device__ __forceinline__ bool src_ok(int32_t) const { return true; }
  __device__ __forceinline__ bool dst_ok(int32_t v) const {
    return *(volatile int32_t *)(depth + v) == -1;
  }
  __device__ __forceinline__ int32_t apply(int32_t, int32_t d, int32_t) const {
    return cas(depth + d, -1, level) ? d : -1;
  }
};

__global__ void k_noalloc_init(int32_t *scratch, int32_t *depth, int32_t V, int32_t src) {
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
    depth[v] = v == src ? 0 : -1;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    scratch[0] = 1;  // count of the first queue: {src}
    scratch[1] = 0;
    scratch[2] = 0;
    scratch[3] = 0;  // barrier arrivals
    scratch[4] = 0;  // barrier generation
    scratch[5] = 0;  // status word
    scratch[6] = 0;  // iterations
    scratch[kNoAllocHeader] = src;
  }
}

__global__ void __launch_bounds__(512) k_noalloc_bfs(DGraph g, int32_t *scratch, int32_t *depth,
                                                     uint64_t timeout_ns) {
  extern __shared__ int4 smem[];
  int32_t *cnt3 = scratch;
  uint32_t *bar = reinterpret_cast<uint32_t *>(scratch + 3);
  int32_t *err = scratch + 5;
  int32_t *qs[2] = {scratch + kNoAllocHeader, scratch + kNoAllocHeader + kNoAllocMaxVertices};
  int in = 0;
  int64_t level = 1;
  for (;; ++level) {
    const int32_t n = *(volatile int32_t *)(cnt3 + (level - 1) % 3);
    if (n == 0 || *(volatile int32_t *)err) break;
    if (blockIdx.x == 0 && threadIdx.x == 0) cnt3[(level + 1) % 3] = 0;
    const Enum en{qs[in], nullptr, n};
    const UDepth f{depth, (int32_t)level};
    DOut out{};
    out.mode = OUT_SPARSE;
    out.q = qs[in ^ 1];
    out.cnt = cnt3 + level % 3;
    out.cap = kNoAllocMaxVertices;  // each vertex is enqueued once (CAS)
    out.err = err;
    const int32_t nv = ceil_div(n, blockDim.x / kStage1);
    for (int32_t v = blockIdx.x; v < nv; v += gridDim.x)
      lb_twce<UDepth, true>(g, en, n, f, out, v, *reinterpret_cast<TwceSmem *>(smem));
    if (!grid_barrier(bar, gridDim.x, err, timeout_ns)) break;
    in ^= 1;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) scratch[6] = (int32_t)(level - 1);
}

// Unique id of the calling thread's current context (0 when none is current
// yet), through the driver entry points the runtime hands out (no libcuda link).
static gg_status current_context_id(unsigned long long *id) {
  using GetCurrent = CUresult (*)(CUcontext *);
  using GetId = CUresult (*)(CUcontext, unsigned long long *);
  struct Entry {
    GetCurrent get_current = nullptr;
    GetId get_id = nullptr;
  };
  static const Entry fn = [] {  // resolved once (thread-safe static initialisation)
    Entry e;
    void *a = nullptr, *b = nullptr;
    cudaDriverEntryPointQueryResult qa{}, qb{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) == cudaSuccess &&
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) == cudaSuccess &&
        qa == cudaDriverEntryPointSuccess && qb == cudaDriverEntryPointSuccess) {
      e.get_current = reinterpret_cast<GetCurrent>(a);
      e.get_id = reinterpret_cast<GetId>(b);
    }
    return e;
  }();
  if (!fn.get_current || !fn.get_id)
    return set_error(GG_ERR_CUDA, "driver entry points cuCtxGetCurrent / cuCtxGetId not found");
  CUcontext ctx = nullptr;
  if (fn.get_current(&ctx) != CUDA_SUCCESS) return set_error(GG_ERR_CUDA, "cuCtxGetCurrent failed");
  *id = 0;
  if (ctx && fn.get_id(ctx, id) != CUDA_SUCCESS) return set_error(GG_ERR_CUDA, "cuCtxGetId failed");
  return GG_OK;
}

// Device address of the scratch array in the current context of the current
// device.  Set-up on the first call per device and context: cudaGetSymbolAddress
// (which loads the module into the context if it is not loaded yet).
static gg_status noalloc_scratch(int32_t **out) {
  int dev = 0;
  GG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoAllocMaxDevices)
    return set_error(GG_ERR_UNSUPPORTED, "device %d beyond the %d supported", dev, kNoAllocMaxDevices);
  unsigned long long id = 0;
  GG_TRY(current_context_id(&id));
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  NoAllocSlot &slot = g_noalloc_slot[dev];
  if (!slot.ptr || id == 0 || slot.ctx_id != id) {
    int32_t *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress((void **)&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      return set_error(GG_ERR_CUDA, "cudaGetSymbolAddress of the no-alloc scratch failed: %s",
                       cudaGetErrorString(e));
    if (id == 0) GG_TRY(current_context_id(&id));  // the lookup made the primary context current
    slot.ptr = p;
    slot.ctx_id = id;
  }
  *out = slot.ptr;
  return GG_OK;
}

}  // namespace gg

using namespace gg;

extern "C" gg_status gg_bfs_noalloc(const int32_t *offsets, const int32_t *dst,
                                    int32_t num_vertices, int32_t num_edges, int32_t src,
                                    int32_t *depth_out, void *stream) {
  GG_CHECK_ARG(offsets && depth_out, "offsets and depth_out must be device pointers");
  GG_CHECK_ARG(num_edges == 0 || dst, "dst must be a device pointer");
  if (num_vertices < 1 || num_vertices > kNoAllocMaxVertices)
    return set_error(GG_ERR_INVALID,
                     "gg_bfs_noalloc: %d vertices is outside [1, %d], the size of its "
                     "preallocated scratch",
                     num_vertices, kNoAllocMaxVertices);
  GG_CHECK_ARG(num_edges >= 0, "negative edge count");
  GG_CHECK_ARG(src >= 0 && src < num_vertices, "source out of range");
  int32_t *scratch = nullptr;
  GG_TRY(noalloc_scratch(&scratch));
  cudaStream_t st = (cudaStream_t)stream;
  int dev = 0, sms = 0, coop = 0;
  GG_CUDA(cudaGetDevice(&dev));
  GG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  GG_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
  if (!coop) return set_error(GG_ERR_UNSUPPORTED, "device lacks cooperative launch");
  const int cta = 512;
  const size_t smem = twce_smem_bytes(cta);
  int per_sm = 0;
  GG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_noalloc_bfs, cta, smem));
  if (per_sm < 1) return set_error(GG_ERR_UNSUPPORTED, "BFS kernel does not fit on an SM");
  note_launch();
  k_noalloc_init<<<sms * 4, 256, 0, st>>>(scratch, depth_out, num_vertices, src);
  GG_CUDA(cudaGetLastError());
  DGraph g{num_vertices, num_edges, offsets, dst, nullptr, nullptr, nullptr, 0};
  uint64_t timeout = barrier_timeout_ns();
  void *args[] = {&g, &scratch, &depth_out, &timeout};
  note_launch();
  GG_CUDA(cudaLaunchCooperativeKernel((const void *)k_noalloc_bfs, per_sm * sms, cta, args, smem, st));
  int32_t status = 0;
  GG_CUDA(cudaMemcpyFromSymbolAsync(&status, g_noalloc_scratch, sizeof(int32_t), 5 * sizeof(int32_t),
                                    cudaMemcpyDeviceToHost, st));
  GG_CUDA(cudaStreamSynchronize(st));
  if (status & DEV_ERR_TIMEOUT) return set_error(GG_ERR_TIMEOUT, "gg_bfs_noalloc: grid barrier timed out");
  if (status & DEV_ERR_OVERFLOW) return set_error(GG_ERR_OVERFLOW, "gg_bfs_noalloc: queue overflow");
  return GG_OK;
}
