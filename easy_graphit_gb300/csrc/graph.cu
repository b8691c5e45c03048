// Device graphs: graphit_runtime::GraphT<int> (runtime/infra_gpu/graph.h).
//  - gg_graph_create uploads a CSR like load_graph (graph.h:305-320) and builds
//    the COO source column on the GPU.
//  - get_transposed_graph (graph.h:165-234, a host counting sort in the
//    reference) is a GPU counting sort here, cached in the handle.
//  - get_blocked_graph (graph.h:105-163, a host bucketing by dst/block_size
//    that also frees the source arrays) is a GPU bucketing into a separate copy.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "engine.h"
#include "scan.cuh"

namespace gg {

__global__ void __launch_bounds__(1024) k_scan_partials(int32_t *partial, int32_t nb) {
  __shared__ int32_t ws[32];
  int32_t carry = 0;
  for (int32_t base = 0; base < nb; base += blockDim.x) {
    const int32_t i = base + threadIdx.x;
    const int32_t x = i < nb ? partial[i] : 0;
    int32_t tot;
    const int32_t ex = block_scan_excl(x, ws, &tot);
    if (i < nb) partial[i] = carry + ex;
    carry += tot;
  }
}

// COO source of every edge: binary search of the edge index in the offsets.
__global__ void k_coo_src(const int32_t *__restrict__ off, int32_t V, int32_t E,
                          int32_t *__restrict__ src) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < E;
       k += (int64_t)gridDim.x * blockDim.x) {
    int32_t lo = 0, len = V;
    while (len > 0) {  // upper_bound(off[0..V), k) - 1
      const int32_t half = len >> 1;
      if (__ldg(off + lo + half) > k) {
        len = half;
      } else {
        lo += half + 1;
        len -= half + 1;
      }
    }
    src[k] = lo - 1;
  }
}

__global__ void k_count_dst(const int32_t *__restrict__ dst, int32_t E, int32_t *__restrict__ cnt) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < E;
       k += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(cnt + __ldg(dst + k), 1);
}

struct ArrIn {
  const int32_t *a;
  __device__ int32_t operator()(int64_t i) const { return a[i]; }
};

// Scatter every edge (u -> v, w) to position cursor[v]++ of the transposed CSR.
__global__ void k_transpose_scatter(const int32_t *__restrict__ src, const int32_t *__restrict__ dst,
                                   const int32_t *__restrict__ w, int32_t E,
                                   int32_t *__restrict__ cursor, int32_t *__restrict__ tdst,
                                   int32_t *__restrict__ tw, int32_t *__restrict__ tsrc) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < E;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int32_t v = __ldg(dst + k);
    const int32_t p = atomicAdd(cursor + v, 1);
    tdst[p] = __ldg(src + k);
    tw[p] = __ldg(w + k);
    tsrc[p] = v;
  }
}

// In-list order after an atomic scatter is arbitrary; sort each list by
// neighbour id so the transposed graph (and everything that iterates it) is
// deterministic.  Lists up to kSortTile entries are bitonic-sorted by one
// block in shared memory; the rare longer ones (hubs) in global memory.
__device__ __forceinline__ void swap_if(int32_t &a, int32_t &b, int32_t &wa, int32_t &wb, bool up) {
  if ((a > b) == up) {
    int32_t t = a; a = b; b = t;
    t = wa; wa = wb; wb = t;
  }
}

constexpr int kSortTile = 2048;

// Block bitonic sort of one list of length len <= kSortTile in shared memory.
__global__ void __launch_bounds__(1024) k_sort_lists(const int32_t *__restrict__ off, int32_t V,
                                                     int32_t *__restrict__ nbr,
                                                     int32_t *__restrict__ wt) {
  __shared__ int32_t sk[kSortTile], sw[kSortTile];
  for (int32_t v = blockIdx.x; v < V; v += gridDim.x) {
    const int32_t b = off[v], len = off[v + 1] - b;
    if (len <= 1 || len > kSortTile) continue;
    int32_t p2 = 1;
    while (p2 < len) p2 <<= 1;
    for (int32_t i = threadIdx.x; i < p2; i += blockDim.x) {
      sk[i] = i < len ? nbr[b + i] : INT_MAX;
      sw[i] = i < len ? wt[b + i] : 0;
    }
    __syncthreads();
    for (int32_t k = 2; k <= p2; k <<= 1)
      for (int32_t j = k >> 1; j > 0; j >>= 1) {
        for (int32_t i = threadIdx.x; i < p2; i += blockDim.x) {
          const int32_t ixj = i ^ j;
          if (ixj > i) {
            const bool up = (i & k) == 0;
            int32_t a = sk[i], c = sk[ixj], wa = sw[i], wc = sw[ixj];
            swap_if(a, c, wa, wc, up);
            sk[i] = a; sk[ixj] = c; sw[i] = wa; sw[ixj] = wc;
          }
        }
        __syncthreads();
      }
    for (int32_t i = threadIdx.x; i < len; i += blockDim.x) {
      nbr[b + i] = sk[i];
      wt[b + i] = sw[i];
    }
    __syncthreads();
  }
}

// Lists longer than the tile are copied into power-of-two padded slots
// (+inf padding) and sorted there by global bitonic steps, all lists at once.
__global__ void k_long_copy_in(const int32_t *__restrict__ off, const int32_t *__restrict__ ids,
                               const int64_t *__restrict__ poff, int32_t nids,
                               const int32_t *__restrict__ nbr, const int32_t *__restrict__ wt,
                               int32_t *__restrict__ tk, int32_t *__restrict__ tw) {
  for (int32_t l = blockIdx.y; l < nids; l += gridDim.y) {
    const int32_t v = ids[l], b = off[v], len = off[v + 1] - b;
    const int64_t p2 = poff[l + 1] - poff[l];
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < p2;
         i += (int64_t)gridDim.x * blockDim.x) {
      tk[poff[l] + i] = i < len ? nbr[b + i] : INT_MAX;
      tw[poff[l] + i] = i < len ? wt[b + i] : 0;
    }
  }
}

__global__ void k_long_step(const int64_t *__restrict__ poff, int32_t nids, int32_t *__restrict__ tk,
                            int32_t *__restrict__ tw, int64_t k, int64_t j) {
  for (int32_t l = blockIdx.y; l < nids; l += gridDim.y) {
    const int64_t p2 = poff[l + 1] - poff[l];
    if (k > p2) continue;
    int32_t *K = tk + poff[l], *W = tw + poff[l];
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < p2;
         i += (int64_t)gridDim.x * blockDim.x) {
      const int64_t ixj = i ^ j;
      if (ixj <= i) continue;
      const bool up = (i & k) == 0;
      const int32_t a = K[i], c = K[ixj];
      if ((a > c) == up) {
        const int32_t wa = W[i];
        K[i] = c; K[ixj] = a; W[i] = W[ixj]; W[ixj] = wa;
      }
    }
  }
}

__global__ void k_long_copy_out(const int32_t *__restrict__ off, const int32_t *__restrict__ ids,
                                const int64_t *__restrict__ poff, int32_t nids,
                                int32_t *__restrict__ nbr, int32_t *__restrict__ wt,
                                const int32_t *__restrict__ tk, const int32_t *__restrict__ tw) {
  for (int32_t l = blockIdx.y; l < nids; l += gridDim.y) {
    const int32_t v = ids[l], b = off[v], len = off[v + 1] - b;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len;
         i += (int64_t)gridDim.x * blockDim.x) {
      nbr[b + i] = tk[poff[l] + i];
      wt[b + i] = tw[poff[l] + i];
    }
  }
}

__global__ void k_bucket_count(const int32_t *__restrict__ dst, int32_t E, int32_t bs,
                               int32_t *__restrict__ cnt) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < E;
       k += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(cnt + __ldg(dst + k) / bs, 1);
}

__global__ void k_bucket_scatter(const int32_t *__restrict__ src, const int32_t *__restrict__ dst,
                                 const int32_t *__restrict__ w, int32_t E, int32_t bs,
                                 int32_t *__restrict__ cursor, int32_t *__restrict__ osrc,
                                 int32_t *__restrict__ odst, int32_t *__restrict__ ow) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < E;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int32_t d = __ldg(dst + k);
    const int32_t p = atomicAdd(cursor + d / bs, 1);
    osrc[p] = __ldg(src + k);
    odst[p] = d;
    ow[p] = __ldg(w + k);
  }
}

static int stream_grid(gg_graph *g) { return g->sm_count * 8; }

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_pool_mu;
cudaMemPool_t g_pool[kMaxDevices] = {};
}  // namespace

// GG_DEVICE_POOL_LIMIT_BYTES caps what the pool hands out (allocations beyond
// it fail as out of memory): a way to run the engine inside a fixed memory
// budget, and to exercise the GG_ERR_OOM path without exhausting a GPU.
static uint64_t pool_limit_bytes() {
  static const uint64_t lim = [] {
    const char *e = getenv("GG_DEVICE_POOL_LIMIT_BYTES");
    const unsigned long long v = e ? strtoull(e, nullptr, 10) : 0ull;
    return v ? (uint64_t)v : UINT64_MAX;
  }();
  return lim;
}

cudaError_t dev_alloc(void **p, size_t bytes, cudaStream_t st) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaMallocAsync(p, bytes, st);
  cudaMemPool_t pool = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (!g_pool[dev]) {
      cudaMemPoolProps props{};
      props.allocType = cudaMemAllocationTypePinned;
      props.handleTypes = cudaMemHandleTypeNone;
      props.location.type = cudaMemLocationTypeDevice;
      props.location.id = dev;
      e = cudaMemPoolCreate(&g_pool[dev], &props);
      if (e != cudaSuccess) return e;
      uint64_t keep = UINT64_MAX;
      e = cudaMemPoolSetAttribute(g_pool[dev], cudaMemPoolAttrReleaseThreshold, &keep);
      if (e != cudaSuccess) return e;
    }
    pool = g_pool[dev];
  }
  const uint64_t limit = pool_limit_bytes();
  if (limit != UINT64_MAX) {
    uint64_t used = 0;
    e = cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used);
    if (e != cudaSuccess) return e;
    if (used + bytes > limit) return cudaErrorMemoryAllocation;
  }
  return cudaMallocFromPoolAsync(p, bytes, pool, st);
}

gg_status ensure_coo(GraphStore &s, cudaStream_t st) {
  if (s.src || s.E == 0) return GG_OK;
  GG_CUDA(dev_alloc(&s.src, sizeof(int32_t) * (size_t)s.E, st));
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  { gg::note_launch(); k_coo_src<<<sms * 8, 256, 0, st>>>(s.off, s.V, s.E, s.src); }
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

static void free_store(GraphStore &s, cudaStream_t st) {
  for (int32_t *p : {s.off, s.dst, s.w, s.src, s.bucket})
    if (p) cudaFreeAsync(p, st);
  s = GraphStore();
}

gg_status ensure_transpose(gg_graph *g) {
  if (g->csc) return GG_OK;
  if (g->symmetric) return GG_OK;  // the transpose of a symmetric graph is itself
  cudaStream_t st = g->stream;
  const GraphStore &f = g->csr;
  auto t = std::make_unique<GraphStore>();
  t->V = f.V;
  t->E = f.E;
  GG_TRY(ensure_coo(g->csr, st));
  int32_t *cnt = nullptr, *partial = nullptr;
  GG_CUDA(dev_alloc(&t->off, sizeof(int32_t) * (f.V + 1), st));
  GG_CUDA(dev_alloc(&t->dst, sizeof(int32_t) * std::max(f.E, 1), st));
  GG_CUDA(dev_alloc(&t->w, sizeof(int32_t) * std::max(f.E, 1), st));
  GG_CUDA(dev_alloc(&t->src, sizeof(int32_t) * std::max(f.E, 1), st));
  GG_CUDA(dev_alloc(&cnt, sizeof(int32_t) * (f.V + 1), st));
  GG_CUDA(dev_alloc(&partial, sizeof(int32_t) * scan_scratch_ints(f.V), st));
  GG_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (f.V + 1), st));
  const int grid = stream_grid(g);
  { gg::note_launch(); k_count_dst<<<grid, 256, 0, st>>>(f.dst, f.E, cnt); }
  GG_CUDA(exclusive_scan(ArrIn{cnt}, f.V, t->off, partial, st));
  GG_CUDA(cudaMemcpyAsync(cnt, t->off, sizeof(int32_t) * f.V, cudaMemcpyDeviceToDevice, st));
  { gg::note_launch(); k_transpose_scatter<<<grid, 256, 0, st>>>(g->csr.src, f.dst, f.w, f.E, cnt, t->dst, t->w, t->src); }
  GG_CUDA(cudaGetLastError());
  // Deterministic in-lists.
  { gg::note_launch(); k_sort_lists<<<grid, 256, 0, st>>>(t->off, t->V, t->dst, t->w); }
  GG_CUDA(cudaGetLastError());
  // Lists longer than the shared-memory tile (hubs): bitonic in global memory.
  std::vector<int32_t> hoff(t->V + 1);
  GG_CUDA(cudaMemcpyAsync(hoff.data(), t->off, sizeof(int32_t) * (t->V + 1), cudaMemcpyDeviceToHost, st));
  GG_CUDA(cudaStreamSynchronize(st));
  std::vector<int32_t> longs;
  for (int32_t v = 0; v < t->V; ++v)
    if (hoff[v + 1] - hoff[v] > kSortTile) longs.push_back(v);
  if (!longs.empty()) {
    std::vector<int64_t> poff(longs.size() + 1, 0);
    int64_t maxp2 = 1;
    for (size_t l = 0; l < longs.size(); ++l) {
      int64_t p2 = 1;
      while (p2 < hoff[longs[l] + 1] - hoff[longs[l]]) p2 <<= 1;
      poff[l + 1] = poff[l] + p2;
      maxp2 = std::max(maxp2, p2);
    }
    const int32_t nl = (int32_t)longs.size();
    int32_t *ids = nullptr, *tk = nullptr, *tw = nullptr;
    int64_t *dpoff = nullptr;
    GG_CUDA(dev_alloc(&ids, sizeof(int32_t) * nl, st));
    GG_CUDA(dev_alloc(&dpoff, sizeof(int64_t) * (nl + 1), st));
    GG_CUDA(dev_alloc(&tk, sizeof(int32_t) * poff[nl], st));
    GG_CUDA(dev_alloc(&tw, sizeof(int32_t) * poff[nl], st));
    GG_CUDA(cudaMemcpyAsync(ids, longs.data(), sizeof(int32_t) * nl, cudaMemcpyHostToDevice, st));
    GG_CUDA(cudaMemcpyAsync(dpoff, poff.data(), sizeof(int64_t) * (nl + 1), cudaMemcpyHostToDevice, st));
    dim3 grd((unsigned)std::min<int64_t>(64, (maxp2 + 255) / 256), (unsigned)std::min(nl, 1024));
    { gg::note_launch(); k_long_copy_in<<<grd, 256, 0, st>>>(t->off, ids, dpoff, nl, t->dst, t->w, tk, tw); }
    for (int64_t k = 2; k <= maxp2; k <<= 1)
      for (int64_t j = k >> 1; j > 0; j >>= 1)
        { gg::note_launch(); k_long_step<<<grd, 256, 0, st>>>(dpoff, nl, tk, tw, k, j); }
    { gg::note_launch(); k_long_copy_out<<<grd, 256, 0, st>>>(t->off, ids, dpoff, nl, t->dst, t->w, tk, tw); }
    GG_CUDA(cudaGetLastError());
    GG_CUDA(cudaStreamSynchronize(st));
    for (void *p : {(void *)ids, (void *)dpoff, (void *)tk, (void *)tw}) cudaFreeAsync(p, st);
  }
  // The COO column of the transpose (src) was written by the scatter and is
  // sorted with the list order unchanged (all entries of a list equal v).
  cudaFreeAsync(cnt, st);
  cudaFreeAsync(partial, st);
  g->csc = std::move(t);
  return GG_OK;
}

gg_status ensure_blocked(gg_graph *g, bool reverse, int32_t block_size, const GraphStore **out) {
  if (block_size <= 0) return set_error(GG_ERR_INVALID, "invalid block size %d", block_size);
  auto &cache = reverse ? g->blocked_rev : g->blocked_fwd;
  auto it = cache.find(block_size);
  if (it != cache.end()) {
    *out = &it->second;
    return GG_OK;
  }
  cudaStream_t st = g->stream;
  if (reverse) GG_TRY(ensure_transpose(g));
  GraphStore &base = (reverse && g->csc) ? *g->csc : g->csr;
  GG_TRY(ensure_coo(base, st));
  GraphStore b;
  b.V = base.V;
  b.E = base.E;
  b.nbuckets = (base.V + block_size - 1) / block_size;
  int32_t *cnt = nullptr, *partial = nullptr;
  const size_t E1 = std::max(base.E, 1);
  GG_CUDA(dev_alloc(&b.src, sizeof(int32_t) * E1, st));
  GG_CUDA(dev_alloc(&b.dst, sizeof(int32_t) * E1, st));
  GG_CUDA(dev_alloc(&b.w, sizeof(int32_t) * E1, st));
  GG_CUDA(dev_alloc(&b.bucket, sizeof(int32_t) * (b.nbuckets + 1), st));
  GG_CUDA(dev_alloc(&cnt, sizeof(int32_t) * (b.nbuckets + 1), st));
  GG_CUDA(dev_alloc(&partial, sizeof(int32_t) * scan_scratch_ints(b.nbuckets), st));
  GG_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (b.nbuckets + 1), st));
  const int grid = stream_grid(g);
  { gg::note_launch(); k_bucket_count<<<grid, 256, 0, st>>>(base.dst, base.E, block_size, cnt); }
  GG_CUDA(exclusive_scan(ArrIn{cnt}, b.nbuckets, b.bucket, partial, st));
  GG_CUDA(cudaMemcpyAsync(cnt, b.bucket, sizeof(int32_t) * b.nbuckets, cudaMemcpyDeviceToDevice, st));
  { gg::note_launch(); k_bucket_scatter<<<grid, 256, 0, st>>>(base.src, base.dst, base.w, base.E, block_size, cnt, b.src,
                                         b.dst, b.w); }
  GG_CUDA(cudaGetLastError());
  cudaFreeAsync(cnt, st);
  cudaFreeAsync(partial, st);
  auto res = cache.emplace(block_size, b);
  *out = &res.first->second;
  return GG_OK;
}

gg_status check_device_error(gg_graph *g, const char *what) {
  GG_CUDA(cudaMemcpyAsync(g->h_pinned + 63, g->d_err, sizeof(int32_t), cudaMemcpyDeviceToHost, g->stream));
  GG_CUDA(cudaStreamSynchronize(g->stream));
  const int32_t e = g->h_pinned[63];
  if (!e) return GG_OK;
  GG_CUDA(cudaMemsetAsync(g->d_err, 0, sizeof(int32_t), g->stream));
  if (e & DEV_ERR_TIMEOUT)
    return set_error(GG_ERR_TIMEOUT, "%s: a grid barrier wait timed out", what);
  return set_error(GG_ERR_OVERFLOW, "%s: frontier queue capacity exceeded", what);
}

gg_status scratch_get(gg_graph *g, int slot, size_t bytes, void **p) {
  Scratch &s = g->scratch[slot];
  if (s.bytes < bytes) {
    if (s.p) cudaFreeAsync(s.p, g->stream);
    s.p = nullptr;
    s.bytes = 0;
    GG_CUDA(dev_alloc(&s.p, bytes, g->stream));
    s.bytes = bytes;
  }
  *p = s.p;
  return GG_OK;
}

int resident_grid(const void *kernel, int cta, size_t smem, int sm_count) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, cta, smem) != cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  return per_sm * sm_count;
}

}  // namespace gg

using namespace gg;

extern "C" {

// Everything gg_graph_create sets up; on failure the caller releases what was
// made (gg_graph_destroy takes a partly built graph).
static gg_status graph_init(gg_graph *g, const int32_t *offsets, const int32_t *dst, const int32_t *weights,
                            int32_t V, int64_t E, uint32_t flags) {
  GG_CUDA(cudaGetDevice(&g->device));
  GG_CUDA(cudaDeviceGetAttribute(&g->sm_count, cudaDevAttrMultiProcessorCount, g->device));
  GG_CUDA(cudaStreamCreateWithFlags(&g->own_stream, cudaStreamNonBlocking));
  g->stream = g->own_stream;
  g->symmetric = (flags & GG_GRAPH_SYMMETRIC) != 0;
  cudaStream_t st = g->stream;
  GraphStore &s = g->csr;
  s.V = V;
  s.E = (int32_t)E;
  const size_t E1 = std::max<int64_t>(E, 1);
  GG_CUDA(dev_alloc(&s.off, sizeof(int32_t) * (V + 1), st));
  GG_CUDA(dev_alloc(&s.dst, sizeof(int32_t) * E1, st));
  GG_CUDA(dev_alloc(&s.w, sizeof(int32_t) * E1, st));
  GG_CUDA(cudaMemcpyAsync(s.off, offsets, sizeof(int32_t) * (V + 1), cudaMemcpyDefault, st));
  if (E) {
    GG_CUDA(cudaMemcpyAsync(s.dst, dst, sizeof(int32_t) * E, cudaMemcpyDefault, st));
    if (weights) {
      GG_CUDA(cudaMemcpyAsync(s.w, weights, sizeof(int32_t) * E, cudaMemcpyDefault, st));
    } else {
      std::vector<int32_t> ones(E, 1);
      GG_CUDA(cudaMemcpyAsync(s.w, ones.data(), sizeof(int32_t) * E, cudaMemcpyHostToDevice, st));
      GG_CUDA(cudaStreamSynchronize(st));
    }
  }
  GG_CUDA(dev_alloc(&g->d_err, sizeof(int32_t), st));
  GG_CUDA(dev_alloc(&g->d_bar, sizeof(uint32_t) * 2, st));
  GG_CUDA(dev_alloc(&g->d_misc, sizeof(int32_t) * 64, st));
  GG_CUDA(cudaMemsetAsync(g->d_err, 0, sizeof(int32_t), st));
  GG_CUDA(cudaMemsetAsync(g->d_bar, 0, sizeof(uint32_t) * 2, st));
  GG_CUDA(cudaMemsetAsync(g->d_misc, 0, sizeof(int32_t) * 64, st));
  GG_CUDA(cudaMallocHost(&g->h_pinned, sizeof(int32_t) * 64));
  GG_CUDA(cudaEventCreate(&g->ev0));
  GG_CUDA(cudaEventCreate(&g->ev1));
  GG_CUDA(cudaEventCreate(&g->ev2));
  GG_CUDA(cudaEventCreate(&g->ev3));
  GG_CUDA(cudaStreamSynchronize(st));  // the COO source column is built on first use (ensure_coo)
  return GG_OK;
}

gg_status gg_graph_create(const int32_t *offsets, const int32_t *dst, const int32_t *weights,
                          int32_t V, int64_t E, uint32_t flags, gg_graph **out) {
  GG_CHECK_ARG(out && offsets, "offsets/out is NULL");
  GG_CHECK_ARG(V > 0, "graph needs at least one vertex");
  GG_CHECK_ARG(E >= 0 && E <= INT32_MAX, "edge count outside the int32 CSR layout");
  GG_CHECK_ARG(E == 0 || dst, "dst is NULL");
  auto *g = new (std::nothrow) gg_graph();
  if (!g) return set_error(GG_ERR_OOM, "graph handle allocation failed");
  const gg_status st = graph_init(g, offsets, dst, weights, V, E, flags);
  if (st != GG_OK) {
    gg_graph_destroy(g);  // the pool takes back what was allocated
    return st;
  }
  *out = g;
  return GG_OK;
}

gg_status gg_graph_destroy(gg_graph *g) {
  if (!g) return GG_OK;
  if (g->app_pq) gg_pq_destroy(g->app_pq);
  if (g->app_frontier) gg_frontier_destroy(g->app_frontier);
  if (g->app_list) gg_frontier_list_destroy(g->app_list);
  cudaStream_t st = g->stream;
  for (auto &s : g->app)
    if (s.p) cudaFreeAsync(s.p, st);
  free_store(g->csr, st);
  if (g->csc) free_store(*g->csc, st);
  for (auto &kv : g->blocked_fwd) free_store(kv.second, st);
  for (auto &kv : g->blocked_rev) free_store(kv.second, st);
  free_relabel(g);
  for (auto &s : g->scratch)
    if (s.p) cudaFreeAsync(s.p, st);
  if (g->bq_cta.p) cudaFreeAsync(g->bq_cta.p, st);
  for (void *p : {(void *)g->d_err, (void *)g->d_bar, (void *)g->d_misc})
    if (p) cudaFreeAsync(p, st);
  cudaStreamSynchronize(st);
  if (g->h_pinned) cudaFreeHost(g->h_pinned);
  if (g->ev0) cudaEventDestroy(g->ev0);
  if (g->ev1) cudaEventDestroy(g->ev1);
  if (g->ev2) cudaEventDestroy(g->ev2);
  if (g->ev3) cudaEventDestroy(g->ev3);
  if (g->own_stream) cudaStreamDestroy(g->own_stream);
  delete g;
  // Any failure above is reported here rather than by the next call's launch check.
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(GG_ERR_CUDA, "releasing the graph failed: %s", cudaGetErrorString(e));
  return GG_OK;
}

gg_status gg_graph_info(const gg_graph *g, int32_t *V, int64_t *E) {
  GG_CHECK_ARG(g, "graph is NULL");
  if (V) *V = g->csr.V;
  if (E) *E = g->csr.E;
  return GG_OK;
}

gg_status gg_graph_set_stream(gg_graph *g, void *stream) {
  GG_CHECK_ARG(g, "graph is NULL");
  GG_CUDA(cudaStreamSynchronize(g->stream));
  g->stream = stream ? (cudaStream_t)stream : g->own_stream;
  return GG_OK;
}

gg_status gg_graph_sync(gg_graph *g) {
  GG_CHECK_ARG(g, "graph is NULL");
  GG_CUDA(cudaStreamSynchronize(g->stream));
  return GG_OK;
}

gg_status gg_graph_transpose(gg_graph *g) {
  GG_CHECK_ARG(g, "graph is NULL");
  GG_TRY(ensure_transpose(g));
  GG_CUDA(cudaStreamSynchronize(g->stream));
  return GG_OK;
}

gg_status gg_graph_blocked(gg_graph *g, int32_t block_size) {
  GG_CHECK_ARG(g, "graph is NULL");
  const GraphStore *b = nullptr;
  GG_TRY(ensure_blocked(g, false, block_size, &b));
  GG_CUDA(cudaStreamSynchronize(g->stream));
  return GG_OK;
}

gg_status gg_graph_device_arrays(const gg_graph *g, const int32_t **off, const int32_t **dst,
                                 const int32_t **w) {
  GG_CHECK_ARG(g, "graph is NULL");
  if (off) *off = g->csr.off;
  if (dst) *dst = g->csr.dst;
  if (w) *w = g->csr.w;
  return GG_OK;
}

}  // extern "C"

// Hands the library pools' unused memory back to the driver, keeping at most
// keep_bytes reserved per device.
extern "C" gg_status gg_memory_trim(size_t keep_bytes) {
  std::lock_guard<std::mutex> lk(g_pool_mu);
  for (int d = 0; d < kMaxDevices; ++d)
    if (g_pool[d]) GG_CUDA(cudaMemPoolTrimTo(g_pool[d], keep_bytes));
  return GG_OK;
}
