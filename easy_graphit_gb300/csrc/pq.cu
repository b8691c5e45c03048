// Delta-stepping priority queue: graphit_runtime::GPUPriorityQueue<int>
// (runtime/infra_gpu/gpu_priority_queue.h:21-247).
//
// finished()/dequeue() follow the reference's host logic (:63-153): when the
// frontier runs empty the queue advances to the smallest priority at or above
// the old window (update_nodes_identify_min, :250-268) and enqueues every vertex
// inside [cur, cur+delta) (update_nodes_special, :272-288).  Here the minimum
// is a block reduction with one atomic per block, and the enqueue compacts
// with warp ballots.
#include "engine.h"

namespace gg {

constexpr int kPqThreads = 512;

__global__ void __launch_bounds__(kPqThreads)
    k_pq_min(const int32_t *__restrict__ prio, int32_t V, int32_t window_upper, int32_t *gmin) {
  int32_t m = INT_MAX;
  const int32_t V4 = ((uintptr_t)prio & 15) == 0 ? V / 4 : 0;  // int4 loads when aligned
  const int4 *p4 = reinterpret_cast<const int4 *>(prio);
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < V4; i += gridDim.x * blockDim.x) {
    const int4 x = __ldg(p4 + i);
    const int32_t a[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (a[k] >= window_upper && a[k] != INT_MAX && a[k] < m) m = a[k];
  }
  for (int32_t i = V4 * 4 + blockIdx.x * blockDim.x + threadIdx.x; i < V; i += gridDim.x * blockDim.x) {
    const int32_t a = prio[i];
    if (a >= window_upper && a != INT_MAX && a < m) m = a;
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) m = min(m, __shfl_xor_sync(0xffffffffu, m, d));
  __shared__ int32_t wm[32];
  if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = threadIdx.x < (blockDim.x >> 5) ? wm[threadIdx.x] : INT_MAX;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) m = min(m, __shfl_xor_sync(0xffffffffu, m, d));
    if (threadIdx.x == 0 && m != INT_MAX) atomicMin(gmin, m);
  }
}

__global__ void __launch_bounds__(kPqThreads)
    k_pq_bucket(const int32_t *__restrict__ prio, int32_t V, int32_t lo, int64_t hi,
                int32_t *__restrict__ q, int32_t *__restrict__ cnt) {
  const int32_t stride = gridDim.x * blockDim.x;
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < ceil_div(V, stride) * stride; v += stride) {
    bool p = false;
    if (v < V) {
      const int32_t a = prio[v];
      p = a >= lo && (int64_t)a < hi;
    }
    const uint32_t m = __ballot_sync(0xffffffffu, p);
    if (m) {
      const int32_t lane = threadIdx.x & 31;
      int32_t base = 0;
      if (lane == 0) base = atomicAdd(cnt, __popc(m));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (p) q[base + __popc(m & ((1u << lane) - 1))] = v;
    }
  }
}

// dequeueReadySet's advance (gpu_priority_queue.h:125-149).
gg_status pq_advance(gg_pq *pq) {
  gg_graph *g = pq->g;
  cudaStream_t st = g->stream;
  const int32_t V = g->csr.V;
  pq->window_upper = pq->cur + pq->delta;
  pq->cur = INT_MAX;
  pq->advances++;
  int32_t *gmin = g->d_misc + 16;
  g->h_pinned[5] = INT_MAX;
  GG_CUDA(cudaMemcpyAsync(gmin, g->h_pinned + 5, sizeof(int32_t), cudaMemcpyHostToDevice, st));
  const int grid = g->sm_count * 4;
  if (pq->window_upper < INT_MAX)
    { gg::note_launch(); k_pq_min<<<grid, kPqThreads, 0, st>>>(pq->prio, V, (int32_t)pq->window_upper, gmin); }
  GG_CUDA(cudaGetLastError());
  GG_CUDA(cudaMemcpyAsync(g->h_pinned + 6, gmin, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  GG_CUDA(cudaStreamSynchronize(st));
  pq->cur = g->h_pinned[6];
  gg_frontier *f = pq->frontier;
  GG_CUDA(cudaMemsetAsync(f->cnt_out, 0, sizeof(int32_t), st));
  if (pq->cur != INT_MAX)
    { gg::note_launch(); k_pq_bucket<<<grid, kPqThreads, 0, st>>>(pq->prio, V, (int32_t)pq->cur, pq->cur + pq->delta,
                                             f->q_out, f->cnt_out); }
  GG_CUDA(cudaGetLastError());
  std::swap(f->q_in, f->q_out);
  std::swap(f->cnt_in, f->cnt_out);
  f->fmt = GG_FMT_SPARSE;
  return GG_OK;
}

int32_t pq_cutoff(const gg_pq *pq) {
  const int64_t c = pq->cur + pq->delta;
  return c > INT_MAX ? INT_MAX : (int32_t)c;
}

gg_status pq_finished(gg_pq *pq, bool *fin) {
  if (pq->cur == INT_MAX) {
    *fin = true;
    return GG_OK;
  }
  if (!pq->ready_set_dequeued) {
    int32_t n = 0;
    GG_TRY(frontier_size(pq->frontier, &n));
    if (n == 0) {
      GG_TRY(pq_advance(pq));
      pq->ready_set_dequeued = true;
      *fin = pq->cur == INT_MAX;
      return GG_OK;
    }
  }
  *fin = false;
  return GG_OK;
}

gg_status pq_dequeue(gg_pq *pq) {
  if (pq->ready_set_dequeued) {
    pq->ready_set_dequeued = false;
    return GG_OK;
  }
  int32_t n = 0;
  GG_TRY(frontier_size(pq->frontier, &n));
  if (n == 0) GG_TRY(pq_advance(pq));
  return GG_OK;
}

gg_status pq_reset(gg_pq *pq, int32_t init_priority, int32_t delta, int32_t src) {
  pq->cur = init_priority;
  pq->delta = delta;
  pq->window_upper = 0;
  pq->ready_set_dequeued = false;
  pq->advances = 0;
  gg_frontier *f = pq->frontier;
  gg_graph *g = pq->g;
  g->h_pinned[7] = src;
  g->h_pinned[8] = src >= 0 ? 1 : 0;
  GG_CUDA(cudaMemsetAsync(f->cnt, 0, sizeof(int32_t) * 2, g->stream));
  if (src >= 0) GG_CUDA(cudaMemcpyAsync(f->q_in, g->h_pinned + 7, sizeof(int32_t), cudaMemcpyHostToDevice, g->stream));
  GG_CUDA(cudaMemcpyAsync(f->cnt_in, g->h_pinned + 8, sizeof(int32_t), cudaMemcpyHostToDevice, g->stream));
  GG_CUDA(cudaStreamSynchronize(g->stream));
  f->fmt = GG_FMT_SPARSE;
  return GG_OK;
}

}  // namespace gg

using namespace gg;

extern "C" {

gg_status gg_pq_create(gg_graph *g, int32_t *priorities, int32_t init_priority, int32_t delta,
                       int32_t src, gg_pq **out) {
  GG_CHECK_ARG(g && priorities && out, "bad arguments");
  GG_CHECK_ARG(delta >= 1, "delta must be >= 1");
  GG_CHECK_ARG(src >= -1 && src < g->csr.V, "source out of range");
  auto pq = new gg_pq();
  pq->g = g;
  pq->prio = priorities;
  gg_status s = gg_frontier_create(g, 0, &pq->frontier);
  if (s != GG_OK) {
    delete pq;
    return s;
  }
  pq->frontier->owned_by_pq = true;
  s = pq_reset(pq, init_priority, delta, src);
  if (s != GG_OK) {
    gg_frontier_destroy(pq->frontier);
    delete pq;
    return s;
  }
  *out = pq;
  return GG_OK;
}

gg_status gg_pq_destroy(gg_pq *pq) {
  if (!pq) return GG_OK;
  gg_frontier_destroy(pq->frontier);
  delete pq;
  return GG_OK;
}

gg_status gg_pq_finished(gg_pq *pq, int32_t *finished) {
  GG_CHECK_ARG(pq && finished, "bad arguments");
  bool f = false;
  GG_TRY(pq_finished(pq, &f));
  *finished = f;
  return GG_OK;
}

gg_status gg_pq_dequeue(gg_pq *pq, gg_frontier **frontier) {
  GG_CHECK_ARG(pq, "pq is NULL");
  GG_TRY(pq_dequeue(pq));
  if (frontier) *frontier = pq->frontier;
  return GG_OK;
}

gg_status gg_edgeset_apply_priority(gg_graph *g, const gg_schedule *s, gg_pq *pq,
                                    const gg_vertex_data *vd) {
  GG_CHECK_ARG(g && s && pq, "bad arguments");
  VData d = to_vdata(vd);
  d.dist = pq->prio;
  GG_TRY(edgeset_apply_impl(g, s, GG_UDF_SSSP_RELAX, GG_FILTER_NONE, pq->frontier, pq->frontier,
                            true, d, pq_cutoff(pq), false));
  return check_device_error(g, "apply_priority");
}

}  // extern "C"
