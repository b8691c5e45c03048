// Delta-stepping priority queue: graphit_runtime::GPUPriorityQueue<int>
// (runtime/infra_gpu/gpu_priority_queue.h:21-247), host-driven as in the
// reference (finished()/dequeue() decide on the host, :63-153).
//
// The advance keeps the reference rule -- the window moves to the smallest
// priority at or above the old window (update_nodes_identify_min, :250-268)
// and every vertex inside [cur, cur+delta) is enqueued (update_nodes_special,
// :272-288) -- but finds both from the far piles of bucket_queue.cuh, which the
// relax fills, instead of scanning all V twice: a minimum kernel over the low
// pile (or, when that holds nothing live, over the high pile), one read-back of
// the minimum (the reference copies its whole queue back per advance,
// :129-137), and a split kernel that fills the frontier.
#include "engine.h"

namespace gg {

constexpr int kPqThreads = 512;

__global__ void __launch_bounds__(kPqThreads)
    k_bq_min(const int32_t *__restrict__ pile, const int32_t *__restrict__ cnt, int32_t cap, const int32_t *P,
             int32_t U, int32_t *out) {
  __shared__ int32_t red[32];
  bq_pile_min(pile, min(*cnt, cap), P, U, out, blockIdx.x, gridDim.x, red);
}

__global__ void __launch_bounds__(kPqThreads)
    k_bq_split(const int32_t *__restrict__ pile, const int32_t *__restrict__ cnt, const int32_t *P, int32_t U,
               int32_t win_hi, DOut front, BqSplitOut o, int32_t *err) {
  // a count past the capacity only follows an overflow already flagged in *err
  bq_pile_split(pile, min(*cnt, o.cap), P, U, win_hi, front, o, err, blockIdx.x, gridDim.x);
}

gg_status bq_alloc(gg_graph *g, BqBuffers *b) {
  const size_t V = (size_t)std::max(g->csr.V, 1);
  const size_t bytes = sizeof(int32_t) * (5 * V + BQ_CTL_INTS);
  GG_CUDA(dev_alloc(&b->base, bytes, g->stream));
  int32_t *p = static_cast<int32_t *>(b->base);
  b->ctl = p;
  b->stamp = p + BQ_CTL_INTS;
  b->lo[0] = b->stamp + V;
  b->lo[1] = b->lo[0] + V;
  b->hi[0] = b->lo[1] + V;
  b->hi[1] = b->hi[0] + V;
  b->V = g->csr.V;
  return GG_OK;
}

void bq_free(gg_graph *g, BqBuffers *b) {
  if (b->base) cudaFreeAsync(b->base, g->stream);
  *b = BqBuffers{};
}

DFar pq_far(const gg_pq *pq) {
  const BqBuffers &b = pq->bq;
  return DFar{b.stamp, b.lo[pq->gen_lo & 1], b.ctl + BQ_LO + (pq->gen_lo & 1), b.hi[pq->gen_hi & 1],
              b.ctl + BQ_HI + (pq->gen_hi & 1), bq_lo_tag(pq->gen_lo), bq_hi_tag(pq->gen_hi), pq->horizon,
              b.V, pq->g->d_err};
}

// dequeueReadySet's advance (gpu_priority_queue.h:125-149) over the far piles.
gg_status pq_advance(gg_pq *pq) {
  gg_graph *g = pq->g;
  cudaStream_t st = g->stream;
  BqBuffers &b = pq->bq;
  const int32_t U = bq_clamp(pq->cur + pq->delta);  // the old window's upper end
  pq->window_upper = U;
  pq->cur = INT_MAX;
  pq->advances++;
  gg_frontier *f = pq->frontier;
  GG_CUDA(cudaMemsetAsync(f->cnt_out, 0, sizeof(int32_t), st));
  int32_t *h = g->h_pinned + 24;  // [0..15] copy of the control words
  const int grid = g->sm_count * 4;
  // counts of both piles (and the last refill) with one read-back
  GG_CUDA(cudaMemcpyAsync(h, b.ctl, sizeof(int32_t) * 16, cudaMemcpyDeviceToHost, st));
  GG_CUDA(cudaStreamSynchronize(st));
  const int32_t lo = pq->gen_lo & 1, hi = pq->gen_hi & 1;
  const int32_t n_lo = h[BQ_LO + lo], n_hi = h[BQ_HI + hi], fill = h[BQ_FILL];
  int32_t m = INT_MAX;
  bool from_hi = false;
  auto pile_min = [&](const int32_t *pile, const int32_t *cnt) -> gg_status {
    h[BQ_MIN] = INT_MAX;
    GG_CUDA(cudaMemcpyAsync(b.ctl + BQ_MIN, h + BQ_MIN, sizeof(int32_t), cudaMemcpyHostToDevice, st));
    note_launch();
    k_bq_min<<<grid, kPqThreads, 0, st>>>(pile, cnt, b.V, pq->prio, U, b.ctl + BQ_MIN);
    GG_CUDA(cudaGetLastError());
    GG_CUDA(cudaMemcpyAsync(h + BQ_MIN, b.ctl + BQ_MIN, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    GG_CUDA(cudaStreamSynchronize(st));
    m = h[BQ_MIN];
    return GG_OK;
  };
  if (n_lo > 0) GG_TRY(pile_min(b.lo[lo], b.ctl + BQ_LO + lo));
  if (m == INT_MAX && n_hi > 0) {
    GG_TRY(pile_min(b.hi[hi], b.ctl + BQ_HI + hi));
    from_hi = true;
  }
  if (m != INT_MAX) {
    DOut front{};
    front.mode = OUT_SPARSE;
    front.q = f->q_out;
    front.cnt = f->cnt_out;
    front.cap = f->cap;
    front.err = g->d_err;
    const int32_t lo_next = (pq->gen_lo + 1) & 1, hi_next = (pq->gen_hi + 1) & 1;
    const int32_t win = bq_clamp((int64_t)m + pq->delta);
    // a refill, or a window reaching past the horizon, splits the high pile
    // too, under a new horizon above the window
    const bool split_hi = from_hi || win > pq->horizon;
    // next generations start empty
    h[0] = 0;
    GG_CUDA(cudaMemcpyAsync(b.ctl + BQ_LO + lo_next, h, sizeof(int32_t), cudaMemcpyHostToDevice, st));
    BqSplitOut o{b.stamp, b.lo[lo_next], b.ctl + BQ_LO + lo_next, bq_lo_tag(pq->gen_lo + 1),
                 nullptr, nullptr, 0, INT_MAX, nullptr, b.V, false};
    if (split_hi) {
      pq->width = bq_adapt_width(pq->width, fill, 4096);
      pq->horizon = bq_clamp((int64_t)m + (int64_t)pq->width * pq->delta);
      GG_CUDA(cudaMemcpyAsync(b.ctl + BQ_HI + hi_next, h, sizeof(int32_t), cudaMemcpyHostToDevice, st));
      GG_CUDA(cudaMemcpyAsync(b.ctl + BQ_FILL, h, sizeof(int32_t), cudaMemcpyHostToDevice, st));
      o.hi = b.hi[hi_next];
      o.hi_cnt = b.ctl + BQ_HI + hi_next;
      o.hi_tag = bq_hi_tag(pq->gen_hi + 1);
      o.horizon = pq->horizon;
      o.dedup = !from_hi;  // both piles feed the next low pile
    }
    if (!from_hi) {
      note_launch();
      k_bq_split<<<grid, kPqThreads, 0, st>>>(b.lo[lo], b.ctl + BQ_LO + lo, pq->prio, U, win, front, o, g->d_err);
      GG_CUDA(cudaGetLastError());
    }
    if (split_hi) {
      o.fill = b.ctl + BQ_FILL;
      note_launch();
      k_bq_split<<<grid, kPqThreads, 0, st>>>(b.hi[hi], b.ctl + BQ_HI + hi, pq->prio, U, win, front, o, g->d_err);
      GG_CUDA(cudaGetLastError());
      pq->gen_hi++;
    }
    pq->gen_lo++;
    pq->cur = m;
  }
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
  pq->gen_lo = 0;
  pq->gen_hi = 0;
  pq->width = 16;
  pq->horizon = bq_clamp((int64_t)init_priority + (int64_t)pq->width * delta);
  gg_frontier *f = pq->frontier;
  gg_graph *g = pq->g;
  GG_TRY(bq_start(pq->bq, 0, g->stream));
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
  s = bq_alloc(g, &pq->bq);
  if (s == GG_OK) s = pq_reset(pq, init_priority, delta, src);
  if (s != GG_OK) {
    bq_free(g, &pq->bq);
    pq->frontier->owned_by_pq = false;
    gg_frontier_destroy(pq->frontier);
    delete pq;
    return s;
  }
  *out = pq;
  return GG_OK;
}

gg_status gg_pq_destroy(gg_pq *pq) {
  if (!pq) return GG_OK;
  bq_free(pq->g, &pq->bq);
  pq->frontier->owned_by_pq = false;
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
  d.far = pq_far(pq);
  GG_TRY(edgeset_apply_impl(g, s, GG_UDF_SSSP_RELAX, GG_FILTER_NONE, pq->frontier, pq->frontier,
                            true, d, pq_cutoff(pq), false));
  return check_device_error(g, "apply_priority");
}

}  // extern "C"
