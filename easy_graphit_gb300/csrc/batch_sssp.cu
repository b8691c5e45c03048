// Batched SSSP: up to 32 sources per pass, delta-stepping per source, one
// persistent kernel.
//
// Layout: distances are vertex-major, dist[v*32 + s], so the 32 sources of a
// vertex share one 128-byte line.  A warp owns one queue entry (a vertex u and
// a chunk of at most S.chunk of its edges); lane s relaxes source s.  For each
// edge the warp loads one line of dist[v][*] and issues atomicMin only where a
// source improves, so an edge is read once for all sources that have u on their
// frontier.
//
// Delta-stepping (gpu_priority_queue.h semantics, per source): source s relaxes
// with cutoff cur[s]+delta; an improvement below the cutoff sets s in v's near
// mask and queues v, one at or above it sets s in v's far mask and puts v on the
// far list.  When source s has no near work left, it advances: cur[s] becomes
// the smallest far priority >= cur[s]+delta, and far entries inside
// [cur[s], cur[s]+delta) move to the near frontier.  Every vertex whose priority
// is at or above the window was last improved at or above a cutoff, so the far
// list holds exactly the candidates the reference finds by scanning all V.
//
// Iteration: relax | barrier | publish near masks, collect the active sources |
// barrier | [advance pass 1 (minima) | barrier | pass 2 (move/keep) | barrier].
#include <algorithm>

#include "batch.h"

namespace gg {

constexpr int32_t kLanes = kBsLanes;
constexpr int32_t kPrefetch = 8;  // distance lines in flight per warp
// Queue entries active for at most S.ep_max sources are relaxed edge-parallel
// (lanes = edges); busier ones source-parallel (lanes = sources).  S.chunk
// (edges per queue entry) and S.ep_max come from the graph's batch tuning.

__device__ __forceinline__ void bs_enqueue(const BsState &S, int64_t *q, int32_t *qcnt, int32_t v) {
  const int32_t deg = S.off[v + 1] - S.off[v];
  const int32_t nch = max(1, ceil_div(deg, S.chunk));
  const int32_t pos = atomicAdd(qcnt, nch);
  if ((int64_t)pos + nch > S.qcap) {
    atomicOr(S.err, DEV_ERR_OVERFLOW);
    return;
  }
  for (int32_t c = 0; c < nch; ++c) q[pos + c] = ((int64_t)v << 32) | (uint32_t)c;
}

__global__ void __launch_bounds__(256) k_bsssp(BsState S) {
  __shared__ int32_t red[256 / 32][kLanes];
  const int32_t lane = threadIdx.x & 31;
  const int32_t wib = threadIdx.x >> 5;
  const int64_t gwarp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int32_t tstride = gridDim.x * blockDim.x;
  const int32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  int in = 0;
  int64_t adv = 0;
  int32_t it = 1;
  LoopClock clk;
  clk.start(S.loop_limit_ns);
  for (;; ++it) {
    if (stopped(S.stop, S.err)) break;
    const int32_t n = *(volatile int32_t *)(S.cnt + (it - 1) % 3);
    int32_t *qcnt_out = S.cnt + it % 3;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      S.cnt[(it + 1) % 3] = 0;
      S.cnt[5 + (it + 1) % 3] = 0;
    }
    const int p = (int)(adv & 1);
    // ---- relax
    {
      const int32_t curl = __ldcg(S.cur + p * kLanes + lane);
      const int64_t cl = (int64_t)curl + S.delta;
      const int32_t cut = cl > INT_MAX ? INT_MAX : (int32_t)cl;
      const int64_t *qi = S.q[in];
      int64_t *qo = S.q[in ^ 1];
      for (int64_t e = gwarp; e < n; e += nwarps) {
        const int64_t item = __ldcg(qi + e);
        const int32_t u = (int32_t)(item >> 32);
        const int32_t c = (int32_t)(item & 0xffffffff);
        const uint32_t m = __ldcg(S.fr + u);
        if (!m) continue;
        const bool act = (m >> lane) & 1u;
        const int32_t du = act ? __ldcg(S.dist + (int64_t)u * kLanes + lane) : INT_MAX;
        const int32_t b = S.off[u] + c * S.chunk;
        const int32_t eend = min(b + S.chunk, S.off[u + 1]);
        if (__popc(m) <= S.ep_max) {
          // Few active sources: lanes take edges, the warp loops over sources.
          uint32_t mm = m;
          while (mm) {
            const int32_t s = __ffs(mm) - 1;
            mm &= mm - 1;
            const int32_t du_s = __shfl_sync(0xffffffffu, du, s);
            const int32_t cut_s = __shfl_sync(0xffffffffu, cut, s);
            if (du_s == INT_MAX) continue;
            for (int32_t k = b + lane; k < eend; k += 32) {
              const int32_t v = __ldg(S.dst + k);
              const int32_t np = du_s + __ldg(S.w + k);
              int32_t *pd = S.dist + (int64_t)v * kLanes + s;
              if (np < __ldcg(pd) && atomicMin(pd, np) > np) {
                if (np < cut_s) {
                  atomicOr(S.nacc + v, 1u << s);
                  if (atomicMax(S.qstamp + v, it) < it) bs_enqueue(S, qo, qcnt_out, v);
                } else if (atomicOr(S.far + v, 1u << s) == 0u) {
                  const int32_t pos = atomicAdd(S.cnt + 3 + p, 1);
                  if (pos < S.V)
                    S.fl[p][pos] = v;
                  else
                    atomicOr(S.err, DEV_ERR_OVERFLOW);
                }
              }
            }
          }
          continue;
        }
        for (int32_t k0 = b; k0 < eend; k0 += 32) {
          int32_t vv = 0, ww = 0;
          if (k0 + lane < eend) {
            vv = __ldg(S.dst + k0 + lane);
            ww = __ldg(S.w + k0 + lane);
          }
          const int32_t cnt = min(32, eend - k0);
          const bool live = act && du != INT_MAX;
          for (int32_t j0 = 0; j0 < cnt; j0 += kPrefetch) {
            // Issue the distance-line loads of kPrefetch edges before using
            // them.  A stale (larger) value only costs an extra atomicMin.
            int32_t vs[kPrefetch], ws[kPrefetch], dvs[kPrefetch];
#pragma unroll
            for (int32_t t = 0; t < kPrefetch; ++t) {
              vs[t] = __shfl_sync(0xffffffffu, vv, (j0 + t) & 31);
              ws[t] = __shfl_sync(0xffffffffu, ww, (j0 + t) & 31);
              dvs[t] = (live && j0 + t < cnt) ? __ldcg(S.dist + (int64_t)vs[t] * kLanes + lane) : INT_MIN;
            }
#pragma unroll
            for (int32_t t = 0; t < kPrefetch; ++t) {
              if (j0 + t >= cnt) break;  // warp-uniform
              const int32_t v = vs[t];
              bool near = false, farb = false;
              if (live) {
                const int32_t np = du + ws[t];
                if (np < dvs[t] && atomicMin(S.dist + (int64_t)v * kLanes + lane, np) > np) {
                  near = np < cut;
                  farb = !near;
                }
              }
              const uint32_t nb = __ballot_sync(0xffffffffu, near);
              const uint32_t fb = __ballot_sync(0xffffffffu, farb);
              if (lane == 0) {
                if (nb) {
                  atomicOr(S.nacc + v, nb);
                  if (atomicMax(S.qstamp + v, it) < it) bs_enqueue(S, qo, qcnt_out, v);
                }
                if (fb && atomicOr(S.far + v, fb) == 0u) {
                  const int32_t pos = atomicAdd(S.cnt + 3 + p, 1);
                  if (pos < S.V)
                    S.fl[p][pos] = v;
                  else
                    atomicOr(S.err, DEV_ERR_OVERFLOW);
                }
              }
            }
          }
        }
      }
    }
    if (!grid_barrier(S.bar, gridDim.x, S.err, S.timeout_ns)) break;
    // ---- publish near masks of the queued vertices; OR them into the active set
    {
      const int32_t mq = *(volatile int32_t *)qcnt_out;
      const int64_t *qo = S.q[in ^ 1];
      uint32_t act = 0;
      for (int32_t e = tid; e < ceil_div(mq, tstride) * tstride; e += tstride) {
        uint32_t x = 0;
        if (e < mq) {
          const int64_t item = __ldcg(qo + e);
          if ((item & 0xffffffff) == 0) {
            const int32_t v = (int32_t)(item >> 32);
            x = __ldcg(S.nacc + v);
            S.nacc[v] = 0;
            S.fr[v] = x;
          }
        }
        act |= x;
      }
      act = __reduce_or_sync(0xffffffffu, act);
      if (lane == 0 && act) atomicOr(reinterpret_cast<uint32_t *>(S.cnt + 5 + it % 3), act);
    }
    clk.tick(S.stop);
    if (!grid_barrier(S.bar, gridDim.x, S.err, S.timeout_ns)) break;
    // ---- advance the sources with no near work
    uint32_t unfinished = 0;
    {
      const int32_t cv = __ldcg(S.cur + p * kLanes + lane);
      unfinished = __ballot_sync(0xffffffffu, cv != INT_MAX);
    }
    const uint32_t active = (uint32_t)*(volatile int32_t *)(S.cnt + 5 + it % 3);
    const uint32_t A = unfinished & ~active;
    if (A) {
      const int32_t fcount = *(volatile int32_t *)(S.cnt + 3 + p);
      const int32_t *fla = S.fl[p];
      const int32_t curl = __ldcg(S.cur + p * kLanes + lane);
      const int64_t window = (int64_t)curl + S.delta;
      const bool adv_l = (A >> lane) & 1u;
      if (blockIdx.x == 0 && threadIdx.x < kLanes) {
        S.gmin[(p ^ 1) * kLanes + threadIdx.x] = INT_MAX;
        if (threadIdx.x == 0) S.cnt[3 + (p ^ 1)] = 0;
      }
      // pass 1: per-source minimum far priority at or above the window
      int32_t mn = INT_MAX;
      for (int64_t e = gwarp; e < fcount; e += nwarps) {
        const int32_t v = __ldcg(fla + e);
        const uint32_t fm = __ldcg(S.far + v);
        if (adv_l && ((fm >> lane) & 1u)) {
          const int32_t d = __ldcg(S.dist + (int64_t)v * kLanes + lane);
          if ((int64_t)d >= window && d < mn) mn = d;
        }
      }
      red[wib][lane] = mn;
      __syncthreads();
      if (threadIdx.x < kLanes) {
        int32_t m = INT_MAX;
        for (int32_t k = 0; k < (int32_t)(blockDim.x >> 5); ++k) m = min(m, red[k][threadIdx.x]);
        if (m != INT_MAX) atomicMin(S.gmin + p * kLanes + threadIdx.x, m);
      }
      if (!grid_barrier(S.bar, gridDim.x, S.err, S.timeout_ns)) break;
      // pass 2: move [cur', cur'+delta) to the near frontier, keep the rest
      const int32_t g = __ldcg(S.gmin + p * kLanes + lane);
      const int32_t newcur = adv_l ? g : curl;
      const int64_t hi = (int64_t)newcur + S.delta;
      int64_t *qo = S.q[in ^ 1];
      for (int64_t e = gwarp; e < fcount; e += nwarps) {
        const int32_t v = __ldcg(fla + e);
        const uint32_t fm = __ldcg(S.far + v);
        const bool f = (fm >> lane) & 1u;
        bool keep = false, move = false;
        if (f) {
          if (!adv_l) {
            keep = true;
          } else if (newcur != INT_MAX) {
            const int32_t d = __ldcg(S.dist + (int64_t)v * kLanes + lane);
            if ((int64_t)d >= window) {
              if ((int64_t)d < hi)
                move = true;
              else
                keep = true;
            }
          }
        }
        const uint32_t rem = __ballot_sync(0xffffffffu, keep);
        const uint32_t mv = __ballot_sync(0xffffffffu, move);
        if (lane == 0) {
          S.far[v] = rem;
          if (rem) {
            const int32_t pos = atomicAdd(S.cnt + 3 + (p ^ 1), 1);
            if (pos < S.V)
              S.fl[p ^ 1][pos] = v;
            else
              atomicOr(S.err, DEV_ERR_OVERFLOW);
          }
          if (mv) {
            if (atomicMax(S.qstamp + v, it) < it) {
              S.fr[v] = mv;
              bs_enqueue(S, qo, qcnt_out, v);
            } else {
              atomicOr(S.fr + v, mv);
            }
          }
        }
      }
      if (blockIdx.x == 0 && threadIdx.x < kLanes) S.cur[(p ^ 1) * kLanes + threadIdx.x] = newcur;
      if (!grid_barrier(S.bar, gridDim.x, S.err, S.timeout_ns)) break;
      ++adv;
    }
    const int32_t m = *(volatile int32_t *)qcnt_out;
    if (m == 0) break;
    in ^= 1;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    S.stats[0] = it;
    S.stats[1] = (int32_t)adv;
  }
}

__global__ void k_bsssp_init(BsState S, const int32_t *__restrict__ srcs, int32_t nsrc) {
  const int64_t total = (int64_t)S.V * kLanes;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x)
    S.dist[i] = INT_MAX;
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < S.V; v += gridDim.x * blockDim.x) {
    S.fr[v] = 0;
    S.nacc[v] = 0;
    S.far[v] = 0;
    S.qstamp[v] = 0;
  }
}

__global__ void k_bsssp_seed(BsState S, const int32_t *__restrict__ srcs, int32_t nsrc) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  for (int32_t i = 0; i < 8; ++i) S.cnt[i] = 0;
  *S.stop = 0;
  for (int32_t s = 0; s < kLanes; ++s) {
    S.cur[s] = s < nsrc ? 0 : INT_MAX;
    S.cur[kLanes + s] = S.cur[s];
    S.gmin[s] = INT_MAX;
    S.gmin[kLanes + s] = INT_MAX;
  }
  for (int32_t s = 0; s < nsrc; ++s) {
    const int32_t v = srcs[s];
    S.dist[(int64_t)v * kLanes + s] = 0;
    if (!S.fr[v]) bs_enqueue(S, S.q[0], S.cnt + 0, v);
    S.fr[v] |= 1u << s;
  }
}

__global__ void k_bsssp_out(const int32_t *__restrict__ dist, int32_t V, int32_t nsrc,
                            int32_t *__restrict__ out) {
  const int64_t total = (int64_t)nsrc * V;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t s = (int32_t)(i / V), v = (int32_t)(i % V);
    out[i] = dist[(int64_t)v * kLanes + s];
  }
}

// ------------------------------------------------------------------ host
BsBuffers::~BsBuffers() {
  if (owned)
    for (void *p : {(void *)dist, (void *)masks, (void *)ints, (void *)queues, (void *)out, (void *)dsrc})
      if (p) cudaFree(p);
}

gg_status bsssp_buffers(gg_graph *g, int32_t nsrc, bool owned, BsBuffers *b) {
  const int32_t V = g->csr.V;
  const int64_t E = g->csr.E;
  b->qcap = (int64_t)V + E / kMinChunk + 64;  // any tuning's chunk fits
  b->owned = owned;
  const size_t sz[6] = {sizeof(int32_t) * (size_t)V * kLanes, sizeof(uint32_t) * 3 * (size_t)V,
                        sizeof(int32_t) * (3 * (size_t)V + 256), sizeof(int64_t) * 2 * (size_t)b->qcap,
                        sizeof(int32_t) * (size_t)std::min(nsrc, kLanes) * V,
                        sizeof(int32_t) * (size_t)std::max(nsrc, kLanes)};
  void **ptr[6] = {(void **)&b->dist, (void **)&b->masks, (void **)&b->ints, (void **)&b->queues,
                   (void **)&b->out, (void **)&b->dsrc};
  for (int i = 0; i < 6; ++i) {
    if (owned)
      GG_CUDA(cudaMalloc(ptr[i], sz[i]));
    else
      GG_TRY(scratch_get_app(g, i, sz[i], ptr[i]));
  }
  return GG_OK;
}

BsState bsssp_state(gg_graph *g, const BsBuffers &b, int32_t delta) {
  const int32_t V = g->csr.V;
  BsState S{};
  S.dist = b.dist;
  S.fr = b.masks;
  S.nacc = b.masks + V;
  S.far = b.masks + 2 * (size_t)V;
  S.qstamp = b.ints;
  S.fl[0] = b.ints + V;
  S.fl[1] = b.ints + 2 * (size_t)V;
  int32_t *hdr = b.ints + 3 * (size_t)V;
  S.cnt = hdr;              // 8
  S.cur = hdr + 8;          // 64
  S.gmin = hdr + 72;        // 64
  S.stats = hdr + 136;      // 2
  S.stop = hdr + 140;
  S.q[0] = b.queues;
  S.q[1] = b.queues + b.qcap;
  S.qcap = b.qcap;
  S.off = g->csr.off;
  S.dst = g->csr.dst;
  S.w = g->csr.w;
  S.V = V;
  S.delta = delta;
  const gg_batch_tuning t = effective_tuning(g, GG_BATCH_SSSP, 1);
  S.chunk = t.chunk;
  S.ep_max = t.edge_parallel_max;
  S.bar = g->d_bar;
  S.err = g->d_err;
  S.timeout_ns = barrier_timeout_ns();
  S.loop_limit_ns = loop_timeout_ns();
  return S;
}

const void *bsssp_kernel() { return (const void *)k_bsssp; }

// One group of k <= 32 sources (device array dsrc): reset, seed, the
// persistent loop, and the per-source rows into out_rows.  Issues only
// stream-ordered work, so it can be captured into a CUDA graph.
gg_status bsssp_enqueue(gg_graph *g, cudaStream_t st, const BsState &S, const int32_t *dsrc, int32_t k,
                        int32_t *out_rows, bool timed) {
  int per_sm = 0;
  GG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bsssp, 256, 0));
  if (per_sm < 1) return set_error(GG_ERR_UNSUPPORTED, "batched SSSP kernel does not fit an SM");
  note_launch();
  k_bsssp_init<<<g->sm_count * 8, 256, 0, st>>>(S, dsrc, k);
  note_launch();
  k_bsssp_seed<<<1, 32, 0, st>>>(S, dsrc, k);
  GG_CUDA(cudaMemsetAsync(S.bar, 0, sizeof(uint32_t) * 2, st));
  BsState arg = S;
  void *args[] = {&arg};
  if (timed) GG_CUDA(cudaEventRecord(g->ev2, st));
  note_launch();
  const int bps = effective_tuning(g, GG_BATCH_SSSP, per_sm).blocks_per_sm;
  GG_CUDA(cudaLaunchCooperativeKernel((const void *)k_bsssp, bps * g->sm_count, 256, args, 0, st));
  if (timed) GG_CUDA(cudaEventRecord(g->ev3, st));
  note_launch();
  k_bsssp_out<<<g->sm_count * 8, 256, 0, st>>>(S.dist, S.V, k, out_rows);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

}  // namespace gg

using namespace gg;

// Batched delta-stepping SSSP from nsrc sources: dist_out[s*V + v].
extern "C" gg_status gg_sssp_batch(gg_graph *g, const int32_t *sources, int32_t nsrc, int32_t delta,
                                   int32_t *dist_out, gg_stats *stats) {
  GG_CHECK_ARG(g && sources && nsrc > 0 && dist_out, "bad arguments");
  GG_CHECK_ARG(delta >= 1, "delta must be >= 1");
  const int32_t V = g->csr.V;
  for (int32_t i = 0; i < nsrc; ++i)
    GG_CHECK_ARG(sources[i] >= 0 && sources[i] < V, "source out of range");
  if (stats) *stats = gg_stats{};
  cudaStream_t st = g->stream;
  BsBuffers b;
  GG_TRY(bsssp_buffers(g, nsrc, false, &b));
  const BsState S = bsssp_state(g, b, delta);
  const uint64_t l0 = launches();
  cudaEventRecord(g->ev0, st);
  float loop_ms = 0;
  int32_t iters = 0, advs = 0;
  for (int32_t base = 0; base < nsrc; base += kLanes) {
    const int32_t k = std::min(kLanes, nsrc - base);
    GG_CUDA(cudaMemcpyAsync(b.dsrc, sources + base, sizeof(int32_t) * k, cudaMemcpyDefault, st));
    GG_TRY(bsssp_enqueue(g, st, S, b.dsrc, k, b.out, true));
    GG_CUDA(cudaMemcpyAsync(dist_out + (size_t)base * V, b.out, sizeof(int32_t) * (size_t)k * V,
                            cudaMemcpyDefault, st));
    GG_CUDA(cudaMemcpyAsync(g->h_pinned + 30, S.stats, sizeof(int32_t) * 2, cudaMemcpyDeviceToHost, st));
    GG_CUDA(cudaStreamSynchronize(st));
    float ms = 0;
    cudaEventElapsedTime(&ms, g->ev2, g->ev3);
    loop_ms += ms;
    iters = std::max(iters, g->h_pinned[30]);
    advs += g->h_pinned[31];
  }
  cudaEventRecord(g->ev1, st);
  GG_CUDA(cudaEventSynchronize(g->ev1));
  GG_TRY(check_device_error(g, "sssp_batch"));
  if (stats) {
    cudaEventElapsedTime(&stats->device_ms, g->ev0, g->ev1);
    stats->loop_ms = loop_ms;
    stats->iterations = iters;
    stats->bucket_advances = advs;
    stats->fused = 1;
    stats->launches = (int32_t)(launches() - l0);
  }
  return GG_OK;
}
