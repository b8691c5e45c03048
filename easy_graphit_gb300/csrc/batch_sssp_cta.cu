// Batched SSSP for high-diameter graphs: every source gets a CTA of its own,
// which runs the whole delta-stepping loop of bq_loop.cuh for that source
// alone -- its frontier queues, far piles and stamps private to it, its control
// words in shared memory, __syncthreads between steps and no grid barrier at
// all.  The CTAs of a pass run side by side, one source each.
//
// Why: on a mesh such as the 4096^2 grid, a 32-source pass of the lane-per-
// source kernel (batch_sssp.cu) needs ~10^5 iterations of three grid-wide
// phases each, for a handful of vertices per source per iteration; the time
// goes to barriers.  Here a bucket of a source costs the few L2 round trips of
// its own steps.  On low-diameter graphs (R-MAT) a source's buckets are large
// and one CTA per source is too little parallelism: the lane-per-source
// kernel stays the choice there (gg_batch_tuning.per_source_cta).
//
// Results are each source's exact distances (the bucket rule of
// gpu_priority_queue.h, as in the single-source loop).
#include <vector>

#include "batch.h"
#include "bq_loop.cuh"

namespace gg {

struct CtaSsspArgs {
  DGraph g;
  const int32_t *srcs;  // k sources
  int32_t *rows;        // [k][V] distances (parts mode: one row of V)
  int32_t *q;           // [k][2][qcap] frontier queues
  int64_t qcap;
  int32_t *stamp;       // [k][V]
  int32_t *piles;       // [k][4][V]: low piles of both generations, then the high ones
  int32_t V, delta;
  int32_t *err;
  int32_t *stats;       // [0] most relax steps of a source, [1] bucket advances of all sources
  uint64_t loop_limit_ns;
  // Parts mode (gg_sssp_parts): CTA k owns the vertices [part_lo[k],
  // part_lo[k+1]) of a disjoint union and one row of distances and stamps;
  // its piles and queues start at piles + part_base[k].
  const int32_t *part_lo;
  const int64_t *part_base;
};

// Piles (4 of cap) and queues (2 of 2 cap) of a part of Vp vertices.
__host__ __device__ __forceinline__ int64_t part_cap(int64_t Vp) { return Vp > 512 ? Vp : 512; }

// Distances (INT_MAX, 0 at the source) and stamps of every source's row.
__global__ void k_sssp_cta_init(CtaSsspArgs c, int32_t k) {
  const int64_t V = c.V, total = (int64_t)k * V;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t s = (int32_t)(i / V);
    const int32_t v = (int32_t)(i - (int64_t)s * V);
    c.rows[i] = v == c.srcs[s] ? 0 : INT_MAX;
    c.stamp[i] = 0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    c.stats[0] = 0;
    c.stats[1] = 0;
  }
}

template <int LB>
__global__ void __launch_bounds__(512) k_sssp_cta(CtaSsspArgs c) {
  extern __shared__ int4 smem[];
  __shared__ int32_t red[33];
  __shared__ int32_t sctl[BQ_STOP];
  __shared__ int32_t s_quit;
  const int64_t k = blockIdx.x, V = c.V;
  BqArgs a{};
  a.g = c.g;
  if (c.part_lo) {
    const int32_t Vp = c.part_lo[k + 1] - c.part_lo[k];
    const int64_t cap = part_cap(Vp);
    int32_t *pl = c.piles + c.part_base[k];
    a.b.lo[0] = pl;
    a.b.lo[1] = pl + cap;
    a.b.hi[0] = pl + 2 * cap;
    a.b.hi[1] = pl + 3 * cap;
    a.q0 = pl + 4 * cap;
    a.q1 = a.q0 + 2 * cap;
    a.qcap = 2 * cap;
    a.dist = c.rows;
    a.b.stamp = c.stamp;
    a.b.V = Vp;
    if (threadIdx.x == 0) a.dist[c.srcs[k]] = 0;
  } else {
    a.q0 = c.q + k * 2 * c.qcap;
    a.q1 = a.q0 + c.qcap;
    a.qcap = c.qcap;
    a.dist = c.rows + k * V;
    a.b.stamp = c.stamp + k * V;
    int32_t *pl = c.piles + k * 4 * V;
    a.b.lo[0] = pl;
    a.b.lo[1] = pl + V;
    a.b.hi[0] = pl + 2 * V;
    a.b.hi[1] = pl + 3 * V;
    a.b.V = c.V;
  }
  a.err = c.err;
  a.delta = c.delta;
  a.fill_target = 1024;
  a.width0 = 16;
  a.rec_mode = 1;
  if (threadIdx.x < BQ_STOP) {
    const int32_t i = threadIdx.x;
    const bool big = (i >= BQ_MIN && i < BQ_MIN + 3) || (i >= BQ_REC && i < BQ_REC + 2);
    sctl[i] = i == BQ_NEAR ? 1 : (big ? INT_MAX : (i == BQ_FILL ? -1 : 0));
  }
  if (threadIdx.x == 0) a.q0[0] = c.srcs[k];
  __syncthreads();
  BqLoop s{1, 0, 0, 0, 0, bq_clamp((int64_t)a.width0 * a.delta), a.width0, 0, 0, 0};
  uint64_t deadline = 0;
  if (threadIdx.x == 0) deadline = globaltimer_ns() + c.loop_limit_ns;
  for (uint32_t n = 0;; ++n) {
    if ((n & 255u) == 0) {  // the wall-clock bound and overflow, checked every 256 steps
      if (threadIdx.x == 0) {
        const bool late = globaltimer_ns() > deadline;
        if (late) atomicOr(c.err, DEV_ERR_TIMEOUT);
        s_quit = late || (*(volatile int32_t *)c.err & (DEV_ERR_OVERFLOW | DEV_ERR_TIMEOUT)) != 0;
      }
      __syncthreads();
      const bool quit = s_quit != 0;
      __syncthreads();
      if (quit) break;
    }
    const BqStep st = bq_decide(s, sctl, c.delta);
    if (st.kind == BQ_DONE) {
      if (s.phase == 0) s.adv++;  // the reference's last advance finds no priority left
      break;
    }
    bq_step<LB>(s, a, st, sctl, 0, 1, smem, red);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    atomicMax(c.stats, s.relax);
    atomicAdd(c.stats + 1, s.adv);
  }
}

// Sources per pass: one CTA each; per source V ints of distances, V of
// stamps, 4 V of piles and 2 qcap of frontier queues, within a 24 GB budget.
int32_t bsssp_cta_width(const gg_graph *g) {
  const size_t V = (size_t)std::max(g->csr.V, 512);
  const size_t per = sizeof(int32_t) * (6 * V + 4 * V);
  const size_t budget = size_t(24) << 30;
  return (int32_t)std::max<size_t>(1, std::min<size_t>(kBsLanes, budget / per));
}

gg_status bsssp_cta_buffers(gg_graph *g, int32_t k, Scratch *sc, CtaBuffers *b) {
  const size_t V = (size_t)g->csr.V;
  b->qcap = 2 * (int64_t)std::max<size_t>(V, 512);
  const size_t ints = (size_t)k * 6 * V + (size_t)k * 2 * b->qcap + k + 8;
  if (sc->bytes < sizeof(int32_t) * ints) {
    if (sc->p) cudaFreeAsync(sc->p, g->stream);
    sc->p = nullptr;
    sc->bytes = 0;
    GG_CUDA(dev_alloc(&sc->p, sizeof(int32_t) * ints, g->stream));
    sc->bytes = sizeof(int32_t) * ints;
  }
  int32_t *p = static_cast<int32_t *>(sc->p);
  b->stats = p;  // 8
  b->dsrc = p + 8;
  b->rows = b->dsrc + k;
  b->stamp = b->rows + (size_t)k * V;
  b->piles = b->stamp + (size_t)k * V;
  b->q = b->piles + (size_t)k * 4 * V;
  b->k = k;
  return GG_OK;
}

// One pass over the k sources in b.dsrc: distance rows rows[k][V] (device
// memory), stats b.stats.  Stream-ordered only (capturable).
gg_status bsssp_cta_run(gg_graph *g, cudaStream_t st, const CtaBuffers &b, int32_t *rows, int32_t k,
                        int32_t delta, bool timed) {
  CtaSsspArgs c{};
  c.g = g->csr.view();
  c.g.nbuckets = 0;
  c.srcs = b.dsrc;
  c.rows = rows;
  c.stamp = b.stamp;
  c.piles = b.piles;
  c.q = b.q;
  c.qcap = b.qcap;
  c.V = g->csr.V;
  c.delta = delta;
  c.err = g->d_err;
  c.stats = b.stats;
  c.loop_limit_ns = loop_timeout_ns();
  note_launch();
  k_sssp_cta_init<<<g->sm_count * 8, 256, 0, st>>>(c, k);
  GG_CUDA(cudaGetLastError());
  if (timed) GG_CUDA(cudaEventRecord(g->ev2, st));
  note_launch();
  k_sssp_cta<GG_LB_VERTEX_BASED><<<k, 512, 0, st>>>(c);
  GG_CUDA(cudaGetLastError());
  if (timed) GG_CUDA(cudaEventRecord(g->ev3, st));
  return GG_OK;
}

__global__ void k_max_degree(const int32_t *__restrict__ off, int32_t V, int32_t *out) {
  int32_t m = 0;
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
    m = max(m, __ldg(off + v + 1) - __ldg(off + v));
  m = __reduce_max_sync(0xffffffffu, m);
  if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

// Largest out-degree of the graph (computed once, then cached).
gg_status graph_max_degree(gg_graph *g, int32_t *out) {
  if (g->max_degree < 0) {
    int32_t *d = g->d_misc + 60;
    GG_CUDA(cudaMemsetAsync(d, 0, sizeof(int32_t), g->stream));
    note_launch();
    k_max_degree<<<g->sm_count * 4, 256, 0, g->stream>>>(g->csr.off, g->csr.V, d);
    GG_CUDA(cudaGetLastError());
    GG_CUDA(cudaMemcpyAsync(g->h_pinned + 60, d, sizeof(int32_t), cudaMemcpyDeviceToHost, g->stream));
    GG_CUDA(cudaStreamSynchronize(g->stream));
    g->max_degree = g->h_pinned[60];
  }
  *out = g->max_degree;
  return GG_OK;
}

// The per-source-CTA mode applies when the tuning asks for it, or by default
// on graphs without hubs (largest out-degree at most kMeshDegree): meshes and
// road-like graphs, whose diameter makes the lane-per-source kernel barrier-bound.
constexpr int32_t kMeshDegree = 32;
gg_status bsssp_use_cta(gg_graph *g, bool *use) {
  const int32_t mode = g->tuning[GG_BATCH_SSSP].per_source_cta;
  if (mode != 0) {
    *use = mode > 0;
    return GG_OK;
  }
  int32_t md = 0;
  GG_TRY(graph_max_degree(g, &md));
  *use = md <= kMeshDegree;
  return GG_OK;
}

// Parts mode: every distance INT_MAX and every stamp 0 (the CTAs set their
// sources' distances).
__global__ void k_sssp_parts_init(int32_t *dist, int32_t *stamp, int32_t V, int32_t *stats) {
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    dist[v] = INT_MAX;
    stamp[v] = 0;
  }
  if (blockIdx.x == 0 && threadIdx.x < 8) stats[threadIdx.x] = 0;
}

// Sets *bad when an edge leaves its part (block p walks part p).
__global__ void k_parts_check(const int32_t *__restrict__ off, const int32_t *__restrict__ dst,
                              const int32_t *__restrict__ part_lo, int32_t *bad) {
  const int32_t lo = part_lo[blockIdx.x], hi = part_lo[blockIdx.x + 1];
  bool out = false;
  for (int32_t v = lo + threadIdx.x; v < hi; v += blockDim.x)
    for (int32_t e = off[v]; e < off[v + 1]; ++e) {
      const int32_t u = dst[e];
      out |= u < lo || u >= hi;
    }
  if (__syncthreads_or(out) && threadIdx.x == 0) atomicOr(bad, 1);
}

}  // namespace gg

using namespace gg;

// SSSP on a disjoint union of graphs, one source per part, every part's
// delta-stepping loop in a CTA of its own (no grid barrier; the parts run side
// by side).  The batched mode's answer for many small or high-diameter graphs,
// whose single-source loops are barrier-bound.  Each result equals that part's
// own gg_sssp (the bucket rule of gpu_priority_queue.h).
extern "C" gg_status gg_sssp_parts(gg_graph *g, const int32_t *part_begin, int32_t nparts,
                                   const int32_t *sources, int32_t delta, int32_t *dist_out, gg_stats *stats) {
  GG_CHECK_ARG(g && part_begin && sources && nparts >= 1, "bad arguments");
  GG_CHECK_ARG(delta >= 1, "delta must be >= 1");
  const int32_t V = g->csr.V;
  GG_CHECK_ARG(part_begin[0] >= 0 && part_begin[nparts] <= V, "parts outside the graph");
  for (int32_t p = 0; p < nparts; ++p) {
    if (part_begin[p + 1] <= part_begin[p]) return set_error(GG_ERR_INVALID, "part %d is empty", p);
    if (sources[p] < part_begin[p] || sources[p] >= part_begin[p + 1])
      return set_error(GG_ERR_INVALID, "the source of part %d lies outside it", p);
  }
  if (stats) *stats = gg_stats{};
  cudaStream_t st = g->stream;
  std::vector<int64_t> base(nparts);
  int64_t tot = 0;
  for (int32_t p = 0; p < nparts; ++p) {
    base[p] = tot;
    tot += 8 * part_cap(part_begin[p + 1] - part_begin[p]);
  }
  // ints: stats 8, sources, part_lo, part_base (int64), stamps, piles and queues
  const size_t head = 8 + (size_t)nparts + (size_t)nparts + 1 + 2 * (size_t)nparts + 2;
  const size_t ints = head + (size_t)V + (size_t)tot;
  Scratch *sc = &g->bq_cta;
  if (sc->bytes < sizeof(int32_t) * ints) {
    if (sc->p) cudaFreeAsync(sc->p, st);
    sc->p = nullptr;
    sc->bytes = 0;
    GG_CUDA(dev_alloc(&sc->p, sizeof(int32_t) * ints, st));
    sc->bytes = sizeof(int32_t) * ints;
  }
  int32_t *p32 = static_cast<int32_t *>(sc->p);
  int32_t *dstats = p32, *dsrc = p32 + 8, *dlo = dsrc + nparts;
  int64_t *dbase = reinterpret_cast<int64_t *>(p32 + ((8 + 2 * (size_t)nparts + 1 + 1) & ~(size_t)1));
  int32_t *stamp = reinterpret_cast<int32_t *>(dbase + nparts);
  int32_t *piles = stamp + V;
  int32_t *dist = nullptr;
  GG_TRY(scratch_get_app(g, 2, sizeof(int32_t) * (size_t)V, (void **)&dist));
  GG_CUDA(cudaMemcpyAsync(dsrc, sources, sizeof(int32_t) * nparts, cudaMemcpyHostToDevice, st));
  GG_CUDA(cudaMemcpyAsync(dlo, part_begin, sizeof(int32_t) * (nparts + 1), cudaMemcpyHostToDevice, st));
  GG_CUDA(cudaMemcpyAsync(dbase, base.data(), sizeof(int64_t) * nparts, cudaMemcpyHostToDevice, st));
  GG_CUDA(cudaEventRecord(g->ev0, st));
  note_launch();
  k_sssp_parts_init<<<g->sm_count * 8, 256, 0, st>>>(dist, stamp, V, dstats);
  GG_CUDA(cudaGetLastError());
  note_launch();
  k_parts_check<<<nparts, 256, 0, st>>>(g->csr.off, g->csr.dst, dlo, dstats + 7);
  GG_CUDA(cudaGetLastError());
  GG_CUDA(cudaMemcpyAsync(g->h_pinned + 61, dstats + 7, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  GG_CUDA(cudaStreamSynchronize(st));
  if (g->h_pinned[61]) return set_error(GG_ERR_INVALID, "an edge leaves its part: the parts are not a disjoint union");
  CtaSsspArgs c{};
  c.g = g->csr.view();
  c.g.nbuckets = 0;
  c.srcs = dsrc;
  c.rows = dist;
  c.stamp = stamp;
  c.piles = piles;
  c.V = V;
  c.delta = delta;
  c.err = g->d_err;
  c.stats = dstats;
  c.loop_limit_ns = loop_timeout_ns();
  c.part_lo = dlo;
  c.part_base = dbase;
  GG_CUDA(cudaEventRecord(g->ev2, st));
  note_launch();
  k_sssp_cta<GG_LB_VERTEX_BASED><<<nparts, 512, 0, st>>>(c);
  GG_CUDA(cudaGetLastError());
  GG_CUDA(cudaEventRecord(g->ev3, st));
  GG_CUDA(cudaEventRecord(g->ev1, st));
  GG_CUDA(cudaMemcpyAsync(g->h_pinned + 56, dstats, sizeof(int32_t) * 2, cudaMemcpyDeviceToHost, st));
  GG_CUDA(cudaStreamSynchronize(st));
  GG_TRY(check_device_error(g, "sssp_parts"));
  if (stats) {
    stats->iterations = g->h_pinned[56];
    stats->push_iterations = g->h_pinned[56];
    stats->bucket_advances = g->h_pinned[57];
    stats->fused = 1;
    stats->launches = 3;
    GG_CUDA(cudaEventElapsedTime(&stats->device_ms, g->ev0, g->ev1));
    GG_CUDA(cudaEventElapsedTime(&stats->loop_ms, g->ev2, g->ev3));
  }
  if (dist_out) GG_CUDA(cudaMemcpyAsync(dist_out, dist, sizeof(int32_t) * V, cudaMemcpyDefault, st));
  GG_TRY(app_reach_stats(g, dist, stats));
  GG_CUDA(cudaStreamSynchronize(st));
  return GG_OK;
}
