// Whole-loop persistent kernels: the fuse_kernel(true, ...) form of the BFS and
// SSSP loops (src/graphit/operators.cpp:652-672, gpu_intrinsics.h:113-117).
// One cooperatively launched grid (all CTAs co-resident) runs every iteration;
// the LB functions of lb.cuh process virtual CTAs, and a bounded grid barrier
// (common.cuh) separates iterations.  Frontier sizes never leave the device.
//
// Sparse-queue counts rotate through three slots: iteration L reads slot
// (L-1)%3, appends to slot L%3 and clears slot (L+1)%3, whose last reader
// finished before the previous barrier -- one barrier per iteration.
#include <cooperative_groups/reduce.h>

#include <cstdlib>

#include "bq_loop.cuh"
#include "bucket_queue.cuh"
#include "engine.h"
#include "lb.cuh"
#include "selector.h"
#include "udf.cuh"

namespace gg {

uint64_t barrier_timeout_ns() {
  static uint64_t t = [] {
    const char *e = getenv("GG_BARRIER_TIMEOUT_MS");
    const long ms = e ? atol(e) : 0;
    return (uint64_t)(ms > 0 ? ms : 30000) * 1000000ull;
  }();
  return t;
}

uint64_t loop_timeout_ns() {
  static uint64_t t = [] {
    const char *e = getenv("GG_LOOP_TIMEOUT_MS");
    const long ms = e ? atol(e) : 0;
    return (uint64_t)(ms > 0 ? ms : 120000) * 1000000ull;
  }();
  return t;
}

bool fused_supported(const gg_schedule *s) {
  if (s->direction != GG_PUSH || s->frontier_creation != GG_FC_SPARSE) return false;
  switch (s->load_balancing) {
    case GG_LB_VERTEX_BASED:
    case GG_LB_WM:
    case GG_LB_TWCE:
    case GG_LB_CM:
      return true;
    default:
      return false;
  }
}

struct FusedArgs {
  DGraph g;
  int32_t *q0, *q1;
  int32_t *cnt3;  // rotating counts [3]
  int64_t cap;
  uint32_t *bar;
  int32_t *err;
  uint64_t timeout_ns;
  int32_t *stats;  // [0] iterations, [1] bucket advances
  VData vd;
  int32_t delta;
  int32_t *gmin2;  // SSSP bucket-advance minima [2]
  int32_t *stop;   // loop time limit flag (see LoopClock)
  uint64_t loop_limit_ns;
};

__device__ __forceinline__ DOut sparse_out(const FusedArgs &a, int32_t *q, int64_t it) {
  DOut o{};
  o.mode = OUT_SPARSE;
  o.q = q;
  o.cnt = a.cnt3 + it % 3;
  o.cap = a.cap;
  o.err = a.err;
  return o;
}

template <int LB>
__global__ void __launch_bounds__(1024) k_bfs_fused(FusedArgs a) {
  extern __shared__ int4 smem[];
  int32_t *qs[2] = {a.q0, a.q1};
  int in = 0;
  int64_t level = 1;
  LoopClock clk;
  clk.start(a.loop_limit_ns);
  for (;; ++level) {
    const int32_t n = *(volatile int32_t *)(a.cnt3 + (level - 1) % 3);
    if (n == 0 || stopped(a.stop, (int32_t)level)) break;
    if (blockIdx.x == 0 && threadIdx.x == 0) a.cnt3[(level + 1) % 3] = 0;
    const Enum en{qs[in], nullptr, n};
    const EdgeF<UBfs, false> f{UBfs{a.vd.parent, a.vd.depth, (int32_t)level},
                               DIn{IN_ALL, nullptr, nullptr}, DIn{IN_ALL, nullptr, nullptr}, true};
    run_lb<LB>(a.g, en, n, f, sparse_out(a, qs[in ^ 1], level), smem, blockIdx.x, gridDim.x);
    clk.tick(a.stop, (int32_t)level, a.err);
    if (!grid_barrier(a.bar, gridDim.x, a.err, a.timeout_ns)) break;
    in ^= 1;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) a.stats[0] = (int32_t)(level - 1);
}

// ------------------------------------------------------ delta-stepping SSSP
// The persistent form of the bucket-queue loop of bq_loop.cuh: every CTA runs
// each step on its share and steps end at a grid barrier.
//
// One-CTA mode: a step whose work (frontier or pile entries) is small
// (bq_small) runs on CTA 0 alone, and so do the steps after it while they stay
// that small, separated by __syncthreads; the other CTAs wait at the grid
// barrier.  CTA 0 begins only when all of them have arrived there: its first
// steps clear control words that a slower CTA could otherwise still be reading
// to take the same decision.  CTA 0 returns to the barrier when the work
// grows, the loop ends or kSoloSliceNs has passed (so the waiting CTAs see a
// barrier complete at least that often), and publishes the loop state for the
// others.  Small buckets -- a 4096^2 grid at delta 1 has 1.3 M of them, 13
// vertices each on average -- then cost a few L2 round trips instead of three
// grid barriers.

// Loop state of CTA 0 for the other CTAs (read after the next barrier).
__device__ __forceinline__ void bq_publish(const BqLoop &s, int32_t *ctl) {
  if (threadIdx.x == 0) {
    const int32_t *p = reinterpret_cast<const int32_t *>(&s);
    for (int i = 0; i < kBqLoopInts; ++i) ctl[BQ_PUB + i] = p[i];
  }
}

// CTA 0 alone: steps while they stay small (see above), then publishes the
// loop state.  The control words live in shared memory for the session (every
// count, minimum and decision is then an SM-local access) and go back to
// global memory at its end.  The whole CTA calls it.
template <int LB>
__device__ __forceinline__ void bq_solo(BqLoop &s, const BqArgs &a, BqStep st, int4 *smem, int32_t *red,
                                        int32_t *flag, int32_t *sctl) {
  for (int i = threadIdx.x; i < BQ_STOP; i += blockDim.x) sctl[i] = __ldcg(a.b.ctl + i);
  uint64_t t0 = 0;
  if (threadIdx.x == 0) t0 = globaltimer_ns();
  __syncthreads();
  for (;;) {
    bq_step<LB>(s, a, st, sctl, 0, 1, smem, red);
    __syncthreads();
    if (threadIdx.x == 0)
      *flag = (*(volatile int32_t *)a.err & DEV_ERR_OVERFLOW) != 0 || globaltimer_ns() - t0 > kSoloSliceNs;
    __syncthreads();
    const bool quit = *flag != 0;
    __syncthreads();
    if (quit) break;
    st = bq_decide(s, sctl, a.delta);
    if (st.kind == BQ_DONE || !bq_small(st, a)) break;
  }
  for (int i = threadIdx.x; i < BQ_STOP; i += blockDim.x) a.b.ctl[i] = sctl[i];
  __syncthreads();
  bq_publish(s, a.b.ctl);
}

template <int LB>
__global__ void __launch_bounds__(1024) k_sssp_bq(BqArgs a) {
  extern __shared__ int4 smem[];
  __shared__ int32_t red[33];
  __shared__ int32_t sctl[BQ_STOP];  // counts and minima of a one-CTA session
  BqLoop s{1, 0, 0, 0, 0, bq_clamp((int64_t)a.width0 * a.delta), a.width0, 0, 0, 0};
  int32_t *stop = a.b.ctl + BQ_STOP;
  LoopClock clk;
  clk.start(a.loop_limit_ns);
  // Grid iterations (one barrier each), numbered for the stop word: the clock
  // and a flagged overflow stop every block at the top of the same iteration.
  for (int32_t round = 0;; ++round) {
    if (stopped(stop, round)) break;
    const BqStep st = bq_decide(s, a.b.ctl, a.delta);
    if (st.kind == BQ_DONE) {
      if (s.phase == 0) s.adv++;  // the reference's last advance finds no priority left
      break;
    }
    if (bq_small(st, a)) {
      // CTA 0 starts changing the control words only once every other CTA
      // has taken its decision from them and arrived at the barrier.
      if (blockIdx.x == 0) {
        if (grid_wait_others(a.bar, gridDim.x, a.err, a.timeout_ns))
          bq_solo<LB>(s, a, st, smem, red, red + 32, sctl);
        else
          bq_publish(s, a.b.ctl);
      }
      clk.tick(stop, round, a.err);
      stop_on_overflow(stop, round, a.err);
      if (!grid_barrier(a.bar, gridDim.x, a.err, a.timeout_ns)) break;
      const volatile int32_t *pub = a.b.ctl + BQ_PUB;
      int32_t *p = reinterpret_cast<int32_t *>(&s);
      for (int i = 0; i < kBqLoopInts; ++i) p[i] = pub[i];
      continue;
    }
    bq_step<LB>(s, a, st, a.b.ctl, blockIdx.x, gridDim.x, smem, red);
    clk.tick(stop, round, a.err);
    stop_on_overflow(stop, round, a.err);
    if (!grid_barrier(a.bar, gridDim.x, a.err, a.timeout_ns)) break;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.b.ctl[BQ_STATS] = s.relax;
    a.b.ctl[BQ_STATS + 1] = s.adv;
  }
}

// Control words at the start of a run: n0 sources on the first frontier, no
// minima, empty piles, no refill yet.
__global__ void k_bq_init(int32_t *ctl, int32_t n0) {
  const int32_t i = threadIdx.x;
  if (i >= BQ_CTL_INTS) return;
  int32_t v = 0;
  if (i == BQ_NEAR) v = n0;
  if (i >= BQ_MIN && i < BQ_MIN + 3) v = INT_MAX;
  if (i == BQ_FILL) v = -1;
  ctl[i] = v;
}

gg_status bq_start(const BqBuffers &b, int32_t n0, cudaStream_t st) {
  GG_CUDA(cudaMemsetAsync(b.stamp, 0, sizeof(int32_t) * (size_t)std::max(b.V, 1), st));
  note_launch();
  k_bq_init<<<1, BQ_CTL_INTS, 0, st>>>(b.ctl, n0);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

template <class K, class A, class... More>
static gg_status coop_launch(gg_graph *g, K kernel, int cta, size_t smem, A &a, More &...more) {
  int per_sm = 0;
  if (smem > 48 * 1024)
    GG_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  GG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, cta, smem));
  if (per_sm < 1) return set_error(GG_ERR_UNSUPPORTED, "fused kernel does not fit on an SM");
  const int grid = per_sm * g->sm_count;
  GG_CUDA(cudaMemsetAsync(g->d_bar, 0, sizeof(uint32_t) * 2, g->stream));
  void *args[] = {&a, &more...};
  GG_CUDA(cudaEventRecord(g->ev2, g->stream));
  note_launch();
  GG_CUDA(cudaLaunchCooperativeKernel((const void *)kernel, grid, cta, args, smem, g->stream));
  GG_CUDA(cudaEventRecord(g->ev3, g->stream));
  g->loop_timed = true;
  return GG_OK;
}

static size_t lb_smem(int lb, int cta) {
  if (lb == GG_LB_TWCE) return twce_smem_bytes(cta);
  if (lb == GG_LB_CM) return cm_smem_bytes(cta);
  return 0;
}

static FusedArgs make_args(gg_graph *g, gg_frontier *f, const VData &vd) {
  FusedArgs a{};
  a.g = g->csr.view();
  a.g.nbuckets = 0;
  a.q0 = f->q_in;
  a.q1 = f->q_out;
  a.cnt3 = g->d_misc + 40;
  a.cap = f->cap;
  a.bar = g->d_bar;
  a.err = g->d_err;
  a.timeout_ns = barrier_timeout_ns();
  a.stats = g->d_misc + 44;
  a.vd = vd;
  a.gmin2 = g->d_misc + 46;
  a.stop = g->d_misc + 48;
  a.loop_limit_ns = loop_timeout_ns();
  return a;
}

// Counts start as {n0 (the sources), 0, 0}; both minima slots at INT_MAX.
static gg_status init_counts(gg_graph *g, int32_t n0) {
  int32_t *h = g->h_pinned + 40;
  h[0] = n0;
  h[1] = 0;
  h[2] = 0;
  h[3] = 0;
  h[4] = 0;
  h[5] = 0;
  h[6] = INT_MAX;
  h[7] = INT_MAX;
  h[8] = 0;  // stop flag
  GG_CUDA(cudaMemcpyAsync(g->d_misc + 40, h, sizeof(int32_t) * 9, cudaMemcpyHostToDevice, g->stream));
  return GG_OK;
}

static gg_status read_stats(gg_graph *g, int32_t *iters, int64_t *adv) {
  GG_CUDA(cudaMemcpyAsync(g->h_pinned + 50, g->d_misc + 44, sizeof(int32_t) * 2, cudaMemcpyDeviceToHost,
                          g->stream));
  GG_CUDA(cudaStreamSynchronize(g->stream));
  *iters = g->h_pinned[50];
  if (adv) *adv = g->h_pinned[51];
  return GG_OK;
}

gg_status fused_bfs(gg_graph *g, const gg_schedule *s, int32_t n0, const VData &vd, gg_frontier *f,
                    int32_t *iters, bool *ran) {
  *ran = false;
  if (!fused_supported(s)) return GG_OK;
  GG_TRY(init_counts(g, n0));
  FusedArgs a = make_args(g, f, vd);
  const int cta = s->cta_size;
  const size_t sm = lb_smem(s->load_balancing, cta);
  switch (s->load_balancing) {
    case GG_LB_VERTEX_BASED: GG_TRY(coop_launch(g, k_bfs_fused<GG_LB_VERTEX_BASED>, cta, sm, a)); break;
    case GG_LB_WM: GG_TRY(coop_launch(g, k_bfs_fused<GG_LB_WM>, cta, sm, a)); break;
    case GG_LB_TWCE: GG_TRY(coop_launch(g, k_bfs_fused<GG_LB_TWCE>, cta, sm, a)); break;
    default: GG_TRY(coop_launch(g, k_bfs_fused<GG_LB_CM>, cta, sm, a)); break;
  }
  GG_TRY(read_stats(g, iters, nullptr));
  *ran = true;
  return GG_OK;
}

// ------------------------------------------- direction-optimising BFS loop
// The fused BFS loop with a direction per level, decided on the device at the
// top of the level by every CTA alike (the same statistics in, the same answer
// out): the HybridGPUSchedule rule "s1 while |frontier| <= t*V, else s2"
// (operators.cpp:516-532) when s1 / s2 are one push and one pull schedule, the
// selector network's direction head, or a forced direction (training data).
//
// Frontiers are always the sparse queue.  A push level runs the push schedule's
// LB function over it; a pull level walks every vertex still without a parent
// with an 8-lane group over its in-list and stops at the first in-neighbour
// whose depth is the previous level (depth doubles as the frontier bitmap of
// bfs.cpp's PULL BITMAP schedule; the vertex's own group is the only writer of
// its parent and depth, so no atomics).  Both directions append the vertices
// they reach to the next queue and add their out-degrees to the statistics of
// that frontier (sum, sum of squares, maximum), which the next level's rule or
// network reads: nothing returns to the host between levels.

struct DoArgs {
  DGraph t;                    // in-lists: the transpose, or the CSR itself on a symmetric graph
  unsigned long long *lstat;   // [3][4] statistics of the frontier of each level (rotating):
                               // out-degree sum (u64), sum of squares (double), maximum (u64)
  const float *sel;            // network parameters (DO_SELECTOR)
  int32_t mode;
  int32_t stats;               // gather frontier statistics (the network and the logs read them)
  float threshold;             // DO_RULE: small frontier <=> n <= threshold * V
  int32_t small_pull;          // DO_RULE: the small-frontier schedule is the pull one
  float *feat_log;             // optional: features of level l (training data)
  unsigned long long *time_log;  // optional: start time of level l, end time last
  int32_t max_log;
};

struct DoKernelArgs {
  FusedArgs a;
  DoArgs d;
};

// A CTA's statistics of the next frontier, in shared memory.
struct DoStat {
  unsigned int sum, mx;
  float sq;
};

// Adds the out-degree k of a vertex entering the next frontier: one reduction
// over the threads that reach this point together, one shared atomic each.
__device__ __forceinline__ void do_note(DoStat *s, uint32_t k) {
  cg::coalesced_group g = cg::coalesced_threads();
  const uint32_t sum = cg::reduce(g, k, cg::plus<uint32_t>());
  const float sq = cg::reduce(g, (float)k * (float)k, cg::plus<float>());
  const uint32_t mx = cg::reduce(g, k, cg::greater<uint32_t>());
  if (g.thread_rank() == 0) {
    atomicAdd(&s->sum, sum);
    atomicAdd(&s->sq, sq);
    atomicMax(&s->mx, mx);
  }
}

// bfs.cpp's UDF (UBfs) that also notes the out-degree of each vertex it
// reaches when the loop gathers statistics.
struct UBfsNote {
  static constexpr bool kWeight = false;
  int32_t *parent, *depth;
  const int32_t *off;
  DoStat *stat;  // shared memory; null: no statistics
  int32_t level;
  __device__ __forceinline__ bool filter(int32_t v) const { return vload(parent + v) == -1; }
  __device__ __forceinline__ bool apply(int32_t s, int32_t d, int32_t) const {
    // the degree is loaded alongside the CAS (not after it): one round trip
    const int32_t o0 = stat ? __ldg(off + d) : 0, o1 = stat ? __ldg(off + d + 1) : 0;
    if (!cas(parent + d, -1, s)) return false;
    depth[d] = level;
    if (stat) do_note(stat, (uint32_t)(o1 - o0));
    return true;
  }
};

// Dynamic shared memory: the push strategy's, then (DO_SELECTOR) the staged
// network parameters.
__host__ __device__ __forceinline__ size_t do_lb_smem_aligned(size_t lb_bytes) { return (lb_bytes + 15) & ~size_t(15); }

template <int LB>
__global__ void __launch_bounds__(kBfsDoMaxCta, 4) k_bfs_do(DoKernelArgs ka, uint32_t lb_bytes) {
  extern __shared__ int4 smem[];
  __shared__ DoStat s_stat;
  __shared__ float s_x[16 + 64];
  __shared__ int32_t s_pull;
  __shared__ float s_in[4];    // n, out-degree sum, sum of squares, maximum of this level's frontier
  __shared__ float s_vis[2];   // vertices and out-edges of the frontiers so far (the same in every CTA)
  __shared__ int32_t s_pulls;
  const FusedArgs &a = ka.a;
  const DoArgs &d = ka.d;
  float *wsel = reinterpret_cast<float *>(reinterpret_cast<char *>(smem) + do_lb_smem_aligned(lb_bytes));
  if (d.mode == DO_SELECTOR) selector_stage(d.sel, wsel);
  if (threadIdx.x == 0) {
    s_vis[0] = s_vis[1] = 0.f;
    s_pulls = 0;
  }
  __syncthreads();
  int32_t level = 1;
  LoopClock clk;
  clk.start(a.loop_limit_ns);
  for (;; ++level) {
    // the frontier statistics are loaded together with its size (one round trip)
    unsigned long long r = 0ull;
    if (d.stats && threadIdx.x < 3) r = *(volatile unsigned long long *)(d.lstat + 4 * ((level - 1) % 3) + threadIdx.x);
    const int32_t n = *(volatile int32_t *)(a.cnt3 + (level - 1) % 3);
    if (n == 0 || stopped(a.stop, level)) break;
    const bool logged = d.feat_log && level - 1 <= d.max_log;
    // The level's direction, decided by warp 0 alone (statistics, features,
    // network) and handed to the CTA by one barrier.
    if (threadIdx.x < 32) {
      const int32_t l = threadIdx.x;
      bool pull = d.mode == DO_FORCE_PULL ||
                  (d.mode == DO_RULE && ((float)n <= d.threshold * (float)a.g.V) == (d.small_pull != 0));
      if (d.stats) {
        if (l < 3) s_in[1 + l] = l == 1 ? (float)__longlong_as_double((long long)r) : (float)r;
        if (l == 0) {
          s_in[0] = (float)n;
          s_stat.sum = s_stat.mx = 0u;
          s_stat.sq = 0.f;
        }
        __syncwarp();
        if (l < kSelectorFeatures && (d.mode == DO_SELECTOR || logged))
          s_x[l] = selector_feature(l, s_in[0], s_in[1], s_in[2], s_in[3], s_vis[0], s_vis[1], level - 1,
                                    (float)a.g.V, (float)a.g.E);
        __syncwarp();
        if (d.mode == DO_SELECTOR) pull = selector_pull_warp(wsel, s_x, s_x + 16);
      }
      if (l == 0) {
        s_pull = pull;
        if (blockIdx.x == 0) {
          a.cnt3[(level + 1) % 3] = 0;
          if (d.stats)
            for (int i = 0; i < 4; ++i) d.lstat[4 * ((level + 1) % 3) + i] = 0ull;
          if (logged) {
            if (level - 1 < d.max_log)
              for (int i = 0; i < kSelectorFeatures; ++i) d.feat_log[(level - 1) * kSelectorFeatures + i] = s_x[i];
            d.time_log[level - 1] = globaltimer_ns();
          }
        }
      }
    }
    __syncthreads();
    const bool pull = s_pull != 0;
    DoStat *stat = d.stats ? &s_stat : nullptr;
    const DOut out = sparse_out(a, (level & 1) ? a.q1 : a.q0, level);
    if (!pull) {
      const Enum en{(level & 1) ? a.q0 : a.q1, nullptr, n};
      const EdgeF<UBfsNote, false> f{UBfsNote{a.vd.parent, a.vd.depth, a.g.off, stat, level},
                                     DIn{IN_ALL, nullptr, nullptr}, DIn{IN_ALL, nullptr, nullptr}, true};
      run_lb<LB>(a.g, en, n, f, out, smem, blockIdx.x, gridDim.x);
    } else {
      if (threadIdx.x == 0) ++s_pulls;
      const int32_t lane = threadIdx.x & 31, sub = lane & 7, gbase = lane & ~7;
      const uint32_t gmask = 0xFFu << gbase;
      const int32_t prev = level - 1;
      for (int32_t v = (blockIdx.x * blockDim.x + threadIdx.x) >> 3; v < a.g.V;
           v += (gridDim.x * blockDim.x) >> 3) {
        if (__ldcg(a.vd.parent + v) != -1) continue;
        const int32_t kb = __ldg(d.t.off + v), ke = __ldg(d.t.off + v + 1);
        const int32_t deg = stat && sub == 0 ? __ldg(a.g.off + v + 1) - __ldg(a.g.off + v) : 0;
        int32_t hit = -1;
        for (int32_t k0 = kb; k0 < ke; k0 += 8) {
          int32_t u = -1;
          if (k0 + sub < ke) {
            u = __ldg(d.t.dst + k0 + sub);
            if (__ldcg(a.vd.depth + u) != prev) u = -1;
          }
          const uint32_t bits = (__ballot_sync(gmask, u >= 0) >> gbase) & 0xFFu;
          if (bits) {
            hit = __shfl_sync(gmask, u, gbase + __ffs(bits) - 1);
            break;
          }
        }
        if (hit >= 0 && sub == 0) {
          a.vd.parent[v] = hit;
          a.vd.depth[v] = level;
          out.sparse(v);
          if (stat) do_note(stat, (uint32_t)deg);
        }
      }
    }
    __syncthreads();
    if (d.stats && threadIdx.x == 0) {
      s_vis[0] = fminf((float)a.g.V, s_vis[0] + s_in[0]);
      s_vis[1] = fminf((float)a.g.E, s_vis[1] + s_in[1]);
      if (s_stat.sum | s_stat.mx) {
        unsigned long long *nx = d.lstat + 4 * (level % 3);
        atomicAdd(nx, (unsigned long long)s_stat.sum);
        atomicAdd(reinterpret_cast<double *>(nx + 1), (double)s_stat.sq);
        atomicMax(nx + 2, (unsigned long long)s_stat.mx);
      }
    }
    clk.tick(a.stop, level, a.err);
    if (!grid_barrier(a.bar, gridDim.x, a.err, a.timeout_ns)) break;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.stats[0] = level - 1;
    a.stats[1] = s_pulls;
    if (d.time_log && level - 1 <= d.max_log) d.time_log[level - 1] = globaltimer_ns();
  }
}

// Statistics of the first frontier (the n0 sources on the queue); the other
// two slots cleared.
__global__ void k_bfs_do_seed(const int32_t *__restrict__ q, int32_t n0, const int32_t *__restrict__ off,
                              unsigned long long *lstat) {
  __shared__ unsigned long long s[2];
  __shared__ double sq;
  if (threadIdx.x < 2) s[threadIdx.x] = 0ull;
  if (threadIdx.x == 0) sq = 0.0;
  __syncthreads();
  for (int32_t i = threadIdx.x; i < n0; i += blockDim.x) {
    const int32_t v = q[i];
    const unsigned long long k = (unsigned long long)(off[v + 1] - off[v]);
    atomicAdd(s, k);
    atomicAdd(&sq, (double)k * (double)k);
    atomicMax(s + 1, k);
  }
  __syncthreads();
  if (threadIdx.x < 12) {
    unsigned long long v = 0ull;
    if (threadIdx.x == 0) v = s[0];
    if (threadIdx.x == 1) v = (unsigned long long)__double_as_longlong(sq);
    if (threadIdx.x == 2) v = s[1];
    lstat[threadIdx.x] = v;
  }
}

gg_status fused_bfs_do(gg_graph *g, const BfsDoPlan &p, int32_t n0, const VData &vd, gg_frontier *f,
                       int32_t *iters, int32_t *pulls) {
  const gg_schedule *s = p.push;
  if (!s || !fused_supported(s) || s->cta_size > kBfsDoMaxCta)
    return set_error(GG_ERR_UNSUPPORTED, "push schedule cannot be fused (or CTA size above %d)", kBfsDoMaxCta);
  GG_CHECK_ARG(vd.parent && vd.depth, "the direction-optimising loop needs parent and depth");
  GG_CHECK_ARG(p.mode != DO_SELECTOR || p.sel, "no selector");
  GG_TRY(ensure_transpose(g));
  const GraphStore *t = g->csc ? g->csc.get() : &g->csr;
  void *ls = nullptr;
  GG_TRY(scratch_get_app(g, 7, sizeof(unsigned long long) * 12, &ls));
  GG_TRY(init_counts(g, n0));
  note_launch();
  k_bfs_do_seed<<<1, 256, 0, g->stream>>>(f->q_in, n0, g->csr.off, static_cast<unsigned long long *>(ls));
  GG_CUDA(cudaGetLastError());
  DoKernelArgs ka{};
  ka.a = make_args(g, f, vd);
  ka.d.t = t->view();
  ka.d.t.nbuckets = 0;
  ka.d.lstat = static_cast<unsigned long long *>(ls);
  ka.d.sel = p.mode == DO_SELECTOR ? selector_params(p.sel) : nullptr;
  ka.d.mode = p.mode;
  ka.d.stats = p.mode == DO_SELECTOR || p.feat_log;
  ka.d.threshold = p.threshold;
  ka.d.small_pull = p.small_pull;
  ka.d.feat_log = p.feat_log;
  ka.d.time_log = p.time_log;
  ka.d.max_log = p.max_log;
  const int cta = s->cta_size;
  uint32_t lbb = (uint32_t)lb_smem(s->load_balancing, cta);
  const size_t sm = p.mode == DO_SELECTOR ? do_lb_smem_aligned(lbb) + sizeof(float) * kSelectorParams : lbb;
  switch (s->load_balancing) {
    case GG_LB_VERTEX_BASED: GG_TRY(coop_launch(g, k_bfs_do<GG_LB_VERTEX_BASED>, cta, sm, ka, lbb)); break;
    case GG_LB_WM: GG_TRY(coop_launch(g, k_bfs_do<GG_LB_WM>, cta, sm, ka, lbb)); break;
    case GG_LB_TWCE: GG_TRY(coop_launch(g, k_bfs_do<GG_LB_TWCE>, cta, sm, ka, lbb)); break;
    default: GG_TRY(coop_launch(g, k_bfs_do<GG_LB_CM>, cta, sm, ka, lbb)); break;
  }
  int64_t np = 0;
  GG_TRY(read_stats(g, iters, &np));
  *pulls = (int32_t)np;
  return GG_OK;
}

// Largest relax step the SSSP loop runs on one CTA, in frontier entries per
// thread of the CTA (GG_BQ_SOLO_PER_THREAD overrides; 0 turns the one-CTA
// mode off).  Pile steps take 8 times as many entries: one load and a
// compare each.
static int32_t bq_solo_per_thread() {
  static const long env = [] {
    const char *e = getenv("GG_BQ_SOLO_PER_THREAD");
    return e ? atol(e) : -1L;
  }();
  return env >= 0 ? (int32_t)env : 4;
}

static BqArgs bq_args(gg_graph *g, gg_frontier *f, const BqBuffers &b, int32_t *dist, int32_t delta, int cta) {
  BqArgs a{};
  a.g = g->csr.view();
  a.g.nbuckets = 0;
  a.q0 = f->q_in;
  a.q1 = f->q_out;
  a.qcap = f->cap;
  a.dist = dist;
  a.b = b;
  a.bar = g->d_bar;
  a.err = g->d_err;
  a.timeout_ns = barrier_timeout_ns();
  a.loop_limit_ns = loop_timeout_ns();
  a.delta = delta;
  a.solo_max = bq_solo_per_thread() * cta;
  a.solo_pile_max = 8 * a.solo_max;
  a.fill_target = 1024;
  a.width0 = 16;
  return a;
}

gg_status fused_sssp(gg_graph *g, const gg_schedule *s, int32_t n0, int32_t delta, const VData &vd,
                     gg_pq *pq, int32_t *iters, int64_t *advances, bool *ran) {
  *ran = false;
  if (!fused_supported(s)) return GG_OK;
  const int cta = s->cta_size;
  GG_TRY(bq_start(pq->bq, n0, g->stream));
  BqArgs a = bq_args(g, pq->frontier, pq->bq, vd.dist, delta, cta);
  const size_t sm = lb_smem(s->load_balancing, cta);
  switch (s->load_balancing) {
    case GG_LB_VERTEX_BASED: GG_TRY(coop_launch(g, k_sssp_bq<GG_LB_VERTEX_BASED>, cta, sm, a)); break;
    case GG_LB_WM: GG_TRY(coop_launch(g, k_sssp_bq<GG_LB_WM>, cta, sm, a)); break;
    case GG_LB_TWCE: GG_TRY(coop_launch(g, k_sssp_bq<GG_LB_TWCE>, cta, sm, a)); break;
    default: GG_TRY(coop_launch(g, k_sssp_bq<GG_LB_CM>, cta, sm, a)); break;
  }
  GG_CUDA(cudaMemcpyAsync(g->h_pinned + 50, pq->bq.ctl + BQ_STATS, sizeof(int32_t) * 2, cudaMemcpyDeviceToHost,
                          g->stream));
  GG_CUDA(cudaStreamSynchronize(g->stream));
  *iters = g->h_pinned[50];
  *advances = g->h_pinned[51];
  *ran = true;
  return GG_OK;
}

// ------------------------------------------------- capturable multi-source run
// Reset of the vertex data, then the sources (device array) seeded into the
// frontier queue and the loop's counters set, all on the device, so the whole
// run is stream-ordered and can be captured into a CUDA graph.
__global__ void k_multi_reset(VData vd, int32_t sssp, int32_t V) {
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    if (sssp) {
      vd.dist[v] = INT_MAX;
    } else {
      vd.parent[v] = -1;
      vd.depth[v] = -1;
    }
  }
}

__global__ void k_multi_seed(VData vd, int32_t sssp, const int32_t *__restrict__ srcs, int32_t n, int32_t *q,
                             int32_t *cnt3, int32_t *stats, int32_t *gmin2, int32_t *stop) {
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int32_t s = srcs[i];
    if (sssp) {
      vd.dist[s] = 0;
    } else {
      vd.parent[s] = s;
      vd.depth[s] = 0;
    }
    q[i] = s;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    cnt3[0] = n;
    cnt3[1] = 0;
    cnt3[2] = 0;
    stats[0] = 0;
    stats[1] = 0;
    gmin2[0] = INT_MAX;
    gmin2[1] = INT_MAX;
    *stop = 0;
  }
}

gg_status fused_multi_enqueue(gg_graph *g, cudaStream_t st, bool sssp, const int32_t *dsrc, int32_t n,
                              int32_t delta, int32_t *parent, int32_t *out, const BqBuffers *bq,
                              const int32_t **stats) {
  gg_frontier *f = g->app_frontier;
  if (!f) return set_error(GG_ERR_STATE, "multi-source run: the graph's frontier is not created");
  if (sssp && !bq) return set_error(GG_ERR_STATE, "multi-source SSSP needs its bucket-queue buffers");
  VData vd{};
  if (sssp) {
    vd.dist = out;
  } else {
    vd.parent = parent;
    vd.depth = out;
  }
  vd.src = -1;
  FusedArgs a = make_args(g, f, vd);
  a.delta = delta;
  const int cta = 512;
  const size_t smem = twce_smem_bytes(cta);
  const void *kernel = sssp ? (const void *)k_sssp_bq<GG_LB_TWCE> : (const void *)k_bfs_fused<GG_LB_TWCE>;
  int per_sm = 0;
  GG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, cta, smem));
  if (per_sm < 1) return set_error(GG_ERR_UNSUPPORTED, "fused kernel does not fit on an SM");
  note_launch();
  k_multi_reset<<<g->sm_count * 8, 256, 0, st>>>(vd, sssp, g->csr.V);
  note_launch();
  k_multi_seed<<<std::max(1, std::min(ceil_div(n, 256), g->sm_count)), 256, 0, st>>>(
      vd, sssp, dsrc, n, a.q0, a.cnt3, a.stats, a.gmin2, a.stop);
  GG_CUDA(cudaMemsetAsync(g->d_bar, 0, sizeof(uint32_t) * 2, st));
  if (sssp) {
    GG_TRY(bq_start(*bq, n, st));
    BqArgs b = bq_args(g, f, *bq, out, delta, cta);
    void *args[] = {&b};
    note_launch();
    GG_CUDA(cudaLaunchCooperativeKernel(kernel, per_sm * g->sm_count, cta, args, smem, st));
    if (stats) *stats = bq->ctl + BQ_STATS;
  } else {
    void *args[] = {&a};
    note_launch();
    GG_CUDA(cudaLaunchCooperativeKernel(kernel, per_sm * g->sm_count, cta, args, smem, st));
    if (stats) *stats = a.stats;
  }
  return GG_OK;
}

// A barrier that waits for one block more than were launched: it can only end
// by its time limit.
__global__ void k_barrier_never(uint32_t *bar, int32_t *err, uint64_t timeout_ns) {
  grid_barrier(bar, gridDim.x + 1, err, timeout_ns);
}

}  // namespace gg

using namespace gg;

extern "C" gg_status gg_debug_barrier_timeout(int32_t timeout_us) {
  GG_CHECK_ARG(timeout_us > 0 && timeout_us <= 10 * 1000 * 1000, "timeout must be in (0, 10 s]");
  uint32_t *bar = nullptr;
  int32_t *err = nullptr;
  GG_CUDA(cudaMalloc(&bar, sizeof(uint32_t) * 2));
  GG_CUDA(cudaMalloc(&err, sizeof(int32_t)));
  GG_CUDA(cudaMemset(bar, 0, sizeof(uint32_t) * 2));
  GG_CUDA(cudaMemset(err, 0, sizeof(int32_t)));
  { gg::note_launch(); k_barrier_never<<<2, 32>>>(bar, err, (uint64_t)timeout_us * 1000ull); }
  cudaError_t le = cudaGetLastError();
  cudaError_t se = cudaDeviceSynchronize();
  int32_t h = 0;
  cudaMemcpy(&h, err, sizeof(int32_t), cudaMemcpyDeviceToHost);
  cudaFree(bar);
  cudaFree(err);
  if (le != cudaSuccess || se != cudaSuccess)
    return set_error(GG_ERR_CUDA, "barrier probe launch failed: %s",
                     cudaGetErrorString(le != cudaSuccess ? le : se));
  if (h & DEV_ERR_TIMEOUT) return set_error(GG_ERR_TIMEOUT, "grid barrier wait timed out as designed");
  return GG_OK;
}
