// The delta-stepping step machine over the bucket queue of bucket_queue.cuh,
// run by the persistent single-source loop (fused.cu, k_sssp_bq).
#pragma once

#include "bucket_queue.cuh"
#include "engine.h"
#include "lb.cuh"
#include "udf.cuh"

namespace gg {

// Runs one LB strategy over the n enumerated vertices; CTA `rank` of `nparts`
// takes every nparts-th virtual CTA (nparts = 1: one CTA does all of it).
template <int LB, class F>
__device__ __forceinline__ void run_lb(const DGraph &g, const Enum &en, int32_t n, const F &f,
                                       const DOut &out, int4 *smem, int32_t rank, int32_t nparts) {
  if (LB == GG_LB_VERTEX_BASED) {
    const int32_t nv = ceil_div(n, blockDim.x);
    for (int32_t v = rank; v < nv; v += nparts) lb_vertex(g, en, n, f, out, v);
  } else if (LB == GG_LB_WM) {
    const int32_t nv = ceil_div(n, blockDim.x >> 5);
    for (int32_t v = rank; v < nv; v += nparts) lb_wm(g, en, n, f, out, v);
  } else if (LB == GG_LB_TWCE) {
    const int32_t nv = ceil_div(n, blockDim.x / kStage1);
    for (int32_t v = rank; v < nv; v += nparts)
      lb_twce<F, true>(g, en, n, f, out, v, *reinterpret_cast<TwceSmem *>(smem));
  } else {
    const int32_t nv = ceil_div(n, blockDim.x);
    for (int32_t v = rank; v < nv; v += nparts)
      lb_cm(g, en, n, f, out, v, *reinterpret_cast<CmSmem *>(smem));
  }
}

// ------------------------------------------------------ delta-stepping SSSP
// The sssp.cpp loop (apps/sssp.cpp:47-52) over the bucket queue of
// bucket_queue.cuh, as a sequence of steps, each one of
//   relax     the frontier with cutoff cur+delta (improvements below it queue
//             the vertex, the others park it on a far pile),
//   lo-min    exact minimum of the low pile's live entries,
//   lo-split  window entries to the frontier, the rest to the next low pile
//             (a window reaching past the horizon splits the high pile too),
//   hi-min / hi-split  the same over the high pile when the low pile holds
//             nothing live (a refill, which also sets the next horizon).
// Between steps the CTAs that run them synchronise (a grid barrier, or
// __syncthreads when one CTA runs them).  Frontier counts and minima rotate
// through three slots: a step clears the slot two steps ahead, whose readers
// finished before the previous synchronisation.
enum : int32_t { BQ_RELAX = 0, BQ_LOMIN = 1, BQ_LOSPLIT = 2, BQ_HIMIN = 3, BQ_HISPLIT = 4, BQ_DONE = 5 };
constexpr uint64_t kSoloSliceNs = 1000000;

struct BqArgs {
  DGraph g;
  int32_t *q0, *q1;  // frontier queues
  int64_t qcap;
  int32_t *dist;
  BqBuffers b;       // stamps, piles, control words
  uint32_t *bar;
  int32_t *err;
  uint64_t timeout_ns, loop_limit_ns;
  int32_t delta;
  int32_t solo_max;     // largest relax step (frontier entries) CTA 0 runs alone
  int32_t solo_pile_max;  // largest pile step (pile entries) CTA 0 runs alone
  int32_t fill_target;  // low-pile entries a refill aims for
  int32_t width0;       // first horizon width, in buckets
};

// Loop state, the same in every CTA: every decision is taken from control
// words read after a barrier.
struct BqLoop {
  int32_t it;     // step number (slot rotation)
  int32_t in;     // frontier queue read by this step
  int32_t cur;    // window start
  int32_t g, gh;  // low / high pile generations
  int32_t hz;     // horizon
  int32_t k;      // horizon width in buckets
  int32_t phase;  // 0: normal, 1: after a lo-min, 2: after a hi-min
  int32_t relax, adv;
};
constexpr int kBqLoopInts = 10;
static_assert(sizeof(BqLoop) == kBqLoopInts * sizeof(int32_t), "BqLoop is published as ints");

struct BqStep {
  int32_t kind, work, m;
};

// Small enough for CTA 0 alone: frontier entries of a relax, pile entries of
// the other steps (one load and a compare each).
__device__ __forceinline__ bool bq_small(const BqStep &st, const BqArgs &a) {
  return st.work <= (st.kind == BQ_RELAX ? a.solo_max : a.solo_pile_max);
}

// The next step (pure: every CTA computes the same one).
__device__ __forceinline__ BqStep bq_decide(const BqLoop &s, const int32_t *ctl, int32_t delta) {
  const volatile int32_t *c = ctl;
  const int32_t prev = (s.it + 2) % 3;
  if (s.phase == 1) {
    const int32_t m = c[BQ_MIN + prev];
    if (m != INT_MAX) {
      const bool cross = bq_clamp((int64_t)m + delta) > s.hz;  // the window reaches the high pile
      return BqStep{BQ_LOSPLIT, c[BQ_LO + (s.g & 1)] + (cross ? c[BQ_HI + (s.gh & 1)] : 0), m};
    }
    const int32_t nh = c[BQ_HI + (s.gh & 1)];
    return nh > 0 ? BqStep{BQ_HIMIN, nh, 0} : BqStep{BQ_DONE, 0, 0};
  }
  if (s.phase == 2) {
    const int32_t m = c[BQ_MIN + prev];
    return m != INT_MAX ? BqStep{BQ_HISPLIT, c[BQ_HI + (s.gh & 1)], m} : BqStep{BQ_DONE, 0, 0};
  }
  const int32_t n = c[BQ_NEAR + prev];
  if (n > 0) return BqStep{BQ_RELAX, n, 0};
  const int32_t nl = c[BQ_LO + (s.g & 1)];
  if (nl > 0) return BqStep{BQ_LOMIN, nl, 0};
  const int32_t nh = c[BQ_HI + (s.gh & 1)];
  return nh > 0 ? BqStep{BQ_HIMIN, nh, 0} : BqStep{BQ_DONE, 0, 0};
}

// One step, CTA `rank` of `nparts` taking its share.
// `ctl` holds the control words: global memory in grid mode, CTA 0's shared
// copy in a one-CTA session.
template <int LB>
__device__ __forceinline__ void bq_step(BqLoop &s, const BqArgs &a, const BqStep &st, int32_t *ctl,
                                        int32_t rank, int32_t nparts, int4 *smem, int32_t *red) {
  const bool lead = rank == 0 && threadIdx.x == 0;
  if (lead) {
    ctl[BQ_NEAR + (s.it + 1) % 3] = 0;
    ctl[BQ_MIN + (s.it + 1) % 3] = INT_MAX;
  }
  const int32_t U = bq_clamp((int64_t)s.cur + a.delta);  // cutoff of the current window
  int32_t *qin = s.in ? a.q1 : a.q0, *qout = s.in ? a.q0 : a.q1;
  DOut front{};
  front.mode = OUT_SPARSE;
  front.q = qout;
  front.cnt = ctl + BQ_NEAR + s.it % 3;
  front.cap = a.qcap;
  front.err = a.err;
  const int32_t lo_next = (s.g + 1) & 1;
  switch (st.kind) {
    case BQ_RELAX: {
      const DFar far{a.b.stamp, a.b.lo[s.g & 1], ctl + BQ_LO + (s.g & 1), a.b.hi[s.gh & 1],
                     ctl + BQ_HI + (s.gh & 1), bq_lo_tag(s.g), bq_hi_tag(s.gh), s.hz, a.b.V, a.err};
      const EdgeF<USssp, false> f{USssp{a.dist, U, far}, DIn{IN_ALL, nullptr, nullptr},
                                  DIn{IN_ALL, nullptr, nullptr}, false};
      const int32_t n = (int64_t)st.work > a.qcap ? (int32_t)a.qcap : st.work;  // past qcap only after a flagged overflow
      run_lb<LB>(a.g, Enum{qin, nullptr, n}, n, f, front, smem, rank, nparts);
      s.in ^= 1;
      s.relax++;
      s.phase = 0;
      break;
    }
    case BQ_LOMIN:
      if (s.phase == 0) s.adv++;
      if (lead) {
        ctl[BQ_LO + lo_next] = 0;
        ctl[BQ_HI + ((s.gh + 1) & 1)] = 0;
        ctl[BQ_FILL + ((s.gh + 1) & 1)] = 0;
      }
      bq_pile_min(a.b.lo[s.g & 1], min(st.work, a.b.V), a.dist, U, ctl + BQ_MIN + s.it % 3, rank, nparts, red);
      s.phase = 1;
      break;
    case BQ_LOSPLIT: {
      const int32_t win = bq_clamp((int64_t)st.m + a.delta);
      const int32_t n_lo = min(*(volatile int32_t *)(ctl + BQ_LO + (s.g & 1)), a.b.V);
      if (win <= s.hz) {
        const BqSplitOut o{a.b.stamp, a.b.lo[lo_next], ctl + BQ_LO + lo_next, bq_lo_tag(s.g + 1),
                           nullptr, nullptr, 0, INT_MAX, nullptr, a.b.V, false};
        bq_pile_split(a.b.lo[s.g & 1], n_lo, a.dist, U, win, front, o, a.err, rank, nparts);
      } else {
        // the window reaches past the horizon: split both piles under a new one
        const int32_t hi_next = (s.gh + 1) & 1;
        s.k = bq_adapt_width(s.k, *(volatile int32_t *)(ctl + BQ_FILL + (s.gh & 1)), a.fill_target);
        const int32_t hz = bq_clamp((int64_t)st.m + (int64_t)s.k * a.delta);
        BqSplitOut o{a.b.stamp, a.b.lo[lo_next], ctl + BQ_LO + lo_next, bq_lo_tag(s.g + 1),
                     a.b.hi[hi_next], ctl + BQ_HI + hi_next, bq_hi_tag(s.gh + 1), hz, nullptr, a.b.V, true};
        bq_pile_split(a.b.lo[s.g & 1], n_lo, a.dist, U, win, front, o, a.err, rank, nparts);
        o.fill = ctl + BQ_FILL + hi_next;
        bq_pile_split(a.b.hi[s.gh & 1], min(*(volatile int32_t *)(ctl + BQ_HI + (s.gh & 1)), a.b.V), a.dist, U,
                      win, front, o, a.err, rank, nparts);
        s.hz = hz;
        s.gh++;
      }
      s.cur = st.m;
      s.g++;
      s.in ^= 1;
      s.phase = 0;
      break;
    }
    case BQ_HIMIN: {
      if (s.phase == 0) s.adv++;
      const int32_t hi_next = (s.gh + 1) & 1;
      if (lead) {
        ctl[BQ_LO + lo_next] = 0;
        ctl[BQ_HI + hi_next] = 0;
        ctl[BQ_FILL + hi_next] = 0;
      }
      bq_pile_min(a.b.hi[s.gh & 1], min(st.work, a.b.V), a.dist, U, ctl + BQ_MIN + s.it % 3, rank, nparts, red);
      s.phase = 2;
      break;
    }
    case BQ_HISPLIT: {
      const int32_t hi_next = (s.gh + 1) & 1;
      s.k = bq_adapt_width(s.k, *(volatile int32_t *)(ctl + BQ_FILL + (s.gh & 1)), a.fill_target);
      const int32_t hz = bq_clamp((int64_t)st.m + (int64_t)s.k * a.delta);
      const BqSplitOut o{a.b.stamp, a.b.lo[lo_next], ctl + BQ_LO + lo_next, bq_lo_tag(s.g + 1),
                         a.b.hi[hi_next], ctl + BQ_HI + hi_next, bq_hi_tag(s.gh + 1), hz,
                         ctl + BQ_FILL + hi_next, a.b.V, false};
      bq_pile_split(a.b.hi[s.gh & 1], min(st.work, a.b.V), a.dist, U, bq_clamp((int64_t)st.m + a.delta), front,
                    o, a.err, rank, nparts);
      s.cur = st.m;
      s.hz = hz;
      s.g++;
      s.gh++;
      s.in ^= 1;
      s.phase = 0;
      break;
    }
    default:
      break;
  }
  s.it++;
}

}  // namespace gg
