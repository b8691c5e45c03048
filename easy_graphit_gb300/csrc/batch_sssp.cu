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
// the smallest far priority recorded for s since its last advance, and far
// entries inside [cur[s], cur[s]+delta) move to the near frontier.  Every vertex
// whose priority is at or above the window was last improved at or above a
// cutoff, so the far list holds exactly the candidates the reference finds by
// scanning all V.  The recorded minimum (relaxes fold their far values into a
// per-CTA minimum, the advance folds in what it keeps) is never above the
// smallest pending far priority and never below the old window; it equals the
// reference's next window (gpu_priority_queue.h: min P[v] >= cur+delta) unless
// that vertex has since been settled through a lighter path, and then the
// window only starts lower -- at worst it is empty and the next advance starts
// from exact minima.  Distances are the same either way.
//
// A relaxation registers (near or far) when its value is below the distance
// read before its atomicMin, which is issued without waiting for the old value:
// a concurrent smaller write can only make the registration redundant, never
// lose one.  The first thread to set a near bit of v in an iteration (its
// atomicOr on the near mask returns 0) queues v.
//
// A relax over a large queue (at least V/scan_div entries) does not decide
// who queues: it ORs the near and far masks without reading them back, the
// publish phase then queues every vertex with a near mask by one coalesced
// scan over all V, and the next advance scans all V for far masks (rebuilding
// the far list).  Small relaxes keep the queue-on-first-bit path, so graphs
// with thousands of small iterations never pay a V-sized scan per iteration.
//
// Iteration: relax | barrier | publish near masks, collect the active sources |
// barrier | [advance: move / keep far entries | barrier].
#include <cooperative_groups/scan.h>

#include <algorithm>

#include "batch.h"

namespace gg {

constexpr int32_t kLanes = kBsLanes;
// Queue entries active for at most S.ep_max sources are relaxed edge-parallel
// (lanes = edges); busier ones source-parallel (lanes = sources).  S.chunk
// (edges per queue entry) and S.ep_max come from the graph's batch tuning.

constexpr uint32_t kFull = 0xffffffffu;

// 16-byte asynchronous copy global -> shared (L2 only), and its wait.
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)),
               "l"(__cvta_generic_to_global(gmem))
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Fire-and-forget global reductions: the relax never uses the old value, and
// plain atomics on generic pointers compile to value-returning atomics.
__device__ __forceinline__ void red_min(int32_t *p, int32_t v) {
  asm volatile("red.relaxed.gpu.global.min.s32 [%0], %1;" ::"l"(__cvta_generic_to_global(p)), "r"(v) : "memory");
}
__device__ __forceinline__ void red_or(uint32_t *p, uint32_t v) {
  asm volatile("red.relaxed.gpu.global.or.b32 [%0], %1;" ::"l"(__cvta_generic_to_global(p)), "r"(v) : "memory");
}
constexpr int32_t kBsScanDiv = 64;  // relaxes over >= V/64 entries mark masks without queueing

// Queues v as ceil(deg/chunk) entries.  The threads of a warp that enqueue
// together reserve their entries with one atomic (coalesced-group scan).
__device__ __forceinline__ void bs_enqueue(const BsState &S, int64_t *q, int32_t *qcnt, int32_t v) {
  const int32_t deg = S.off[v + 1] - S.off[v];
  const int32_t nch = max(1, ceil_div(deg, S.chunk));
  cg::coalesced_group grp = cg::coalesced_threads();
  const int32_t excl = cg::exclusive_scan(grp, nch);
  const uint32_t last = grp.size() - 1;
  int32_t base = 0;
  if (grp.thread_rank() == last) base = atomicAdd(qcnt, excl + nch);
  const int32_t pos = grp.shfl(base, last) + excl;
  if ((int64_t)pos + nch > S.qcap) {
    atomicOr(S.err, DEV_ERR_OVERFLOW);
    return;
  }
  for (int32_t c = 0; c < nch; ++c) q[pos + c] = ((int64_t)v << 32) | (uint32_t)c;
}

// Entries per warp step: 32 when the list is long, fewer when it is short.
__device__ __forceinline__ int32_t bs_batch(int64_t n, int64_t nwarps) {
  const int64_t per = (n + nwarps - 1) / nwarps;
  return (int32_t)(per < 1 ? 1 : (per > 32 ? 32 : per));
}

// Relax-time queueing: one entry (chunk 0) per vertex, without the degree
// lookup; the publish phase adds the further chunks of high-degree vertices.
__device__ __forceinline__ void bs_enqueue_first(const BsState &S, int64_t *q, int32_t *qcnt, int32_t v) {
  const int32_t pos = agg_inc(qcnt);
  if (pos < S.qcap)
    q[pos] = (int64_t)v << 32;
  else
    atomicOr(S.err, DEV_ERR_OVERFLOW);
}

// Appends of a warp to a global list (queue or far list), collected in a
// shared-memory buffer of kStage entries and written out with one atomicAdd
// on the list's counter per kStage entries instead of one per warp step: the
// scans over all V append from every warp, and one counter taking an atomic
// from every warp step serialises.  The whole warp calls push() and flush().
constexpr int32_t kStage = 128;

template <typename T>
struct WarpStage {
  T *buf;     // kStage entries of this warp (shared memory)
  T *list;    // the global list
  int32_t *cnt;
  int64_t cap;
  int32_t n;  // staged entries (warp-uniform)

  __device__ __forceinline__ void flush(int32_t *err) {
    if (n == 0) return;
    const int32_t lane = threadIdx.x & 31;
    int32_t base = 0;
    if (lane == 0) base = atomicAdd(cnt, n);
    base = __shfl_sync(kFull, base, 0);
    for (int32_t i = lane; i < n; i += 32) {
      const int64_t pos = (int64_t)base + i;
      if (pos < cap)
        list[pos] = buf[i];
      else
        atomicOr(err, DEV_ERR_OVERFLOW);
    }
    __syncwarp();
    n = 0;
  }
  __device__ __forceinline__ void push(bool app, T val, int32_t *err) {
    const uint32_t am = __ballot_sync(kFull, app);
    if (!am) return;
    const int32_t k = __popc(am);
    if (n + k > kStage) flush(err);
    const int32_t lane = threadIdx.x & 31;
    if (app) buf[n + __popc(am & ((1u << lane) - 1u))] = val;
    __syncwarp();
    n += k;
  }
};

// Final flush of every warp's staged entries with one atomicAdd per CTA: the
// warps' counts go through shared memory (s_cnt: one int per warp + 1) and
// thread 0 reserves the CTA's total.  The whole CTA calls it together.
template <typename T>
__device__ __forceinline__ void cta_flush(WarpStage<T> &st, int32_t *s_cnt, int32_t *err) {
  const int32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) s_cnt[w] = st.n;
  __syncthreads();
  if (threadIdx.x == 0) {
    int32_t tot = 0;
    for (int32_t i = 0; i < nw; ++i) {
      const int32_t c = s_cnt[i];
      s_cnt[i] = tot;
      tot += c;
    }
    s_cnt[nw] = tot ? atomicAdd(st.cnt, tot) : 0;
  }
  __syncthreads();
  const int64_t base = (int64_t)s_cnt[nw] + s_cnt[w];
  for (int32_t i = lane; i < st.n; i += 32) {
    if (base + i < st.cap)
      st.list[base + i] = st.buf[i];
    else
      atomicOr(err, DEV_ERR_OVERFLOW);
  }
  __syncwarp();
  st.n = 0;
  __syncthreads();  // s_cnt is reused by the next flush
}

// Advances of at most kAdvFew sources walk the far entries with lane = entry:
// lane l loads the distances of its entry for every advancing source with a
// far bit there, all at once (instead of 4 entries at a time, lane = source).
constexpr int32_t kAdvFew = 8;

// ds[k] = dist[v][k-th source of A] where fa has that source's bit, else INT_MAX.
__device__ __forceinline__ void bs_far_loads(const BsState &S, int32_t v, uint32_t fa, uint32_t A, int32_t nA,
                                             int32_t (&ds)[kAdvFew]) {
#pragma unroll
  for (int32_t k = 0; k < kAdvFew; ++k) {
    const int32_t s = A ? __ffs(A) - 1 : 0;
    A &= A - 1;
    ds[k] = (k < nA && ((fa >> s) & 1u)) ? __ldcg(S.dist + (int64_t)v * kLanes + s) : INT_MAX;
  }
}

__device__ __forceinline__ void bs_far_push(const BsState &S, int p, int32_t v) {
  const int32_t pos = agg_inc(S.cnt + 3 + p);
  if (pos < S.V)
    S.fl[p][pos] = v;
  else
    atomicOr(S.err, DEV_ERR_OVERFLOW);
}

// Relax of queue entries by warps, which take batches of up to 32 entries from
// a shared counter (guided: batches shrink as the queue drains, so the phase
// ends evenly): lane l loads entry l's vertex, frontier mask and edge range, so
// the per-entry load chains overlap.  Entries active for at most ep_max sources have their edges
// flattened over the lanes (lane = edge, looping over the entry's sources);
// the others run one at a time with lane = source.
__device__ __forceinline__ void bs_relax(const BsState &S, int64_t n_main, int64_t n, const int64_t *qi,
                                         const int64_t *hqi, int64_t *qo,
                                         int32_t *qcnt_out, int32_t cut, const int32_t *s_cut, int p,
                                         int32_t it, int32_t *wctr, int64_t nwarps, bool scan, int32_t *dl,
                                         int32_t *s_fmin) {
  const int32_t lane = threadIdx.x & 31;
  // A queue of at most two entries per warp is split statically: no warp
  // touches the shared counter, whose atomics serialise when thousands of
  // warps each take one entry (high-diameter graphs run 10^5 such relaxes).
  const bool fixed = n <= 2 * nwarps;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  for (bool first = true;; first = false) {
    int32_t e0 = 0, B = 1;
    if (fixed) {
      if (!first) break;
      B = (int32_t)((n + nwarps - 1) / nwarps);
      e0 = (int32_t)(gw * B < n ? gw * B : n);
    } else {
      if (lane == 0) {
        const int64_t left = n - *(volatile int32_t *)wctr;
        B = bs_batch(left > 0 ? left / 2 : 1, nwarps);
        e0 = atomicAdd(wctr, B);
      }
      e0 = __shfl_sync(kFull, e0, 0);
      B = __shfl_sync(kFull, B, 0);
    }
    if (e0 >= n) break;
    const int64_t e = (int64_t)e0 + lane;
    int32_t u = 0, b = 0, cnt = 0;
    uint32_t m = 0;
    if (lane < B && e < n) {
      const int64_t item = e < n_main ? __ldcg(qi + e) : __ldcg(hqi + (e - n_main));
      u = (int32_t)(item >> 32);
      const int32_t c = (int32_t)(item & 0xffffffff);
      m = __ldcg(S.fr + u);
      if (m) {
        const int32_t o1 = __ldg(S.off + u + 1);
        b = __ldg(S.off + u) + c * S.chunk;
        cnt = max(0, min(b + S.chunk, o1) - b);
      }
    }
    const bool sparse = __popc(m) <= S.ep_max;
    // (a) sparsely-active entries: lane = edge of the flattened edge list
    {
      const int32_t sc = sparse ? cnt : 0;
      int32_t incl = sc;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int32_t t = __shfl_up_sync(kFull, incl, d);
        if (lane >= d) incl += t;
      }
      const int32_t total = __shfl_sync(kFull, incl, 31);
      const int32_t excl = incl - sc;
      // lane -> (entry, edge) of flattened position idx: the last entry whose
      // exclusive offset is <= idx
      auto locate = [&](int32_t idx, int32_t &uj, int32_t &k, uint32_t &mj) {
        int32_t j = 0;
#pragma unroll
        for (int st = 16; st > 0; st >>= 1) {
          const int32_t ex = __shfl_sync(kFull, excl, j + st);
          if (ex <= idx) j += st;
        }
        uj = __shfl_sync(kFull, u, j);
        k = __shfl_sync(kFull, b, j) + (idx - __shfl_sync(kFull, excl, j));
        mj = __shfl_sync(kFull, m, j);
      };
      // the next 32 positions' edge ids and weights are loaded before this
      // group's distances are compared (one round trip of each group overlaps)
      int32_t nuj = 0, nv = 0, nw = 0;
      uint32_t nmj = 0;
      if (total > 0) {
        int32_t k;
        locate(lane, nuj, k, nmj);
        if (lane < total) {
          nv = __ldg(S.dst + k);
          nw = __ldg(S.w + k);
        }
      }
      for (int32_t t0 = 0; t0 < total; t0 += 32) {
        const int32_t idx = t0 + lane;
        const int32_t uj = nuj, v = nv, w = nw;
        const uint32_t mj = nmj;
        if (t0 + 32 < total) {
          int32_t k;
          locate(idx + 32, nuj, k, nmj);
          if (idx + 32 < total) {
            nv = __ldg(S.dst + k);
            nw = __ldg(S.w + k);
          }
        }
        if (idx < total) {
          // the entry's sources four at a time: their u and v distance loads
          // are issued together
          uint32_t mm = mj;
          while (mm) {
            int32_t ss[4], du[4], dv[4];
#pragma unroll
            for (int t = 0; t < 4; ++t) {
              ss[t] = mm ? __ffs(mm) - 1 : -1;
              mm &= mm - 1;
            }
#pragma unroll
            for (int t = 0; t < 4; ++t) {
              du[t] = ss[t] >= 0 ? __ldcg(S.dist + (int64_t)uj * kLanes + ss[t]) : INT_MAX;
              dv[t] = ss[t] >= 0 ? __ldcg(S.dist + (int64_t)v * kLanes + ss[t]) : INT_MIN;
            }
#pragma unroll
            for (int t = 0; t < 4; ++t) {
              if (du[t] == INT_MAX) continue;
              const int32_t s = ss[t];
              const int32_t np = du[t] + w;
              if (np < dv[t]) {
                red_min(S.dist + (int64_t)v * kLanes + s, np);
                if (np < s_cut[s]) {
                  if (scan) {
                    red_or(S.nacc + v, 1u << s);
                  } else if (atomicOr(S.nacc + v, 1u << s) == 0u) {
                    S.qstamp[v] = it;
                    bs_enqueue_first(S, qo, qcnt_out, v);
                  }
                } else {
                  if (np < *(volatile int32_t *)(s_fmin + s)) atomicMin(s_fmin + s, np);
                  if (scan) {
                    red_or(S.far + v, 1u << s);
                  } else if (atomicOr(S.far + v, 1u << s) == 0u) {
                    bs_far_push(S, p, v);
                  }
                }
              }
            }
          }
        }
      }
    }
    // (b) busy entries: lane = source, one entry at a time, in groups of 32
    // edges.  The distance lines of a group's 32 edges are gathered into the
    // warp's shared buffer with cp.async (one round trip, no registers held);
    // lane t then collects edge t's near / far source masks and updates its
    // vertex.  The next group's edge ids and weights (and, at the start of an
    // entry, the entry's own distances) are loaded before the current
    // gather is waited for, so that round trip overlaps it.
    uint32_t dense = __ballot_sync(kFull, !sparse && cnt > 0);
    int32_t fmin = INT_MAX;  // lane = source: smallest far value this warp produced
    int32_t cu = 0, ck = 0, cend = 0, du = INT_MAX, vv = 0, ww = 0;
    bool have = false, live = false;
    // next group: same entry (ck + 32 < cend) or the next dense entry
    auto load_group = [&](int32_t k0, int32_t kend, int32_t &v_, int32_t &w_) {
      v_ = 0;
      w_ = 0;
      if (k0 + lane < kend) {
        v_ = __ldg(S.dst + k0 + lane);
        w_ = __ldg(S.w + k0 + lane);
      }
    };
    auto open_entry = [&](int32_t j, int32_t &u_, int32_t &k_, int32_t &e_, int32_t &du_, bool &live_) {
      u_ = __shfl_sync(kFull, u, j);
      k_ = __shfl_sync(kFull, b, j);
      e_ = k_ + __shfl_sync(kFull, cnt, j);
      const bool act = (__shfl_sync(kFull, m, j) >> lane) & 1u;
      du_ = act ? __ldcg(S.dist + (int64_t)u_ * kLanes + lane) : INT_MAX;
      live_ = act;
    };
    if (dense) {
      const int32_t j = __ffs(dense) - 1;
      dense &= dense - 1;
      open_entry(j, cu, ck, cend, du, live);
      load_group(ck, cend, vv, ww);
      have = true;
    }
    while (have) {
      const int32_t cn = min(32, cend - ck);
      // lane l copies sources 4(l%8) .. 4(l%8)+3 of edge q + l/8
      for (int32_t q = 0; q < cn; q += 4) {
        const int32_t t = q + (lane >> 3);
        const int32_t vt = __shfl_sync(kFull, vv, t & 31);
        if (t < cn) cp_async16(dl + t * kLanes + (lane & 7) * 4, S.dist + (int64_t)vt * kLanes + (lane & 7) * 4);
      }
      // the next group's loads, issued before the wait
      int32_t nu = cu, nk = ck + 32, nend = cend, ndu = du, nvv = 0, nww = 0;
      bool nlive = live, nhave = true;
      if (nk >= cend) {
        if (dense) {
          const int32_t j = __ffs(dense) - 1;
          dense &= dense - 1;
          open_entry(j, nu, nk, nend, ndu, nlive);
        } else {
          nhave = false;
        }
      }
      if (nhave) load_group(nk, nend, nvv, nww);
      cp_async_wait_all();
      __syncwarp();
      const bool lv = live && du != INT_MAX;
      uint32_t my_nb = 0, my_fb = 0;
      for (int32_t t = 0; t < cn; ++t) {
        const int32_t vt = __shfl_sync(kFull, vv, t);
        const int32_t wt = __shfl_sync(kFull, ww, t);
        bool near = false, farb = false;
        if (lv) {
          const int32_t np = du + wt;
          if (np < dl[t * kLanes + lane]) {
            red_min(S.dist + (int64_t)vt * kLanes + lane, np);
            near = np < cut;
            farb = !near;
            if (farb && np < fmin) fmin = np;
          }
        }
        const uint32_t nb = __ballot_sync(kFull, near);
        const uint32_t fb = __ballot_sync(kFull, farb);
        if (lane == t) {
          my_nb = nb;
          my_fb = fb;
        }
      }
      __syncwarp();  // the buffer is refilled by the next group
      if (scan) {
        if (my_nb) red_or(S.nacc + vv, my_nb);
        if (my_fb) red_or(S.far + vv, my_fb);
      } else {
        if (my_nb && atomicOr(S.nacc + vv, my_nb) == 0u) {
          S.qstamp[vv] = it;
          bs_enqueue_first(S, qo, qcnt_out, vv);
        }
        if (my_fb && atomicOr(S.far + vv, my_fb) == 0u) bs_far_push(S, p, vv);
      }
      cu = nu;
      ck = nk;
      cend = nend;
      du = ndu;
      live = nlive;
      vv = nvv;
      ww = nww;
      have = nhave;
    }
    if (fmin != INT_MAX && fmin < *(volatile int32_t *)(s_fmin + lane)) atomicMin(s_fmin + lane, fmin);
  }
}

__global__ void __launch_bounds__(256, 4) k_bsssp(BsState S) {
  __shared__ int32_t s_cut[kLanes];
  __shared__ int32_t s_fmin[kLanes];  // this CTA's smallest far value per source
  __shared__ int32_t s_fcnt[256 / 32 + 1];  // cta_flush counts
  // per warp: 32 gathered distance lines (relax), or the staged queue and
  // far-list appends (publish, advance)
  __shared__ alignas(16) int32_t s_wbuf[256 / 32][32 * kLanes];
  static_assert(kStage * (sizeof(int64_t) + sizeof(int32_t)) <= sizeof(s_wbuf[0]), "staging fits the warp buffer");
  int64_t *const s_stq = reinterpret_cast<int64_t *>(s_wbuf[threadIdx.x >> 5]);
  int32_t *const s_stl = s_wbuf[threadIdx.x >> 5] + 2 * kStage;
  const int32_t lane = threadIdx.x & 31;
  const int32_t wib = threadIdx.x >> 5;
  const int64_t gwarp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int32_t tstride = gridDim.x * blockDim.x;
  const int32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  int in = 0;
  int64_t adv = 0;
  int32_t it = 1;
  bool fdirty = false;  // a relax since the last advance marked far masks without listing them
  LoopClock clk;
  clk.start(S.loop_limit_ns);
  for (;; ++it) {
    if (stopped(S.stop, it)) break;
    const int32_t n = *(volatile int32_t *)(S.cnt + (it - 1) % 3);
    int32_t *qcnt_out = S.cnt + it % 3;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      S.cnt[(it + 1) % 3] = 0;
      S.cnt[5 + (it + 1) % 3] = 0;
      S.wctr[(it + 1) % 3] = 0;
      S.hcnt[(it + 1) % 3] = 0;
    }
    const int32_t nh = *(volatile int32_t *)(S.hcnt + (it - 1) % 3);
    const bool scan = S.scan_div > 0 && ((int64_t)n + nh) * S.scan_div >= S.V;
    fdirty |= scan;
    const int p = (int)(adv & 1);
    // ---- relax
    {
      const int32_t curl = __ldcg(S.cur + p * kLanes + lane);
      const int64_t cl = (int64_t)curl + S.delta;
      const int32_t cut = cl > INT_MAX ? INT_MAX : (int32_t)cl;
      if (threadIdx.x < kLanes) {
        s_cut[threadIdx.x] = cut;
        s_fmin[threadIdx.x] = INT_MAX;
      }
      // the minima the next advance accumulates and the far list it rebuilds
      // were last read by the previous advance
      if (blockIdx.x == 0 && threadIdx.x < kLanes) S.gmin[(p ^ 1) * kLanes + threadIdx.x] = INT_MAX;
      if (blockIdx.x == 0 && threadIdx.x == 0) S.cnt[3 + (p ^ 1)] = 0;
      __syncthreads();
      bs_relax(S, n, (int64_t)n + nh, S.q[in], S.hq[in], S.q[in ^ 1], qcnt_out, cut, s_cut, p, it, S.wctr + it % 3,
               nwarps, scan, s_wbuf[wib], s_fmin);
      __syncthreads();
      if (threadIdx.x < kLanes && s_fmin[threadIdx.x] != INT_MAX)
        atomicMin(S.gmin + p * kLanes + threadIdx.x, s_fmin[threadIdx.x]);
    }
    if (!grid_barrier(S.bar, gridDim.x, S.err, S.timeout_ns)) break;
    // ---- publish near masks of the queued vertices; OR them into the active set
    if (scan) {  // queue every vertex with a near mask, all its chunks
      WarpStage<int64_t> stq{s_stq, S.q[in ^ 1], qcnt_out, S.qcap, 0};
      uint32_t act = 0;
      for (int64_t v0 = tid - lane; v0 < S.V; v0 += tstride) {
        const int64_t v = v0 + lane;
        const uint32_t x = v < S.V ? __ldcg(S.nacc + v) : 0u;
        bool one = false;
        if (x) {
          S.nacc[v] = 0;
          S.fr[v] = x;
          S.qstamp[v] = it;
          act |= x;
          one = S.off[v + 1] - S.off[v] <= S.chunk;
          if (!one) bs_enqueue(S, S.q[in ^ 1], qcnt_out, (int32_t)v);
        }
        stq.push(one, v << 32, S.err);
      }
      cta_flush(stq, s_fcnt, S.err);
      act = __reduce_or_sync(kFull, act);
      if (lane == 0 && act) atomicOr(reinterpret_cast<uint32_t *>(S.cnt + 5 + it % 3), act);
    } else {
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
            const int32_t nch = ceil_div(S.off[v + 1] - S.off[v], S.chunk);
            if (nch > 1 && x) {  // chunks 1 .. nch-1 of a high-degree vertex queued by the relax
              const int32_t pos = atomicAdd(S.hcnt + it % 3, nch - 1);
              if ((int64_t)pos + nch - 1 > S.qcap) {
                atomicOr(S.err, DEV_ERR_OVERFLOW);
              } else {
                for (int32_t c = 1; c < nch; ++c) S.hq[in ^ 1][pos + c - 1] = ((int64_t)v << 32) | (uint32_t)c;
              }
            }
          }
        }
        act |= x;
      }
      act = __reduce_or_sync(kFull, act);
      if (lane == 0 && act) atomicOr(reinterpret_cast<uint32_t *>(S.cnt + 5 + it % 3), act);
    }
    clk.tick(S.stop, it, S.err);
    if (!grid_barrier(S.bar, gridDim.x, S.err, S.timeout_ns)) break;
    // ---- advance the sources with no near work
    uint32_t unfinished = 0;
    {
      const int32_t cv = __ldcg(S.cur + p * kLanes + lane);
      unfinished = __ballot_sync(kFull, cv != INT_MAX);
    }
    const uint32_t active = (uint32_t)*(volatile int32_t *)(S.cnt + 5 + it % 3);
    const uint32_t A = unfinished & ~active;
    bool pending = false;  // a source is left whose new window came out empty
    if (A) {
      // after a scanning relax the far list misses vertices: walk all V instead
      const bool fscan = fdirty;
      // A pass over all V rebuilds the far list only when the next relax is
      // likely to queue (it is small); before a scanning relax the list would
      // be stale again.  (The queue count is stable here: only pass 2 adds.)
      const bool relist = !fscan || (int64_t)*(volatile int32_t *)qcnt_out * S.scan_div < S.V;
      fdirty = !relist;
      const int32_t fcount = fscan ? S.V : min(*(volatile int32_t *)(S.cnt + 3 + p), S.V);
      const int32_t *fla = S.fl[p];
      const int32_t curl = __ldcg(S.cur + p * kLanes + lane);
      const int64_t window = (int64_t)curl + S.delta;
      const bool adv_l = (A >> lane) & 1u;
      // The new window of an advancing source starts at the smallest far value
      // recorded for it since its last advance (relaxes and the kept entries of
      // that advance add to S.gmin[p]).  That is at most every far entry still
      // pending, so nothing is skipped; a value that has since dropped into an
      // earlier window makes at worst one empty bucket.
      const int32_t nA = __popc(A);
      const bool few = nA <= kAdvFew;
      const int32_t FB = bs_batch(fcount, nwarps);
      if (threadIdx.x < kLanes) s_fmin[threadIdx.x] = INT_MAX;
      __syncthreads();
      // pass 2: move [cur', cur'+delta) to the near frontier, keep the rest
      const int32_t gm = __ldcg(S.gmin + p * kLanes + lane);
      const int32_t newcur = adv_l ? gm : curl;
      const int64_t hi = (int64_t)newcur + S.delta;
      int64_t *qo = S.q[in ^ 1];
      WarpStage<int64_t> stq{s_stq, qo, qcnt_out, S.qcap, 0};
      WarpStage<int32_t> stl{s_stl, S.fl[p ^ 1], S.cnt + 3 + (p ^ 1), S.V, 0};
      int32_t kmin = INT_MAX;  // lane = source: smallest value it keeps far
      for (int64_t e0 = gwarp * FB; e0 < fcount; e0 += nwarps * FB) {
        const int64_t e = e0 + lane;
        const bool mine = lane < FB && e < fcount;
        int32_t vl = 0;
        uint32_t fml = 0;
        if (mine) {
          vl = fscan ? (int32_t)e : __ldcg(fla + e);
          fml = __ldcg(S.far + vl);
        }
        uint32_t rem = fml & ~A;  // far bits of sources that do not advance stay
        uint32_t mv = 0;
        if (few) {
          const uint32_t fa = fml & A;
          int32_t ds[kAdvFew];
          bs_far_loads(S, vl, fa, A, nA, ds);
          uint32_t aa = A;
#pragma unroll
          for (int32_t k = 0; k < kAdvFew; ++k) {
            if (k >= nA) break;  // warp-uniform
            const int32_t s = __ffs(aa) - 1;
            aa &= aa - 1;
            const int64_t win = __shfl_sync(kFull, window, s);
            const int64_t his = __shfl_sync(kFull, hi, s);
            const int32_t ncs = __shfl_sync(kFull, newcur, s);
            int32_t kept = INT_MAX;
            if (((fa >> s) & 1u) && ncs != INT_MAX && (int64_t)ds[k] >= win) {
              if ((int64_t)ds[k] >= his) {
                rem |= 1u << s;
                kept = ds[k];
              } else {
                mv |= 1u << s;
              }
            }
            const int32_t km = __reduce_min_sync(kFull, kept);
            if (lane == 0 && km != INT_MAX && km < *(volatile int32_t *)(s_fmin + s)) atomicMin(s_fmin + s, km);
          }
        }
        uint32_t todo = few ? 0u : __ballot_sync(kFull, (fml & A) != 0u);
        while (todo) {
          int32_t js[4], vs[4];
          bool hs[4];
#pragma unroll
          for (int t = 0; t < 4; ++t) {
            js[t] = -1;
            int32_t j = 0;
            if (todo) {
              j = __ffs(todo) - 1;
              todo &= todo - 1;
              js[t] = j;
            }
            const uint32_t fm = __shfl_sync(kFull, fml, j);
            vs[t] = __shfl_sync(kFull, vl, j);
            hs[t] = js[t] >= 0 && adv_l && ((fm >> lane) & 1u) && newcur != INT_MAX;
          }
          int32_t ds[4];
#pragma unroll
          for (int t = 0; t < 4; ++t) ds[t] = hs[t] ? __ldcg(S.dist + (int64_t)vs[t] * kLanes + lane) : 0;
#pragma unroll
          for (int t = 0; t < 4; ++t) {
            const bool in_win = hs[t] && (int64_t)ds[t] >= window;
            const bool keep = in_win && (int64_t)ds[t] >= hi;
            const bool move = in_win && (int64_t)ds[t] < hi;
            if (keep && ds[t] < kmin) kmin = ds[t];
            const uint32_t kb = __ballot_sync(kFull, keep);
            const uint32_t mb = __ballot_sync(kFull, move);
            if (lane == js[t]) {
              rem |= kb;
              mv = mb;
            }
          }
        }
        if (mine && rem != fml) S.far[vl] = rem;
        if (relist) stl.push(mine && rem != 0u, vl, S.err);
        bool one = false;
        if (mine && mv) {
          if (atomicMax(S.qstamp + vl, it) < it) {
            S.fr[vl] = mv;
            one = S.off[vl + 1] - S.off[vl] <= S.chunk;
            if (!one) bs_enqueue(S, qo, qcnt_out, vl);
          } else {
            atomicOr(S.fr + vl, mv);
          }
        }
        stq.push(one, (int64_t)vl << 32, S.err);
      }
      cta_flush(stq, s_fcnt, S.err);
      cta_flush(stl, s_fcnt, S.err);
      if (kmin != INT_MAX && kmin < *(volatile int32_t *)(s_fmin + lane)) atomicMin(s_fmin + lane, kmin);
      __syncthreads();
      // the next advance's minima: what stayed far, and (block 0) the
      // unchanged minima of the sources that did not advance
      if (threadIdx.x < kLanes) {
        int32_t mm = s_fmin[threadIdx.x];
        if (blockIdx.x == 0 && !((A >> threadIdx.x) & 1u)) mm = min(mm, __ldcg(S.gmin + p * kLanes + threadIdx.x));
        if (mm != INT_MAX) atomicMin(S.gmin + (p ^ 1) * kLanes + threadIdx.x, mm);
      }
      if (blockIdx.x == 0 && threadIdx.x < kLanes) S.cur[(p ^ 1) * kLanes + threadIdx.x] = newcur;
      pending = __ballot_sync(kFull, newcur != INT_MAX) != 0u;
      if (!grid_barrier(S.bar, gridDim.x, S.err, S.timeout_ns)) break;
      ++adv;
    }
    const int32_t m = *(volatile int32_t *)qcnt_out;
    if (m == 0 && !pending) break;  // an empty window advances again from exact minima
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
  for (int32_t i = 0; i < 3; ++i) {
    S.wctr[i] = 0;
    S.hcnt[i] = 0;
  }
  *S.stop = 0;
  for (int32_t s = 0; s < kLanes; ++s) {
    S.cur[s] = s < nsrc ? 0 : INT_MAX;
    S.cur[kLanes + s] = S.cur[s];
    S.gmin[s] = INT_MAX;
    S.gmin[kLanes + s] = INT_MAX;
  }
  for (int32_t s = 0; s < nsrc; ++s) {
    const int32_t v = S.perm[srcs[s]];
    S.dist[(int64_t)v * kLanes + s] = 0;
    if (!S.fr[v]) bs_enqueue(S, S.q[0], S.cnt + 0, v);
    S.fr[v] |= 1u << s;
  }
}

// Rows out[s][v] = dist[perm[v]][s] for s < nsrc (v an original id), through
// 32 x 32 shared-memory tiles so the distance-line reads and the row writes are
// both coalesced.
__global__ void __launch_bounds__(256) k_bsssp_out(const int32_t *__restrict__ dist, const int32_t *__restrict__ perm,
                                                   int32_t V, int32_t nsrc, int32_t *__restrict__ out) {
  __shared__ int32_t tile[kLanes][33];
  for (int64_t v0 = (int64_t)blockIdx.x * 32; v0 < V; v0 += (int64_t)gridDim.x * 32) {
    for (int32_t i = threadIdx.x; i < 32 * kLanes; i += blockDim.x) {
      const int32_t vv = i / kLanes, s = i % kLanes;
      tile[s][vv] = v0 + vv < V ? dist[(int64_t)perm[v0 + vv] * kLanes + s] : 0;
    }
    __syncthreads();
    for (int32_t i = threadIdx.x; i < 32 * nsrc; i += blockDim.x) {
      const int32_t s = i / 32, vv = i % 32;
      if (v0 + vv < V) out[(int64_t)s * V + v0 + vv] = tile[s][vv];
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------ host
BsBuffers::~BsBuffers() {
  if (owned)
    for (void *p : {(void *)dist, (void *)masks, (void *)ints, (void *)queues, (void *)out, (void *)dsrc})
      if (p) cudaFree(p);
}

gg_status bsssp_buffers(gg_graph *g, int32_t nsrc, bool owned, BsBuffers *b) {
  GG_TRY(ensure_relabel(g));
  const int32_t V = g->csr.V;
  const int64_t E = g->csr.E;
  b->qcap = (int64_t)V + E / kMinChunk + 64;  // any tuning's chunk fits
  b->owned = owned;
  const size_t sz[6] = {sizeof(int32_t) * (size_t)V * kLanes, sizeof(uint32_t) * 3 * (size_t)V,
                        sizeof(int32_t) * (3 * (size_t)V + 256), sizeof(int64_t) * 4 * (size_t)b->qcap,
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
  S.wctr = hdr + 144;       // 3
  S.q[0] = b.queues;
  S.q[1] = b.queues + b.qcap;
  S.hq[0] = b.queues + 2 * b.qcap;
  S.hq[1] = b.queues + 3 * b.qcap;
  S.hcnt = hdr + 150;       // 3
  S.qcap = b.qcap;
  S.off = g->rel->g.off;  // the degree-ordered copy (bsssp_buffers built it)
  S.dst = g->rel->g.dst;
  S.w = g->rel->g.w;
  S.perm = g->rel->perm;
  S.V = V;
  S.delta = delta;
  const gg_batch_tuning t = effective_tuning(g, GG_BATCH_SSSP, 1);
  S.chunk = t.chunk;
  S.ep_max = t.edge_parallel_max;
  S.scan_div = kBsScanDiv;
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
  if (reinterpret_cast<uintptr_t>(S.dist) % 16 != 0)  // the relax copies distance lines 16 bytes at a time
    return set_error(GG_ERR_INVALID, "batched SSSP distance buffer is not 16-byte aligned");
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
  k_bsssp_out<<<g->sm_count * 8, 256, 0, st>>>(S.dist, S.perm, S.V, k, out_rows);
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
  bool per_cta = false;
  GG_TRY(bsssp_use_cta(g, &per_cta));
  if (per_cta) {  // a CTA per source (batch_sssp_cta.cu)
    const int32_t W = std::min(bsssp_cta_width(g), nsrc);
    CtaBuffers cb;
    GG_TRY(bsssp_cta_buffers(g, W, &g->bq_cta, &cb));
    const uint64_t l0 = launches();
    cudaEventRecord(g->ev0, st);
    float loop_ms = 0;
    int32_t iters = 0, advs = 0;
    for (int32_t base = 0; base < nsrc; base += W) {
      const int32_t k = std::min(W, nsrc - base);
      GG_CUDA(cudaMemcpyAsync(cb.dsrc, sources + base, sizeof(int32_t) * k, cudaMemcpyDefault, st));
      GG_TRY(bsssp_cta_run(g, st, cb, cb.rows, k, delta, true));
      GG_CUDA(cudaMemcpyAsync(dist_out + (size_t)base * V, cb.rows, sizeof(int32_t) * (size_t)k * V,
                              cudaMemcpyDefault, st));
      GG_CUDA(cudaMemcpyAsync(g->h_pinned + 30, cb.stats, sizeof(int32_t) * 2, cudaMemcpyDeviceToHost, st));
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
