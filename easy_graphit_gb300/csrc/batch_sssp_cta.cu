// Batched SSSP for high-diameter graphs: every source gets a CTA of its own,
// which runs the whole delta-stepping loop for that source alone -- its
// distance row, stamps, piles, ring and queues private to it, its control
// words and relax lists in shared memory, __syncthreads between
// steps and no grid barrier at all.  The CTAs of a pass run side by side, one
// source each.
//
// Why: on a mesh such as the 4096^2 grid, a 32-source pass of the lane-per-
// source kernel (batch_sssp.cu) needs ~10^5 iterations of three grid-wide
// phases each, for a handful of vertices per source per iteration; the time
// goes to barriers.  Here a bucket of a source costs the few L2 round trips of
// its own steps.  On low-diameter graphs (R-MAT) a source's buckets are large
// and one CTA per source is too little parallelism: the lane-per-source
// kernel stays the choice there (gg_batch_tuning.per_source_cta).
//
// The loop is delta-stepping with windows [J delta, (J+1) delta) (the window
// is relaxed until nothing in it improves, then the next nonempty bucket
// opens), over a structure shaped so that a bucket costs one step:
//  - a ring of kMeshSlots buckets ahead of the current one, each a list of
//    whole entries (vertex, priority, first edge, end edge): a relaxation
//    that lowers a vertex to a later bucket lists it in that bucket's slot
//    (stamp[v] = J + 1 keeps it listed once per bucket), so an advance takes
//    the next nonempty slot without scanning anything else, and the entry
//    carries what its relax needs (parks load the target's edge range with its
//    distance);
//  - buckets beyond the ring go to a far pile, split into a new ring when the
//    ring runs dry (its smallest live value opens the next window); a full
//    slot spills to a pile that every advance scans in place (compacted when
//    mostly dead);
//  - the thread that reads a slot entry relaxes it; improvements inside the
//    window go to a shared-memory list and are relaxed in further rounds of
//    the same step (one __syncthreads a round); a full list sends vertices to
//    a per-step queue that the next step relaxes;
//  - warp 0 closes a step and decides the next one in one pass.
// Results are each source's exact distances.  The windows are aligned to
// multiples of delta where the reference's start at the exact minimum, which
// changes the number of advances, never a distance.
#include <atomic>
#include <vector>

#include "batch.h"
#include "bucket_queue.cuh"

namespace gg {

struct CtaSsspArgs {
  DGraph g;
  const int32_t *srcs;  // k sources
  int32_t *rows;        // [k][V] distances (parts mode: one row of V)
  int32_t *stamp;       // [k][V]
  int32_t *piles;       // [k][mesh_block_ints(V)]: far and spill piles, overflow queues, ring
  int32_t V, delta;
  int32_t *err;
  int32_t *stats;       // [0] most steps of a source, [1] bucket advances of all sources
  uint64_t loop_limit_ns;
  // Parts mode (gg_sssp_parts): CTA k owns the vertices [part_lo[k],
  // part_lo[k+1]) of a disjoint union and one row of distances and stamps;
  // its block of mesh_block_ints(part size) starts at piles + part_base[k].
  const int32_t *part_lo;
  const int64_t *part_base;
};

// Entries a far or spill pile holds for a source (or part) of Vp vertices.
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

constexpr int kMeshThreads = 1024;
constexpr int kMeshList = 2048;          // entries of each shared relax list
constexpr int kMeshInFlight = 4;         // pile entries / edges a thread keeps in flight
constexpr int kMeshSlots = 128;          // buckets of the ring (a power of two)
constexpr int32_t kMeshCompactMin = 2048;  // smaller spill piles are never compacted
constexpr size_t kMeshSmem = 2 * kMeshList * sizeof(int4);

// Entries a ring slot holds for a source (or part) of n vertices.
__host__ __device__ __forceinline__ int64_t mesh_slot_cap(int64_t n) {
  const int64_t c = (n / 16 + 31) / 32 * 32;
  return c < 1024 ? 1024 : (c > 16384 ? 16384 : c);
}
// Ints of one source's block: far piles and spill piles (2 cap each), two
// overflow queues (2 cap each), cap = part_cap(n), and the ring of int4
// entries.
__host__ __device__ __forceinline__ int64_t mesh_block_ints(int64_t n) {
  return 8 * part_cap(n) + 4 * kMeshSlots * mesh_slot_cap(n);
}

enum : int32_t { MESH_RELAX = 0, MESH_ADV = 1, MESH_HIMIN = 2, MESH_HISPLIT = 3, MESH_COMPACT = 4, MESH_DONE = 5 };

// Shared control words of one source's loop.  Counters are appended to during
// a step; the state below them is written by warp 0 between steps.
struct MeshCtl {
  int32_t rc[kMeshSlots];  // entries of each ring slot
  int32_t far_cnt[2];      // far piles, by generation parity
  int32_t sp_cnt[2];       // spill piles, by generation parity
  int32_t q_cnt[2];        // overflow queues, by step parity
  int32_t list_cnt[3];     // relax-list counts, rotating by round
  int32_t rquit[3];        // time limit reached, rotating by round like list_cnt
  int32_t srec;            // smallest live spill value listed since the last advance
  int32_t sdead;           // spill entries the last advance found dead or took
  int32_t himin;           // smallest live far value (MESH_HIMIN)
  // loop state
  int32_t kind, in;        // step kind; overflow queue the step reads
  int32_t J;               // bucket of the window being relaxed: [J delta, (J+1) delta)
  int32_t U;               // its end (the cutoff)
  int32_t Jend;            // the ring holds buckets (J, Jend); the far pile the rest
  int32_t hz;              // Jend * delta: parks below it go to the ring
  int32_t nJ, win;         // bucket and window end of an advance
  int32_t gh, gs;          // far / spill pile generations
  int32_t nfar, nsp, nq, nslot;  // entries the step scans
  int32_t gh_w, gs_w;      // generations the step's parks append to
  int32_t after_himin;
  int32_t steps, adv;
  int32_t quit;
};

// Pile, queue and ring pointers of one source.
struct MeshView {
  const int32_t *__restrict__ off;
  const int32_t *__restrict__ dst;
  const int32_t *__restrict__ w;
  int32_t *dist, *stamp;
  int32_t *far[2], *sp[2], *q[2];
  int4 *ring;  // [kMeshSlots][slot_cap] entries (v, p, first edge, end edge)
  int64_t qcap;
  int32_t cap;       // entries a far or spill pile holds
  int32_t slot_cap;  // entries a ring slot holds
  int32_t delta;
  int32_t *err;
};

// Where the current step sends what it finds.
struct MeshSink {
  int32_t lo;               // start of the window being relaxed
  int32_t cutoff;           // improvements below it are relaxed in this step
  int32_t hz;               // parks below it go to the ring, the others far
  int32_t *rc;              // ring slot counts (shared)
  int32_t *far, *far_cnt;   // far pile the step appends to
  int32_t far_tag;
  int32_t *sp, *sp_cnt;     // spill pile (ring slots that are full)
  int4 *list;               // relax list of this round (v, p, b, e); e < 0: a ring entry, end edge ~e
  int32_t *list_cnt;
  int32_t *q, *q_cnt;       // overflow queue of this step
  int32_t qtag;             // stamp of a vertex on that queue (below every pile tag)
};

__device__ __forceinline__ int32_t mesh_far_tag(int32_t gen) { return -gen - 1; }

__device__ __forceinline__ void mesh_append(int32_t *pile, int32_t *cnt, int32_t cap, int32_t v, int32_t *err) {
  const int32_t pos = agg_inc(cnt);
  if (pos < cap)
    pile[pos] = v;
  else
    atomicOr(err, DEV_ERR_OVERFLOW);
}

// v at priority p (edges [b, e)) goes to the ring slot of its bucket as a
// whole entry, so the advance that takes the bucket relaxes it without
// loading anything first; a full slot sends v to the spill pile, whose live
// values fold into the thread's minimum smin.
__device__ __forceinline__ void mesh_ring_append(const MeshView &mv, const MeshSink &s, int32_t v, int32_t p,
                                                 int32_t b, int32_t e, int32_t &smin) {
  const int32_t slot = (p / mv.delta) & (kMeshSlots - 1);
  const int32_t pos = atomicAdd(s.rc + slot, 1);
  if (pos < mv.slot_cap) {
    mv.ring[(int64_t)slot * mv.slot_cap + pos] = make_int4(v, p, b, e);
  } else {
    smin = min(smin, p);
    mesh_append(s.sp, s.sp_cnt, mv.cap, v, mv.err);
  }
}

// v (at priority p, edges [b, e)) goes to the relax list; a full list sends v
// to the step's overflow queue, whose step re-reads its distance and edges.
// The queue takes a vertex once per step (its stamp exchanged for the step's
// tag), so it never holds more than V entries; a stamp taken over this way
// only lets a later park list the vertex again (a duplicate, never a miss).
__device__ __forceinline__ void mesh_list_push(const MeshView &mv, const MeshSink &s, int32_t v, int32_t p,
                                               int32_t b, int32_t e) {
  const int32_t pos = agg_inc(s.list_cnt);
  if (pos < kMeshList) {
    s.list[pos] = make_int4(v, p, b, e);
  } else {
    if (atomicExch(mv.stamp + v, s.qtag) == s.qtag) return;
    const int32_t qp = agg_inc(s.q_cnt);
    if (qp < mv.qcap)
      s.q[qp] = v;
    else
      atomicOr(mv.err, DEV_ERR_OVERFLOW);
  }
}

// Parks v at priority p >= the cutoff: in the ring slot of its bucket below
// the horizon, else on the far pile.  stamp[v] names where v is listed (bucket
// J as J + 1, far generation g as -g - 1); `st` is the stamp as loaded with
// v's distance, and a vertex its target lists already is not listed again.
// In a relax the stamp is written with a plain store: two parks of v into one
// bucket in the same round may both list it (the entry is relaxed twice, the
// second time as a no-op).  Pile splits (EXCH) decide by an exchange, so a
// split never copies a vertex twice.
template <bool EXCH>
__device__ __forceinline__ void mesh_park(const MeshView &mv, const MeshSink &s, int32_t v, int32_t p, int32_t b,
                                          int32_t e, int32_t st, int32_t &smin) {
  const int32_t tag = p < s.hz ? p / mv.delta + 1 : s.far_tag;
  if (st == tag) return;
  if (EXCH) {
    if (atomicExch(mv.stamp + v, tag) == tag) return;
  } else {
    mv.stamp[v] = tag;
  }
  if (p < s.hz)
    mesh_ring_append(mv, s, v, p, b, e, smin);
  else
    mesh_append(s.far, s.far_cnt, mv.cap, v, mv.err);
}

// Relaxes the out-edges [b, e) of v, kMeshInFlight edges at a time: their
// targets and weights -- for a ring entry (`check`) loaded with v's current
// distance, which replaces the entry's priority p when it is lower (v was
// lowered after it was listed; a lowering within the same bucket finds v
// listed there already and adds no entry), and a vertex now below the window
// was relaxed in an earlier window at that value and stops here.  Any other
// entry carries a value that was current when it was listed, and a later
// lowering listed the vertex again, so it needs no such load.  Then the
// targets' distances, stamps and edge
// ranges, then fire-and-forget minima for the improving ones (an improvement
// is decided against the value read: redundant at worst, never lost).
// Improvements below the cutoff go to the next relax list, the others park;
// both carry the target's edge range, so neither needs a load before its own
// relax.
__device__ __forceinline__ void mesh_relax(const MeshView &mv, const MeshSink &s, int32_t v, int32_t p, int32_t b,
                                           int32_t e, bool check, int32_t &smin) {
  for (int32_t k0 = b; k0 < e; k0 += kMeshInFlight) {
    int32_t d[kMeshInFlight], np[kMeshInFlight], prev[kMeshInFlight], st[kMeshInFlight];
    int32_t db[kMeshInFlight], de[kMeshInFlight];
    const int32_t now = check && k0 == b ? __ldcg(mv.dist + v) : p;  // issued with the edges below
#pragma unroll
    for (int j = 0; j < kMeshInFlight; ++j) {
      const int32_t k = k0 + j;
      d[j] = k < e ? __ldg(mv.dst + k) : -1;
      np[j] = k < e ? __ldg(mv.w + k) : INT_MAX;  // the weight, for now
    }
    p = min(p, now);
    if (p < s.lo) return;
#pragma unroll
    for (int j = 0; j < kMeshInFlight; ++j)
      if (d[j] >= 0) np[j] += p;
#pragma unroll
    for (int j = 0; j < kMeshInFlight; ++j) {
      prev[j] = d[j] >= 0 ? __ldcg(mv.dist + d[j]) : INT_MIN;
      st[j] = d[j] >= 0 ? __ldcg(mv.stamp + d[j]) : 0;
      db[j] = d[j] >= 0 ? __ldg(mv.off + d[j]) : 0;
      de[j] = d[j] >= 0 ? __ldg(mv.off + d[j] + 1) : 0;
    }
#pragma unroll
    for (int j = 0; j < kMeshInFlight; ++j)
      if (np[j] < prev[j])
        asm volatile("red.relaxed.gpu.global.min.s32 [%0], %1;" ::"l"(__cvta_generic_to_global(mv.dist + d[j])),
                     "r"(np[j])
                     : "memory");
#pragma unroll
    for (int j = 0; j < kMeshInFlight; ++j) {
      if (prev[j] <= np[j]) continue;
      if (np[j] < s.cutoff)
        mesh_list_push(mv, s, d[j], np[j], db[j], de[j]);
      else
        mesh_park<false>(mv, s, d[j], np[j], db[j], de[j], st[j], smin);
    }
  }
}

// Warp-then-block folds of per-thread values into shared words.
__device__ __forceinline__ void mesh_fold_min(int32_t v, int32_t *dst) {
  v = __reduce_min_sync(0xffffffffu, v);
  if ((threadIdx.x & 31) == 0 && v != INT_MAX) atomicMin(dst, v);
}
__device__ __forceinline__ void mesh_fold_add(int32_t v, int32_t *dst) {
  v = __reduce_add_sync(0xffffffffu, v);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(dst, v);
}

// A ring slot's entries all belong to its bucket: every one goes to the relax
// list as it is, its end edge stored as ~e to mark it as a ring entry, whose
// relax reads the vertex's current distance (mesh_relax).
__device__ __forceinline__ void mesh_scan_slot(const MeshView &mv, const MeshSink &s, const int4 *__restrict__ slot,
                                               int32_t n) {
  for (int32_t i0 = threadIdx.x; i0 < n; i0 += kMeshInFlight * blockDim.x) {
    int4 x[kMeshInFlight];
#pragma unroll
    for (int j = 0; j < kMeshInFlight; ++j)
      x[j] = i0 + j * (int32_t)blockDim.x < n ? __ldcg(slot + i0 + j * blockDim.x) : make_int4(-1, 0, 0, 0);
#pragma unroll
    for (int j = 0; j < kMeshInFlight; ++j)
      if (x[j].x >= 0) mesh_list_push(mv, s, x[j].x, x[j].y, x[j].z, ~x[j].w);
  }
}

// One pass over pile[0, n) (vertex ids) of an advance to the window [lo, win):
// entries below lo are dead (taken in an earlier window), window entries are
// listed for relaxing with the distance and edge range loaded here.  The rest:
//   KEEP_STAY   stays in place, folded into smin (the spill pile);
//   KEEP_SPLIT  re-parked: ring below the horizon, else the next far pile
//               (the far pile at a refill);
//   KEEP_MOVE   appended to the sink's spill pile, folded into smin (spill
//               compaction; no window then).
enum : int { KEEP_STAY = 1, KEEP_SPLIT = 2, KEEP_MOVE = 3 };
template <int KEEP>
__device__ __forceinline__ void mesh_scan(const MeshView &mv, const MeshSink &s, const int32_t *__restrict__ pile,
                                          int32_t n, int32_t lo, int32_t win, int32_t &smin, int32_t &ndead) {
  const int32_t T = blockDim.x;
  for (int32_t i0 = threadIdx.x; i0 < n; i0 += kMeshInFlight * T) {
    int32_t v[kMeshInFlight], p[kMeshInFlight], b[kMeshInFlight], e[kMeshInFlight];
#pragma unroll
    for (int j = 0; j < kMeshInFlight; ++j) v[j] = i0 + j * T < n ? __ldcg(pile + i0 + j * T) : -1;
#pragma unroll
    for (int j = 0; j < kMeshInFlight; ++j) {
      p[j] = v[j] >= 0 ? __ldcg(mv.dist + v[j]) : -1;
      b[j] = v[j] >= 0 && KEEP != KEEP_MOVE ? __ldg(mv.off + v[j]) : 0;
      e[j] = v[j] >= 0 && KEEP != KEEP_MOVE ? __ldg(mv.off + v[j] + 1) : 0;
    }
#pragma unroll
    for (int j = 0; j < kMeshInFlight; ++j) {
      if (v[j] < 0) continue;
      if (p[j] < win) {
        ndead++;
        if (KEEP != KEEP_MOVE && p[j] >= lo) mesh_list_push(mv, s, v[j], p[j], b[j], e[j]);
        continue;
      }
      if (KEEP == KEEP_STAY) {
        smin = min(smin, p[j]);
      } else if (KEEP == KEEP_MOVE) {
        smin = min(smin, p[j]);
        mesh_append(s.sp, s.sp_cnt, mv.cap, v[j], mv.err);
      } else {
        mesh_park<true>(mv, s, v[j], p[j], b[j], e[j], 0, smin);  // 0: no stamp loaded (the exchange decides)
      }
    }
  }
}

__global__ void __launch_bounds__(kMeshThreads) k_sssp_cta(CtaSsspArgs c) {
  extern __shared__ int4 lists[];  // [2][kMeshList]
  __shared__ MeshCtl C;
  const int64_t k = blockIdx.x;
  MeshView mv{};
  mv.off = c.g.off;
  mv.dst = c.g.dst;
  mv.w = c.g.w;
  mv.err = c.err;
  mv.delta = c.delta;
  int64_t n, cap;
  int32_t *blk;
  if (c.part_lo) {
    n = c.part_lo[k + 1] - c.part_lo[k];
    blk = c.piles + c.part_base[k];
    mv.dist = c.rows;
    mv.stamp = c.stamp;
  } else {
    n = c.V;
    blk = c.piles + k * mesh_block_ints(n);
    mv.dist = c.rows + k * (int64_t)c.V;
    mv.stamp = c.stamp + k * (int64_t)c.V;
  }
  cap = part_cap(n);
  mv.cap = (int32_t)cap;
  mv.slot_cap = (int32_t)mesh_slot_cap(n);
  mv.far[0] = blk;
  mv.far[1] = blk + cap;
  mv.sp[0] = blk + 2 * cap;
  mv.sp[1] = blk + 3 * cap;
  mv.q[0] = blk + 4 * cap;
  mv.q[1] = blk + 6 * cap;
  mv.qcap = 2 * cap;
  mv.ring = reinterpret_cast<int4 *>(blk + 8 * cap);
  const int32_t src = c.srcs[k];
  const int32_t delta = c.delta;
  if (c.part_lo && threadIdx.x == 0) mv.dist[src] = 0;
  for (int i = threadIdx.x; i < kMeshSlots; i += blockDim.x) C.rc[i] = 0;
  if (threadIdx.x == 0) {
    C.far_cnt[0] = C.far_cnt[1] = 0;
    C.sp_cnt[0] = C.sp_cnt[1] = 0;
    C.q_cnt[0] = 1;  // the source, read by the first step
    C.q_cnt[1] = 0;
    C.list_cnt[0] = C.list_cnt[1] = C.list_cnt[2] = 0;
    C.srec = INT_MAX;
    C.sdead = 0;
    C.himin = INT_MAX;
    C.in = 0;
    C.J = 0;
    C.U = bq_clamp(delta);
    C.Jend = kMeshSlots;
    C.hz = bq_clamp((int64_t)kMeshSlots * delta);
    C.gh = C.gs = 0;
    C.after_himin = 0;
    C.steps = C.adv = 0;
    C.quit = 0;
    mv.q[0][0] = src;
  }
  uint64_t deadline = 0;
  if (threadIdx.x == 0) {
    deadline = globaltimer_ns() + c.loop_limit_ns;
    C.kind = -1;  // no step before the first
  }
  __syncthreads();
  for (;;) {
    // ---- warp 0 closes the last step (lane 0) and decides the next one
    if (threadIdx.x < 32) {
      const int lane = threadIdx.x;
      if (lane == 0) {
        const int32_t last = C.kind;
        if (last >= 0) C.steps++;
        if (last == MESH_ADV || last == MESH_HISPLIT) {
          C.adv++;
          if (last == MESH_ADV) C.rc[C.nJ & (kMeshSlots - 1)] = 0;  // the bucket's slot is consumed
          C.J = C.nJ;
          C.U = C.win;
          C.gh = C.gh_w;
          C.gs = C.gs_w;
        }
        if (last == MESH_RELAX || last == MESH_ADV || last == MESH_HISPLIT) C.in ^= 1;
        if (last == MESH_HIMIN) C.after_himin = 1;
        if (last == MESH_COMPACT) C.gs = C.gs_w;
      }
      __syncwarp();
      // the next ring bucket that holds entries, if any: (J, Jend) in steps of 32
      const int32_t span = min(C.Jend - C.J - 1, kMeshSlots - 1);
      int32_t jr = INT_MAX;
      for (int32_t base = 1; base <= span; base += 32) {
        const int32_t i = base + lane;
        const bool has = i <= span && C.rc[(C.J + i) & (kMeshSlots - 1)] > 0;
        const uint32_t bal = __ballot_sync(0xffffffffu, has);
        if (bal) {
          jr = C.J + base + __ffs(bal) - 1;
          break;
        }
      }
      if (lane == 0) {
        int32_t kind;
        if ((C.steps & 255) == 0) {  // the wall-clock bound and overflow, checked every 256 steps
          const bool late = globaltimer_ns() > deadline;
          if (late) atomicOr(c.err, DEV_ERR_TIMEOUT);
          C.quit = C.quit || late || (*(volatile int32_t *)c.err & (DEV_ERR_OVERFLOW | DEV_ERR_TIMEOUT)) != 0;
        }
        C.nq = min(C.q_cnt[C.in], (int32_t)mv.qcap);
        C.gh_w = C.gh;
        C.gs_w = C.gs;
        const int32_t js = C.srec != INT_MAX ? C.srec / delta : INT_MAX;
        const int32_t nsp = min(C.sp_cnt[C.gs & 1], mv.cap);
        if (C.quit) {
          kind = MESH_DONE;
        } else if (C.nq > 0) {
          kind = MESH_RELAX;
        } else if (C.after_himin) {
          C.after_himin = 0;
          if (C.himin == INT_MAX) {
            kind = MESH_DONE;
          } else {  // refill: the far pile's smallest value opens the window and a new ring
            kind = MESH_HISPLIT;
            C.nJ = C.himin / delta;
            C.win = bq_clamp(((int64_t)C.nJ + 1) * delta);
            C.Jend = (int32_t)min((int64_t)C.nJ + kMeshSlots, (int64_t)INT_MAX);
            C.hz = bq_clamp((int64_t)C.Jend * delta);
            C.nfar = min(C.far_cnt[C.gh & 1], mv.cap);
            C.gh_w = C.gh + 1;
            C.far_cnt[C.gh_w & 1] = 0;
            C.gs_w = C.gs + 1;  // the spill pile holds nothing live: a fresh generation
            C.sp_cnt[C.gs_w & 1] = 0;
          }
        } else if (nsp >= kMeshCompactMin && C.sdead * 2 > nsp) {
          kind = MESH_COMPACT;
          C.nsp = nsp;
          C.gs_w = C.gs + 1;
          C.sp_cnt[C.gs_w & 1] = 0;
          C.srec = INT_MAX;
          C.sdead = 0;
        } else if (jr != INT_MAX || js != INT_MAX) {
          kind = MESH_ADV;
          C.nJ = min(jr, js);
          C.win = bq_clamp(((int64_t)C.nJ + 1) * delta);
          C.nslot = min(C.rc[C.nJ & (kMeshSlots - 1)], mv.slot_cap);
          C.nsp = nsp;
          C.srec = INT_MAX;
          C.sdead = 0;
        } else if (C.far_cnt[C.gh & 1] > 0) {
          kind = MESH_HIMIN;
          C.himin = INT_MAX;
          C.nfar = min(C.far_cnt[C.gh & 1], mv.cap);
        } else {
          kind = MESH_DONE;
        }
        C.kind = kind;
        C.q_cnt[C.in ^ 1] = 0;
        C.list_cnt[0] = 0;
        C.list_cnt[1] = 0;
        C.rquit[0] = 0;
        C.rquit[1] = 0;
      }
    }
    __syncthreads();
    const int32_t kind = C.kind;
    if (kind == MESH_DONE) break;
    const int32_t in = C.in;
    MeshSink s;
    s.hz = C.hz;
    s.rc = C.rc;
    s.far = (C.gh_w & 1) ? mv.far[1] : mv.far[0];
    s.far_cnt = &C.far_cnt[C.gh_w & 1];
    s.far_tag = mesh_far_tag(C.gh_w);
    s.sp = (C.gs_w & 1) ? mv.sp[1] : mv.sp[0];
    s.sp_cnt = &C.sp_cnt[C.gs_w & 1];
    s.list = lists;
    s.list_cnt = &C.list_cnt[0];
    s.q = in ? mv.q[0] : mv.q[1];
    s.q_cnt = &C.q_cnt[in ^ 1];
    s.qtag = INT_MIN + 1 + (C.steps & 0x3fffffff);
    int32_t smin = INT_MAX;  // smallest value this thread left on a spill pile
    if (kind == MESH_HIMIN) {
      // smallest live value of the far pile (everything at or above the cutoff)
      const int32_t *pile = (C.gh & 1) ? mv.far[1] : mv.far[0];
      const int32_t nf = C.nfar, U = C.U;
      int32_t mn = INT_MAX;
      for (int32_t i0 = threadIdx.x; i0 < nf; i0 += kMeshInFlight * blockDim.x) {
        int32_t v[kMeshInFlight], p[kMeshInFlight];
#pragma unroll
        for (int j = 0; j < kMeshInFlight; ++j)
          v[j] = i0 + j * (int32_t)blockDim.x < nf ? __ldcg(pile + i0 + j * blockDim.x) : -1;
#pragma unroll
        for (int j = 0; j < kMeshInFlight; ++j) p[j] = v[j] >= 0 ? __ldcg(mv.dist + v[j]) : INT_MAX;
#pragma unroll
        for (int j = 0; j < kMeshInFlight; ++j)
          if (p[j] >= U) mn = min(mn, p[j]);
      }
      mesh_fold_min(mn, &C.himin);
      __syncthreads();
      continue;  // the next decision reads the minimum after the barrier above
    }
    if (kind == MESH_COMPACT) {
      // live spill entries (at or above the cutoff) move to a new generation
      int32_t nd = 0;
      mesh_scan<KEEP_MOVE>(mv, s, (C.gs & 1) ? mv.sp[1] : mv.sp[0], C.nsp, C.U, C.U, smin, nd);
      mesh_fold_min(smin, &C.srec);
      __syncthreads();
      continue;
    }
    if (kind == MESH_RELAX) {
      // the overflow queue of the last step: window vertices at their current distance
      s.lo = (int32_t)min((int64_t)C.J * delta, (int64_t)INT_MAX);
      s.cutoff = C.U;
      const int32_t nq = C.nq;
      const int32_t *q = in ? mv.q[1] : mv.q[0];
      for (int32_t i = threadIdx.x; i < nq; i += blockDim.x) {
        const int32_t v = __ldcg(q + i);
        const int32_t p = __ldcg(mv.dist + v), b = __ldg(mv.off + v), e = __ldg(mv.off + v + 1);
        mesh_relax(mv, s, v, p, b, e, false, smin);
      }
    } else {
      // an advance to the window [nJ delta, win): the bucket's ring slot and the
      // spill pile (MESH_ADV), or the far pile (a refill, MESH_HISPLIT)
      s.cutoff = C.win;
      const int32_t lo = (int32_t)min((int64_t)C.nJ * delta, (int64_t)INT_MAX), win = C.win;
      s.lo = lo;
      if (kind == MESH_ADV) {
        const int4 *slot = mv.ring + (int64_t)(C.nJ & (kMeshSlots - 1)) * mv.slot_cap;
        const int32_t ns = C.nslot, T = blockDim.x;
        // the first block-width of entries is relaxed by the thread that reads
        // it; the rest goes to the relax list (even shares in the first round)
        if (ns > T) mesh_scan_slot(mv, s, slot + T, ns - T);
        if ((int32_t)threadIdx.x < ns) {
          const int4 x = __ldcg(slot + threadIdx.x);
          mesh_relax(mv, s, x.x, x.y, x.z, x.w, true, smin);
        }
        if (C.nsp > 0) {
          int32_t nd = 0;
          mesh_scan<KEEP_STAY>(mv, s, (C.gs & 1) ? mv.sp[1] : mv.sp[0], C.nsp, lo, win, smin, nd);
          mesh_fold_add(nd, &C.sdead);
        }
      } else {
        int32_t nd = 0;
        mesh_scan<KEEP_SPLIT>(mv, s, (C.gh & 1) ? mv.far[1] : mv.far[0], C.nfar, lo, win, smin, nd);
      }
    }
    // relax rounds: list r is read in round r + 1, which fills list r + 1;
    // minima of spilled values are folded before every barrier
    mesh_fold_min(smin, &C.srec);
    smin = INT_MAX;
    __syncthreads();
    for (int32_t r = 1;; ++r) {
      const int32_t nl = min(C.list_cnt[(r - 1) % 3], kMeshList);
      if (nl == 0 || C.rquit[(r - 1) % 3]) break;
      if (threadIdx.x == 0) {
        C.list_cnt[(r + 1) % 3] = 0;
        C.rquit[(r + 1) % 3] = 0;
        if ((r & 63) == 0 && globaltimer_ns() > deadline) {  // the wall-clock bound holds inside a step too
          atomicOr(c.err, DEV_ERR_TIMEOUT);
          C.rquit[r % 3] = 1;  // read after this round's barrier
          C.quit = 1;
        }
      }
      const int4 *lin = lists + ((r - 1) & 1) * kMeshList;
      s.list = lists + (r & 1) * kMeshList;
      s.list_cnt = &C.list_cnt[r % 3];
      for (int32_t i = threadIdx.x; i < nl; i += blockDim.x) {
        const int4 x = lin[i];
        mesh_relax(mv, s, x.x, x.y, x.z, x.w < 0 ? ~x.w : x.w, x.w < 0, smin);
      }
      mesh_fold_min(smin, &C.srec);
      smin = INT_MAX;
      __syncthreads();
    }
  }
  if (threadIdx.x == 0) {
    atomicMax(c.stats, C.steps);
    atomicAdd(c.stats + 1, C.adv + 1);  // the reference's last advance finds no priority left
  }
}

// The relax lists take more than the default 48 KB of dynamic shared memory:
// raised once per device (a host-side attribute, so it is done before any
// stream capture of a launch).
static gg_status mesh_kernel_setup() {
  constexpr int kMaxDevices = 64;
  static std::atomic<bool> done[kMaxDevices];
  int dev = 0;
  GG_CUDA(cudaGetDevice(&dev));
  if (dev >= 0 && dev < kMaxDevices && done[dev].load(std::memory_order_acquire)) return GG_OK;
  GG_CUDA(cudaFuncSetAttribute(k_sssp_cta, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMeshSmem));
  if (dev >= 0 && dev < kMaxDevices) done[dev].store(true, std::memory_order_release);
  return GG_OK;
}

// Sources per pass: one CTA each; per source V ints of distances, V of
// stamps and a block of piles, queues and ring, within a 24 GB budget.
int32_t bsssp_cta_width(const gg_graph *g) {
  const size_t V = (size_t)std::max(g->csr.V, 1);
  const size_t per = sizeof(int32_t) * (2 * V + (size_t)mesh_block_ints((int64_t)V));
  const size_t budget = size_t(24) << 30;
  return (int32_t)std::max<size_t>(1, std::min<size_t>(kBsLanes, budget / per));
}

gg_status bsssp_cta_buffers(gg_graph *g, int32_t k, Scratch *sc, CtaBuffers *b) {
  GG_TRY(mesh_kernel_setup());  // before a batch plan captures the launch
  const size_t V = (size_t)g->csr.V;
  const size_t blk = (size_t)mesh_block_ints((int64_t)V);
  // the piles start on a 256-byte boundary: the ring inside each block is read as int4
  const size_t piles_off = (8 + (size_t)k + 2 * (size_t)k * V + 63) / 64 * 64;
  const size_t ints = piles_off + (size_t)k * blk;
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
  b->piles = p + piles_off;
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
  c.V = g->csr.V;
  c.delta = delta;
  c.err = g->d_err;
  c.stats = b.stats;
  c.loop_limit_ns = loop_timeout_ns();
  note_launch();
  k_sssp_cta_init<<<g->sm_count * 8, 256, 0, st>>>(c, k);
  GG_CUDA(cudaGetLastError());
  if (timed) GG_CUDA(cudaEventRecord(g->ev2, st));
  GG_TRY(mesh_kernel_setup());
  note_launch();
  k_sssp_cta<<<k, kMeshThreads, kMeshSmem, st>>>(c);
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
    tot += mesh_block_ints(part_begin[p + 1] - part_begin[p]);
  }
  // ints: stats 8, sources, part_lo, part_base (int64, 8-byte aligned), stamps;
  // then the blocks, on a 256-byte boundary (each block's ring is read as int4)
  const size_t base_off = (8 + 2 * (size_t)nparts + 1 + 1) & ~(size_t)1;
  const size_t stamp_off = base_off + 2 * (size_t)nparts;
  const size_t piles_off = (stamp_off + (size_t)V + 63) / 64 * 64;
  const size_t ints = piles_off + (size_t)tot;
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
  int64_t *dbase = reinterpret_cast<int64_t *>(p32 + base_off);
  int32_t *stamp = p32 + stamp_off;
  int32_t *piles = p32 + piles_off;
  int32_t *dist = nullptr;
  GG_TRY(scratch_get_app(g, 2, sizeof(int32_t) * (size_t)V, (void **)&dist));
  GG_TRY(mesh_kernel_setup());
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
  k_sssp_cta<<<nparts, kMeshThreads, kMeshSmem, st>>>(c);
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
