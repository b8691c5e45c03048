// Batched BC: up to 64 sources per pass in one persistent kernel.
//
// The per-source algorithm is apps/bc.cpp:28-123 (Brandes with the stored
// quantity dep' = (1 + delta) / sigma):
//   forward   sigma[v] = sum of sigma[u] over in-neighbours u one level up;
//   backward  dep'[v] = 1/sigma[v] + sum of dep'[u] over in-neighbours u at a
//             deeper level (bc.cpp pushes dep'[src] to unvisited out-neighbours,
//             i.e. every vertex receives from its in-neighbours that sit deeper);
//   final     delta[v] = (dep'[v] - 1/sigma[v]) * sigma[v], 0 when unreached.
//
// 64 sources share one traversal.  The levels come from the bit-parallel
// multi-source BFS of batch_bfs.cu (one edge visit serves all sources), whose
// queues are kept back to back as the level list Q_0, Q_1, ... (a vertex is in
// Q_d when some source first reaches it at level d).  Per-source values live
// vertex-major -- sigma[v][64], dep'[v][64] in fp64, depth[v][64] in uint16 --
// so the two gathers use one warp per (vertex, chunk of in-edges) work item with
// lane l owning sources l and l + 32: each in-neighbour costs one broadcast
// 8-byte mask load, and only the sources whose bit survives read the neighbour's
// 8-byte value.  A vertex of one chunk writes its own values (no atomics);
// hubs' chunks add fp64 partial sums atomically (sigma sums are integers, exact
// in any order).  dep' is accumulated in fp64 and written out as fp32.
//
// Grid barriers per level: two forward ([sigma of level d] + [relax of level
// d+1] | [publish of level d+1]) and two backward ([mask update of level d+1] +
// [scan of level d] | [gather of level d]).
#include <vector>

#include "batch.h"
#include "lb.cuh"

namespace gg {

constexpr int32_t kBcWidth = 64;         // sources per pass (mask bits)
constexpr int32_t kBcMaxLevels = 65534;  // depth is stored as uint16; 0xFFFF = unreached

struct BcState {
  uint64_t *seen, *acc, *rmask;  // rmask[v]: sources whose level at v is deeper than the current one
  uint64_t *fr[3];               // level masks, by level mod 3
  uint64_t *lm[2];               // backward: sources at v's current level, by level parity
  int32_t *qstamp;
  int32_t *lev;                  // level list
  int32_t levcap;
  int32_t *loff;                 // [kBcMaxLevels + 2] start of each level in lev
  int64_t *work;                 // (v << 32 | chunk)
  int32_t wcap;
  int32_t chunk;                 // in-edges per work item (the graph's batch tuning)
  int32_t *ctr;                  // [0] level-list end, [1..2] forward items, [3..4] backward items,
                                 // [16..19] hand-out counters, [20] end of Q_0
  uint16_t *depth;               // [V][64]
  double *sigma, *dep;           // [V][64]
  const int32_t *toff, *tsrc;    // in-neighbours (the CSR itself for a symmetric graph)
  const int32_t *perm;           // original id -> walked id (degree-ordered copy), or null
  int32_t V, nsrc;
  uint32_t *bar;
  int32_t *err;
  uint64_t timeout_ns;
  int32_t *stats;                // [0] levels
  int32_t *stop;
  uint64_t loop_limit_ns;
};

// Appends nch work items for this lane's vertex; the whole warp calls it
// together (lanes without a vertex pass nch = 0).
__device__ __forceinline__ void bc_push_items(const BcState &st, int32_t *wcnt, int32_t v, int32_t nch) {
  const int32_t lane = threadIdx.x & 31;
  int32_t incl = nch;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int32_t t = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += t;
  }
  const int32_t total = __shfl_sync(0xffffffffu, incl, 31);
  if (total == 0) return;
  int32_t base = 0;
  if (lane == 31) base = atomicAdd(wcnt, total);
  base = __shfl_sync(0xffffffffu, base, 31);
  const int32_t first = base + incl - nch;
  for (int32_t c = 0; c < nch; ++c) {
    if (first + c >= st.wcap) {
      atomicOr(st.err, DEV_ERR_OVERFLOW);
      break;
    }
    st.work[first + c] = ((int64_t)v << 32) | (uint32_t)c;
  }
}

// Selects a level array without indexing the kernel-parameter arrays
// dynamically (which would copy them to local memory).
__device__ __forceinline__ uint64_t *bc_fr(const BcState &st, int32_t level) {
  const int32_t i = level % 3;
  return i == 0 ? st.fr[0] : (i == 1 ? st.fr[1] : st.fr[2]);
}
__device__ __forceinline__ uint64_t *bc_lm(const BcState &st, int32_t level) {
  return (level & 1) ? st.lm[1] : st.lm[0];
}

__device__ __forceinline__ int32_t bc_chunks(const BcState &st, int32_t v) {
  const int32_t deg = __ldg(st.toff + v + 1) - __ldg(st.toff + v);
  return deg <= st.chunk ? 1 : (deg + st.chunk - 1) / st.chunk;
}

// Gather over one work item: lane sums, for its sources s in `own`, val[u][s]
// over in-neighbours u whose mask has s.  Returns the two partial sums.
__device__ __forceinline__ void bc_gather(const BcState &st, int32_t v, int32_t c, uint64_t own,
                                          const uint64_t *mask, const double *val, double &a0,
                                          double &a1) {
  const int32_t lane = threadIdx.x & 31;
  const int32_t kb = __ldg(st.toff + v), ke = __ldg(st.toff + v + 1);
  const int32_t k0 = kb + c * st.chunk, k1 = min(ke, k0 + st.chunk);
  a0 = 0.0;
  a1 = 0.0;
  int32_t k = k0;
  for (; k + 4 <= k1; k += 4) {
    int32_t u[4];
    uint64_t m[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) u[j] = __ldg(st.tsrc + k + j);
#pragma unroll
    for (int j = 0; j < 4; ++j) m[j] = __ldcg(mask + u[j]) & own;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (!m[j]) continue;
      const double *row = val + (int64_t)u[j] * kBcWidth;
      if ((m[j] >> lane) & 1) a0 += __ldcg(row + lane);
      if ((m[j] >> (lane + 32)) & 1) a1 += __ldcg(row + lane + 32);
    }
  }
  for (; k < k1; ++k) {
    const int32_t u = __ldg(st.tsrc + k);
    const uint64_t m = __ldcg(mask + u) & own;
    if (!m) continue;
    const double *row = val + (int64_t)u * kBcWidth;
    if ((m >> lane) & 1) a0 += __ldcg(row + lane);
    if ((m >> (lane + 32)) & 1) a1 += __ldcg(row + lane + 32);
  }
}

// Guided hand-out of a phase's work items: a warp takes a batch of up to 32
// (half of what is left, spread over the warps), so items of very different
// cost still end the phase together instead of leaving CTAs idle at the grid
// barrier.  False when none are left; [i0, i1) is the batch.
__device__ __forceinline__ bool bc_take(int32_t *wc, int32_t ni, int32_t nwarps, int32_t &i0, int32_t &i1) {
  const int32_t lane = threadIdx.x & 31;
  int32_t b = 0, B = 1;
  if (lane == 0) {
    const int32_t left = ni - *(volatile int32_t *)wc;
    const int32_t per = left > 0 ? (left / 2 + nwarps - 1) / nwarps : 1;
    B = per < 1 ? 1 : (per > 32 ? 32 : per);
    b = atomicAdd(wc, B);
  }
  b = __shfl_sync(0xffffffffu, b, 0);
  B = __shfl_sync(0xffffffffu, B, 0);
  i0 = b;
  i1 = min(b + B, ni);
  return b < ni;
}

__global__ void __launch_bounds__(512) k_bc_batch(DGraph g, BcState st) {
  extern __shared__ int4 smem[];
  const int32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int32_t nthreads = gridDim.x * blockDim.x;
  const int32_t lane = threadIdx.x & 31;
  const int32_t nwarps = nthreads >> 5;
  LoopClock clk;
  clk.start(st.loop_limit_ns);
  bool alive = true;
  int32_t d = 0;
  int32_t b_prev = 0, b_d = 0;  // starts of Q_{d-1} and Q_d in the level list
  // End of Q_d in the level list.  Not read from the list's append counter at
  // the top of an iteration: a CTA that is ahead may already be appending
  // Q_{d+1} there while another still reads it, and CTAs that disagree on a
  // level's end disagree on when the loop ends (one leaves, the others wait at
  // the next grid barrier).  Q_0's end comes from a word the seed kernel wrote
  // and nothing appends to; each later one from the publish phase, which reads
  // the counter between the barrier that ends the appends and the one after
  // which the next level's appends begin.
  int32_t e_next = *(volatile int32_t *)(st.ctr + 20);
  // ------------------------------------------------------------- forward
  for (;; ++d) {
    const int32_t e_d = e_next;
    if (e_d == b_d) break;  // Q_d is empty
    if (stopped(st.stop, d)) {
      alive = false;
      break;
    }
    if (d + 1 > kBcMaxLevels) {
      if (tid == 0) atomicOr(st.err, DEV_ERR_OVERFLOW);
      alive = false;
      break;
    }
    if (tid == 0) {
      st.loff[d] = b_d;
      st.loff[d + 1] = e_d;
      st.ctr[1 + (d & 1)] = 0;  // items of Q_{d+1}, filled by the publish below
      st.ctr[16 + ((d + 1) & 1)] = 0;  // hand-out counter of the next level's gather
    }
    // sigma of Q_d from Q_{d-1} (items made by the previous publish)
    if (d > 0) {
      const int32_t ni = min(*(volatile int32_t *)(st.ctr + 1 + ((d - 1) & 1)), st.wcap);
      const uint64_t *pm = bc_fr(st, d - 1), *nm = bc_fr(st, d);
      for (int32_t i0, i1; bc_take(st.ctr + 16 + (d & 1), ni, nwarps, i0, i1);)
      for (int32_t i = i0; i < i1; ++i) {
        const int64_t it = __ldcg(st.work + i);
        const int32_t v = (int32_t)(it >> 32), c = (int32_t)(uint32_t)it;
        const uint64_t own = __ldcg(nm + v);
        double a0, a1;
        bc_gather(st, v, c, own, pm, st.sigma, a0, a1);
        double *row = st.sigma + (int64_t)v * kBcWidth;
        const bool single = bc_chunks(st, v) == 1;
        if ((own >> lane) & 1) {
          if (single) row[lane] = a0;
          else if (a0 != 0.0) atomicAdd(row + lane, a0);
        }
        if ((own >> (lane + 32)) & 1) {
          if (single) row[lane + 32] = a1;
          else if (a1 != 0.0) atomicAdd(row + lane + 32, a1);
        }
      }
    }
    // the mask array P(d) writes next held Q_{d-2}: clear those entries
    if (d >= 2) {
      uint64_t *old = bc_fr(st, d + 1);
      for (int32_t i = __ldcg(st.loff + d - 2) + tid; i < b_prev; i += nthreads) old[__ldcg(st.lev + i)] = 0;
    }
    // relax from Q_d: acc[v] |= fr[u] & ~seen[v], Q_{d+1} appended to the list
    {
      const int32_t n = e_d - b_d;
      const Enum en{st.lev + b_d, nullptr, n};
      const UMsBfs f{st.seen, bc_fr(st, d), st.acc, st.qstamp, d + 1};
      DOut out{};
      out.mode = OUT_SPARSE;
      out.q = st.lev;
      out.cnt = st.ctr + 0;
      out.cap = st.levcap;
      out.err = st.err;
      const int32_t nv = ceil_div(n, blockDim.x / kStage1);
      for (int32_t vc = blockIdx.x; vc < nv; vc += gridDim.x)
        lb_twce<UMsBfs, true>(g, en, n, f, out, vc, *reinterpret_cast<TwceSmem *>(smem));
    }
    if (!grid_barrier(st.bar, gridDim.x, st.err, st.timeout_ns)) {
      alive = false;
      break;
    }
    // publish Q_{d+1}: masks, depths, and its sigma work items
    {
      e_next = min(*(volatile int32_t *)(st.ctr + 0), st.levcap);
      const int32_t m = e_next - e_d;
      const int32_t m_up = (m + 31) & ~31;
      uint64_t *nm = bc_fr(st, d + 1);
      for (int32_t i = tid; i < m_up; i += nthreads) {
        int32_t v = -1, nch = 0;
        if (i < m) {
          v = __ldcg(st.lev + e_d + i);
          const uint64_t a = __ldcg(st.acc + v);
          const uint64_t sv = __ldcg(st.seen + v);
          const uint64_t nb = a & ~sv;
          st.seen[v] = sv | nb;
          nm[v] = nb;
          st.acc[v] = 0;
          uint16_t *drow = st.depth + (int64_t)v * kBcWidth;
          for (uint64_t b = nb; b; b &= b - 1) drow[__ffsll((long long)b) - 1] = (uint16_t)(d + 1);
          nch = bc_chunks(st, v);
        }
        bc_push_items(st, st.ctr + 1 + (d & 1), v, nch);
      }
    }
    clk.tick(st.stop, d, st.err);
    if (!grid_barrier(st.bar, gridDim.x, st.err, st.timeout_ns)) {
      alive = false;
      break;
    }
    b_prev = b_d;
    b_d = e_d;
  }
  const int32_t L = d;  // levels 0 .. L-1 are non-empty
  if (tid == 0) st.stats[0] = L;
  // ------------------------------------------------------------ backward
  // (iterations numbered on from the forward loop's, for the loop clock)
  for (int32_t dd = L - 1, it = L + 1; alive && dd >= 0; --dd, ++it) {
    if (stopped(st.stop, it)) break;
    if (tid == 0) {
      st.ctr[3 + ((dd + 1) & 1)] = 0;   // consumed by the gather of level dd + 1
      st.ctr[18 + ((dd + 1) & 1)] = 0;  // that gather's hand-out counter
    }
    // sources at level dd + 1 become "deeper" for the gathers from here on
    if (dd + 1 < L) {
      uint64_t *lmo = bc_lm(st, dd + 1);
      const int32_t e = __ldcg(st.loff + dd + 2);
      for (int32_t i = __ldcg(st.loff + dd + 1) + tid; i < e; i += nthreads) {
        const int32_t v = __ldcg(st.lev + i);
        st.rmask[v] = __ldcg(st.rmask + v) | __ldcg(lmo + v);
        lmo[v] = 0;
      }
    }
    // scan Q_dd: which sources sit at level dd at v, and the work items
    {
      const int32_t b = __ldcg(st.loff + dd), m = __ldcg(st.loff + dd + 1) - b;
      const int32_t m_up = (m + 31) & ~31;
      uint64_t *lmn = bc_lm(st, dd);
      for (int32_t i = tid; i < m_up; i += nthreads) {
        int32_t v = -1, nch = 0;
        if (i < m) {
          v = __ldcg(st.lev + b + i);
          const uint4 *row = reinterpret_cast<const uint4 *>(st.depth + (int64_t)v * kBcWidth);
          uint64_t mk = 0;
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const uint4 q = __ldcg(row + j);
            const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
            for (int h = 0; h < 4; ++h) {
              if ((w[h] & 0xffffu) == (uint32_t)dd) mk |= 1ull << (8 * j + 2 * h);
              if ((w[h] >> 16) == (uint32_t)dd) mk |= 1ull << (8 * j + 2 * h + 1);
            }
          }
          lmn[v] = mk;
          nch = bc_chunks(st, v);
        }
        bc_push_items(st, st.ctr + 3 + (dd & 1), v, nch);
      }
    }
    if (!grid_barrier(st.bar, gridDim.x, st.err, st.timeout_ns)) break;
    // gather: dep'[v][s] = 1/sigma[v][s] + sum over deeper in-neighbours
    {
      const int32_t ni = min(*(volatile int32_t *)(st.ctr + 3 + (dd & 1)), st.wcap);
      const uint64_t *lmn = bc_lm(st, dd);
      for (int32_t i0, i1; bc_take(st.ctr + 18 + (dd & 1), ni, nwarps, i0, i1);)
      for (int32_t i = i0; i < i1; ++i) {
        const int64_t it = __ldcg(st.work + i);
        const int32_t v = (int32_t)(it >> 32), c = (int32_t)(uint32_t)it;
        const uint64_t own = __ldcg(lmn + v);
        double a0, a1;
        bc_gather(st, v, c, own, st.rmask, st.dep, a0, a1);
        const double *srow = st.sigma + (int64_t)v * kBcWidth;
        double *row = st.dep + (int64_t)v * kBcWidth;
        const bool single = bc_chunks(st, v) == 1;
        if ((own >> lane) & 1) {
          const double t = a0 + (c == 0 ? 1.0 / __ldcg(srow + lane) : 0.0);
          if (single) row[lane] = t;
          else atomicAdd(row + lane, t);
        }
        if ((own >> (lane + 32)) & 1) {
          const double t = a1 + (c == 0 ? 1.0 / __ldcg(srow + lane + 32) : 0.0);
          if (single) row[lane + 32] = t;
          else atomicAdd(row + lane + 32, t);
        }
      }
    }
    clk.tick(st.stop, it, st.err);
    if (!grid_barrier(st.bar, gridDim.x, st.err, st.timeout_ns)) break;
  }
}

// Seeds the k sources (one thread: sources are few; duplicates share a vertex).
__global__ void k_bcb_seed(BcState st, const int32_t *__restrict__ srcs) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  int32_t n = 0;
  for (int32_t s = 0; s < st.nsrc; ++s) {
    const int32_t v = st.perm ? st.perm[srcs[s]] : srcs[s];
    if (!st.seen[v]) st.lev[n++] = v;
    st.seen[v] |= 1ull << s;
    st.fr[0][v] |= 1ull << s;
    st.depth[(int64_t)v * kBcWidth + s] = 0;
    st.sigma[(int64_t)v * kBcWidth + s] = 1.0;
  }
  st.ctr[0] = n;
  st.ctr[20] = n;  // Q_0's end, read by every CTA before any appends to ctr[0]
  *st.stop = 0;
}

// delta[s][v] = (dep'[p][s] - 1/sigma[p][s]) * sigma[p][s] as fp32 rows (v an
// original id, p its walked id), via a shared-memory transpose of 32-vertex
// tiles; also sums E_r over the sources (out-degree times the number of sources
// that reached v).
__global__ void __launch_bounds__(256) k_bcb_out(BcState st, const int32_t *__restrict__ off, float *out,
                                                 int64_t out_stride, unsigned long long *reached) {
  __shared__ float tile[kBcWidth][33];
  const int32_t V = st.V;
  unsigned long long er = 0;
  for (int32_t v0 = blockIdx.x * 32; v0 < V; v0 += gridDim.x * 32) {
    for (int32_t i = threadIdx.x; i < 32 * kBcWidth; i += blockDim.x) {
      const int32_t j = i / kBcWidth, s = i % kBcWidth;
      const int32_t v = v0 + j;
      float r = 0.f;
      if (v < V) {
        const int64_t pv = st.perm ? st.perm[v] : v;
        const double sg = st.sigma[pv * kBcWidth + s];
        if (sg != 0.0) r = (float)((st.dep[pv * kBcWidth + s] - 1.0 / sg) * sg);
      }
      tile[s][j] = r;
    }
    if (threadIdx.x < 32 && v0 + (int32_t)threadIdx.x < V) {
      const int32_t v = v0 + threadIdx.x;
      const int32_t pv = st.perm ? st.perm[v] : v;
      er += (unsigned long long)__popcll(st.seen[pv]) * (unsigned long long)(off[v + 1] - off[v]);
    }
    __syncthreads();
    for (int32_t i = threadIdx.x; i < 32 * st.nsrc; i += blockDim.x) {
      const int32_t s = i / 32, j = i % 32;
      if (v0 + j < V) out[(int64_t)s * out_stride + v0 + j] = tile[s][j];
    }
    __syncthreads();
  }
  if (threadIdx.x < 32) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) er += __shfl_xor_sync(0xffffffffu, er, d);
    if (threadIdx.x == 0 && er) atomicAdd(reached, er);
  }
}

// ------------------------------------------------------------------ host
BcBuffers::~BcBuffers() {
  if (owned)
    for (void *p : {(void *)masks, (void *)ints, (void *)work, (void *)depth, (void *)vals, (void *)dsrc})
      if (p) cudaFree(p);
}

static int64_t bc_levcap(int32_t V) { return (int64_t)V * kBcWidth; }
static int64_t bc_wcap(const gg_graph *g) { return (int64_t)g->csr.V + g->csr.E / kMinChunk + 64; }
static size_t bc_int_words(int32_t V) {  // qstamp, level list, level starts, counters
  return (size_t)V + (size_t)bc_levcap(V) + (kBcMaxLevels + 2) + 32;
}

gg_status bcb_buffers(gg_graph *g, bool owned, BcBuffers *b) {
  const int32_t V = g->csr.V;
  if (bc_levcap(V) >= INT32_MAX || bc_wcap(g) >= INT32_MAX)
    return set_error(GG_ERR_UNSUPPORTED, "batched BC holds 64 level-list entries per vertex in int32: "
                                         "V = %d is too large (use gg_bc)", V);
  GG_TRY(ensure_transpose(g));
  // walk the degree-ordered copy: the rows of the most-gathered vertices share L2
  GG_TRY(ensure_relabel(g));
  if (!g->symmetric) GG_TRY(ensure_relabel_csc(g));  // its in-lists (a symmetric copy serves both)
  b->owned = owned;
  const size_t sz[6] = {sizeof(uint64_t) * 8 * (size_t)V, sizeof(int32_t) * bc_int_words(V),
                        sizeof(int64_t) * (size_t)bc_wcap(g), sizeof(uint16_t) * kBcWidth * (size_t)V,
                        sizeof(double) * 2 * kBcWidth * (size_t)V, sizeof(int32_t) * kBcWidth + 16};
  void **ptr[6] = {(void **)&b->masks, (void **)&b->ints, (void **)&b->work,
                   (void **)&b->depth, (void **)&b->vals, (void **)&b->dsrc};
  for (int i = 0; i < 6; ++i) {
    if (owned)
      GG_CUDA(cudaMalloc(ptr[i], sz[i]));
    else
      GG_TRY(scratch_get_app(g, i, sz[i], ptr[i]));
  }
  b->bytes_masks = sz[0];
  b->bytes_ints = sz[1];
  b->bytes_depth = sz[3];
  b->bytes_vals = sz[4];
  return GG_OK;
}

static BcState bcb_state(gg_graph *g, const BcBuffers &b, int32_t k) {
  const int32_t V = g->csr.V;
  const bool rel = g->rel && (g->symmetric || g->rel->csc.off);
  const GraphStore &t = rel ? (g->symmetric ? g->rel->g : g->rel->csc) : (g->csc ? *g->csc : g->csr);
  BcState S{};
  S.perm = rel ? g->rel->perm : nullptr;
  S.seen = b.masks;
  S.acc = b.masks + V;
  S.rmask = b.masks + 2 * (size_t)V;
  for (int i = 0; i < 3; ++i) S.fr[i] = b.masks + (3 + i) * (size_t)V;
  for (int i = 0; i < 2; ++i) S.lm[i] = b.masks + (6 + i) * (size_t)V;
  S.qstamp = b.ints;
  S.lev = b.ints + V;
  S.levcap = (int32_t)bc_levcap(V);
  S.loff = S.lev + S.levcap;
  S.ctr = S.loff + kBcMaxLevels + 2;
  S.stats = S.ctr + 8;
  S.stop = S.ctr + 12;
  S.work = b.work;
  S.wcap = (int32_t)bc_wcap(g);
  S.chunk = effective_tuning(g, GG_BATCH_BC, 1).chunk;
  S.depth = b.depth;
  S.sigma = b.vals;
  S.dep = b.vals + (size_t)kBcWidth * V;
  S.toff = t.off;
  S.tsrc = t.dst;
  S.V = V;
  S.nsrc = k;
  S.bar = g->d_bar;
  S.err = g->d_err;
  S.timeout_ns = barrier_timeout_ns();
  S.loop_limit_ns = loop_timeout_ns();
  return S;
}

const void *bcb_kernel() { return (const void *)k_bc_batch; }

// One pass of k <= 64 sources, stream-ordered (capturable into a CUDA graph):
// reset, seed, the persistent forward + backward kernel, then the fp32 rows
// out[s * out_stride + v] and the reached-edge count (added to *reached).
gg_status bcb_enqueue(gg_graph *g, cudaStream_t st, const BcBuffers &b, int32_t k, const int32_t *dsrc,
                      float *out, int64_t out_stride, unsigned long long *reached, int32_t *stats,
                      bool timed) {
  const BcState S0 = bcb_state(g, b, k);
  BcState S = S0;
  if (stats) S.stats = stats;
  int per_sm = 0;
  const int cta = 512;
  const size_t smem = twce_smem_bytes(cta);
  GG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bc_batch, cta, smem));
  if (per_sm < 1) return set_error(GG_ERR_UNSUPPORTED, "batched BC kernel does not fit an SM");
  GG_CUDA(cudaMemsetAsync(b.masks, 0, b.bytes_masks, st));
  GG_CUDA(cudaMemsetAsync(b.ints, 0, sizeof(int32_t) * (size_t)g->csr.V, st));            // qstamp
  GG_CUDA(cudaMemsetAsync(S.ctr, 0, sizeof(int32_t) * 32, st));                            // counters
  GG_CUDA(cudaMemsetAsync(b.depth, 0xff, b.bytes_depth, st));
  GG_CUDA(cudaMemsetAsync(b.vals, 0, b.bytes_vals, st));
  note_launch();
  k_bcb_seed<<<1, 32, 0, st>>>(S, dsrc);
  GG_CUDA(cudaMemsetAsync(S.bar, 0, sizeof(uint32_t) * 2, st));
  DGraph dg = (S0.perm != nullptr) ? g->rel->g.view() : g->csr.view();
  dg.nbuckets = 0;
  void *args[] = {&dg, &S};
  if (timed) GG_CUDA(cudaEventRecord(g->ev2, st));
  note_launch();
  const int bps = effective_tuning(g, GG_BATCH_BC, per_sm).blocks_per_sm;
  GG_CUDA(cudaLaunchCooperativeKernel((const void *)k_bc_batch, bps * g->sm_count, cta, args, smem, st));
  if (timed) GG_CUDA(cudaEventRecord(g->ev3, st));
  note_launch();
  k_bcb_out<<<g->sm_count * 8, 256, 0, st>>>(S, g->csr.off, out, out_stride, reached);
  GG_CUDA(cudaGetLastError());
  return GG_OK;
}

}  // namespace gg

using namespace gg;

// Batched BC: dep_out[s*V + v] (fp32) for nsrc sources (host or device memory).
extern "C" gg_status gg_bc_batch(gg_graph *g, const int32_t *sources, int32_t nsrc, float *dep_out,
                                 gg_stats *stats) {
  GG_CHECK_ARG(g && sources && nsrc > 0 && dep_out, "bad arguments");
  const int32_t V = g->csr.V;
  for (int32_t i = 0; i < nsrc; ++i)
    GG_CHECK_ARG(sources[i] >= 0 && sources[i] < V, "source out of range");
  if (stats) *stats = gg_stats{};
  cudaStream_t st = g->stream;
  BcBuffers b;
  GG_TRY(bcb_buffers(g, false, &b));
  float *rows = nullptr;
  GG_TRY(scratch_get_app(g, 6, sizeof(float) * (size_t)std::min(nsrc, kBcWidth) * V, (void **)&rows));
  unsigned long long *reached = reinterpret_cast<unsigned long long *>(b.dsrc + kBcWidth);
  const uint64_t l0 = launches();
  GG_CUDA(cudaMemsetAsync(reached, 0, sizeof(unsigned long long), st));
  cudaEventRecord(g->ev0, st);
  float loop_ms = 0;
  int32_t levels = 0;
  for (int32_t base = 0; base < nsrc; base += kBcWidth) {
    const int32_t k = std::min(kBcWidth, nsrc - base);
    GG_CUDA(cudaMemcpyAsync(b.dsrc, sources + base, sizeof(int32_t) * k, cudaMemcpyDefault, st));
    GG_TRY(bcb_enqueue(g, st, b, k, b.dsrc, rows, V, reached, nullptr, true));
    GG_CUDA(cudaMemcpyAsync(dep_out + (size_t)base * V, rows, sizeof(float) * (size_t)k * V, cudaMemcpyDefault, st));
    const BcState S = bcb_state(g, b, k);
    GG_CUDA(cudaMemcpyAsync(g->h_pinned + 30, S.stats, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    GG_CUDA(cudaStreamSynchronize(st));
    float ms = 0;
    cudaEventElapsedTime(&ms, g->ev2, g->ev3);
    loop_ms += ms;
    levels = std::max(levels, g->h_pinned[30]);
  }
  cudaEventRecord(g->ev1, st);
  GG_CUDA(cudaEventSynchronize(g->ev1));
  GG_TRY(check_device_error(g, "bc_batch"));
  if (stats) {
    unsigned long long er = 0;
    GG_CUDA(cudaMemcpy(&er, reached, sizeof(er), cudaMemcpyDeviceToHost));
    cudaEventElapsedTime(&stats->device_ms, g->ev0, g->ev1);
    stats->loop_ms = loop_ms;
    stats->iterations = levels;
    stats->edges_traversed = 2 * (int64_t)er;  // forward + backward sweeps, as gg_bc
    stats->fused = 1;
    stats->launches = (int32_t)(launches() - l0);
  }
  return GG_OK;
}
