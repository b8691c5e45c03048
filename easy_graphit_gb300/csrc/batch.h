// Shared declarations of the batched mode (batch_bfs.cu, batch_sssp.cu) and its
// CUDA-graph plans (batch_plan.cu).
#pragma once

#include "engine.h"

namespace gg {

constexpr int32_t kBsLanes = 32;  // sources per batched-SSSP pass (warp lanes)
constexpr int32_t kMinChunk = 32;   // smallest work-item chunk (sizes the item queues)
constexpr int32_t kMaxChunk = 4096;

// A graph's tuning of one batched app with the defaults filled in;
// blocks_per_sm capped at `fit` (CTAs of the kernel that fit one SM).
inline gg_batch_tuning effective_tuning(const gg_graph *g, int32_t app, int fit) {
  gg_batch_tuning t = g->tuning[app];
  if (t.blocks_per_sm <= 0 || t.blocks_per_sm > fit) t.blocks_per_sm = fit;
  if (t.chunk <= 0) t.chunk = 256;
  if (t.edge_parallel_max == 0) t.edge_parallel_max = 6;
  if (t.bottom_up_div == 0) t.bottom_up_div = 16;
  return t;
}
constexpr int32_t kMsBfsWidth = 64;  // sources per batched-BFS pass (mask bits)

// Relax functor of the bit-parallel multi-source BFS (batched BFS and the
// forward sweep of batched BC): acc[v] |= fr[u] & ~seen[v]; the first thread
// to touch v at this level queues it.
struct UMsBfs {
  static constexpr bool kWeight = false;
  const uint64_t *seen, *fr;
  uint64_t *acc;
  int32_t *qstamp;
  int32_t level;
  __device__ __forceinline__ bool src_ok(int32_t) const { return true; }
  __device__ __forceinline__ bool dst_ok(int32_t) const { return true; }
  __device__ __forceinline__ int32_t apply(int32_t u, int32_t v, int32_t) const {
    const uint64_t nb = __ldcg(fr + u) & ~__ldcg(seen + v);
    if (!nb) return -1;
    if ((__ldcg(acc + v) & nb) == nb) return -1;  // nothing new for acc
    atomicOr((unsigned long long *)(acc + v), (unsigned long long)nb);
    if (atomicMax(qstamp + v, level) < level) return v;
    return -1;
  }
};

// ---------------------------------------------------------- batched SSSP
struct BsState {
  int32_t *dist;              // [V][32]
  uint32_t *fr, *nacc, *far;  // [V] masks
  int32_t *qstamp;            // [V]
  int64_t *q[2];              // queue entries (u << 32 | chunk)
  int64_t *hq[2];             // further chunks of the queue's high-degree vertices
  int32_t *hcnt;              // [3] their counts (rotating)
  int64_t qcap;
  int32_t *fl[2];             // far lists
  int32_t *cnt;               // [0..2] queue counts (rotating), [3..4] far counts, [5..7] active masks
  int32_t *cur;               // [2][32] current priority per source (double-buffered)
  int32_t *gmin;              // [2][32]
  const int32_t *off, *dst, *w;
  int32_t V;
  int32_t delta;
  int32_t chunk;              // edges per queue entry
  int32_t ep_max;             // entries active for <= ep_max sources run edge-parallel
  uint32_t *bar;
  int32_t *err;
  uint64_t timeout_ns;
  int32_t *stats;             // [0] iterations, [1] advances
  int32_t *stop;              // raised by block 0 when the loop's time limit passes
  uint64_t loop_limit_ns;
  int32_t *wctr;              // [3] relax work counters (rotating)
  const int32_t *perm;        // original id -> id in the degree-ordered graph the kernel walks
  int32_t scan_div;           // a relax over >= V/scan_div queue entries marks masks without queueing (<= 0: never)
};

// Batched SSSP with a CTA per source (batch_sssp_cta.cu): buffers of a pass
// of k sources carved from one scratch allocation.
struct CtaBuffers {
  int32_t *rows = nullptr;   // [k][V] distances
  int32_t *dsrc = nullptr;   // [k]
  int32_t *stats = nullptr;  // [0] most relax steps of a source, [1] bucket advances
  int32_t *stamp = nullptr, *piles = nullptr;
  int32_t k = 0;
};
int32_t bsssp_cta_width(const gg_graph *g);
gg_status bsssp_cta_buffers(gg_graph *g, int32_t k, Scratch *sc, CtaBuffers *b);
gg_status bsssp_cta_run(gg_graph *g, cudaStream_t st, const CtaBuffers &b, int32_t *rows, int32_t k,
                        int32_t delta, bool timed);
gg_status bsssp_use_cta(gg_graph *g, bool *use);
gg_status graph_max_degree(gg_graph *g, int32_t *out);

// Device buffers of one batched-SSSP pass; `owned` buffers are freed with it,
// the others are the graph's reusable app slots.
struct BsBuffers {
  int32_t *dist = nullptr, *ints = nullptr, *out = nullptr, *dsrc = nullptr;
  uint32_t *masks = nullptr;
  int64_t *queues = nullptr;
  int64_t qcap = 0;
  bool owned = false;
  ~BsBuffers();
};
gg_status bsssp_buffers(gg_graph *g, int32_t nsrc, bool owned, BsBuffers *b);
BsState bsssp_state(gg_graph *g, const BsBuffers &b, int32_t delta);
gg_status bsssp_enqueue(gg_graph *g, cudaStream_t st, const BsState &S, const int32_t *dsrc,
                        int32_t k, int32_t *out_rows, bool timed);

// ----------------------------------------------------------- batched BFS
struct MsBfsState {
  uint64_t *seen, *acc;       // V each
  uint64_t *fr[3];            // frontier masks of level L in fr[L % 3]
  unsigned long long *actm;   // [3] OR of level L's masks (sources still expanding)
  int32_t *qstamp;            // V: last top-down level v was queued at
  int32_t *q[3];              // queue of level L in q[L % 3]
  int32_t *cnt4;              // [4] queue count of level L in cnt4[L % 4]
  const int32_t *toff, *tsrc; // in-lists, for bottom-up levels
  int32_t V;
  int32_t bu_div;             // bottom-up when the frontier holds more than V / bu_div vertices (<= 0: never)
  int32_t *depth;             // [nsrc][V] (row-major per source)
  int64_t depth_stride;       // V
  int32_t nsrc;
  uint32_t *bar;
  int32_t *err;
  uint64_t timeout_ns;
  int32_t *stats;             // [0] levels, [1] bottom-up levels
  int32_t *stop;
  uint64_t loop_limit_ns;
  // Per-level direction: the selector network's choice when `sel` is set (its
  // parameters on the device), forced when force_dir >= 0 (0 top-down, 1
  // bottom-up: runs that time each direction on every level), else bu_div.
  const float *sel;
  int32_t force_dir;
  const int32_t *off;             // out-degrees, for the frontier statistics
  int32_t E;
  unsigned long long *lstat;      // [3][4] frontier of level L in lstat[4*(L%3)]: sum deg, sum deg^2, max deg
  float *feat_log;                // [max_log][12] features of each level, or null
  unsigned long long *time_log;   // [max_log + 1] %globaltimer at the start of each level, or null
  int32_t max_log;
};

struct MsBfsBuffers {
  uint64_t *masks = nullptr;
  int32_t *ints = nullptr, *dsrc = nullptr;
  bool owned = false;
  ~MsBfsBuffers();
};
gg_status msbfs_buffers(gg_graph *g, int32_t nsrc, bool owned, MsBfsBuffers *b);
MsBfsState msbfs_state(gg_graph *g, const MsBfsBuffers &b, int32_t k, int32_t *depth_rows);
gg_status msbfs_enqueue(gg_graph *g, cudaStream_t st, const MsBfsState &S, const int32_t *dsrc,
                        bool timed);
// ------------------------------------------------------------ batched BC
// Device buffers of one batched-BC pass (64 sources); `owned` buffers are
// freed with it, the others are the graph's reusable app slots.
struct BcBuffers {
  uint64_t *masks = nullptr;
  int32_t *ints = nullptr, *dsrc = nullptr;
  int64_t *work = nullptr;
  uint16_t *depth = nullptr;
  double *vals = nullptr;
  size_t bytes_masks = 0, bytes_ints = 0, bytes_depth = 0, bytes_vals = 0;
  bool owned = false;
  ~BcBuffers();
};
gg_status bcb_buffers(gg_graph *g, bool owned, BcBuffers *b);

// The persistent kernels (for occupancy queries).
const void *bsssp_kernel();
const void *msbfs_kernel();
const void *bcb_kernel();
gg_status bcb_enqueue(gg_graph *g, cudaStream_t st, const BcBuffers &b, int32_t k, const int32_t *dsrc,
                      float *out, int64_t out_stride, unsigned long long *reached, int32_t *stats,
                      bool timed);

}  // namespace gg
