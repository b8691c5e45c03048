// Host-side state of the engine's handles and the internal interfaces between
// its translation units.
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <memory>
#include <vector>

#include "bucket_queue.cuh"
#include "common.cuh"

namespace gg {

// Device arrays of one graph representation (CSR, its transpose, or a
// dst-blocked COO copy).
struct GraphStore {
  int32_t V = 0, E = 0;
  int32_t *off = nullptr, *dst = nullptr, *w = nullptr, *src = nullptr;
  int32_t *bucket = nullptr;  // nbuckets+1 starts (blocked only)
  int32_t nbuckets = 0;
  DGraph view() const { return DGraph{V, E, off, dst, w, src, bucket, nbuckets}; }
};

// The graph renumbered by descending in-degree class (relabel.cu), with the
// maps old -> new (perm) and new -> old (inv).
struct Relabeled {
  GraphStore g;                      // renumbered CSR
  GraphStore csc;                    // renumbered in-lists (directed graphs, built on demand)
  int32_t *perm = nullptr, *inv = nullptr;
};

// Scratch arena: grows on demand, reused across calls on the same graph.
struct Scratch {
  void *p = nullptr;
  size_t bytes = 0;
};

}  // namespace gg

struct gg_graph {
  gg::GraphStore csr;                        // forward CSR (+ COO src)
  std::unique_ptr<gg::GraphStore> csc;       // get_transposed_graph()
  std::map<int32_t, gg::GraphStore> blocked_fwd, blocked_rev;  // get_blocked_graph()
  std::unique_ptr<gg::Relabeled> rel;        // degree-ordered copy for the batched kernels
  bool symmetric = false;
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  int32_t *d_err = nullptr;       // device status word (DEV_ERR_*)
  uint32_t *d_bar = nullptr;      // grid barrier state [2]
  int32_t *d_misc = nullptr;      // small device scratch (counters, flags), 64 ints
  int32_t *h_pinned = nullptr;    // pinned host scratch, 64 ints
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;  // whole trial
  cudaEvent_t ev2 = nullptr, ev3 = nullptr;  // traversal loop
  bool loop_timed = false;                   // ev2/ev3 bracket the last loop
  int sm_count = 0;
  int device = 0;
  gg::Scratch scratch[4];         // LB scratch (TWC bins, STRICT sums, ETWC chunks)
  gg::Scratch app[8];             // per-app vertex arrays, reused across calls
  gg_frontier *app_frontier = nullptr;
  gg_pq *app_pq = nullptr;
  gg_frontier_list *app_list = nullptr;
  gg_batch_tuning tuning[3] = {};  // batched BFS, SSSP, BC launch shapes (0 = default)
  const gg_selector *batch_selector[3] = {};  // learned per-level choices of the batched kernels
  gg::Scratch bq_cta;             // batched SSSP with a CTA per source
  int32_t max_degree = -1;        // largest out-degree (-1: not computed yet)
};

struct gg_frontier {
  gg_graph *g = nullptr;
  int32_t V = 0;
  int64_t cap = 0;                 // sparse queue capacity (6*V, FRONTIER_MULTIPLIER)
  int32_t *q_in = nullptr, *q_out = nullptr;
  int32_t *cnt = nullptr;          // device [2]
  int32_t *cnt_in = nullptr, *cnt_out = nullptr;
  uint32_t *bm_in = nullptr, *bm_out = nullptr;
  int32_t nwords = 0;
  uint8_t *by_in = nullptr, *by_out = nullptr;
  int32_t bytes_padded = 0;
  int32_t *dedup = nullptr;
  int32_t epoch = 0;               // curr_dedup_counter
  int32_t fmt = GG_FMT_SPARSE;     // format_ready
  bool owned_by_pq = false;
};

struct gg_pq {
  gg_graph *g = nullptr;
  int32_t *prio = nullptr;         // device priorities (not owned)
  int32_t delta = 1;
  int64_t cur = 0;                 // current_priority_
  int64_t window_upper = 0;
  bool ready_set_dequeued = false;
  gg_frontier *frontier = nullptr; // frontier_
  int64_t advances = 0;
  gg::BqBuffers bq;                // far piles (bucket_queue.cuh), also used by the fused loop
  int32_t gen_lo = 0, gen_hi = 0;  // pile generations of the host-driven queue
  int32_t horizon = INT_MAX;
  int32_t width = 16;              // horizon width in buckets
};

struct gg_frontier_list {
  gg_graph *g = nullptr;
  int32_t *vertices = nullptr;     // V
  std::vector<int32_t> level_start{0};  // host copy of level_indices
};

namespace gg {

// Device copies of the vertex-data pointers (gg_vertex_data without host-only
// fields), passed to kernels.
struct VData {
  int32_t *parent, *depth, *dist, *ids, *updates;
  float *old_rank, *new_rank, *contrib;
  double *num_paths;
  float *dependences;
  double *dep64;  // gg_bc: dependencies accumulated in fp64, stored to dependences at the end
  uint8_t *visited;
  int32_t level, src;
  float damping;
  DFar far;  // far piles of the delta-stepping queue (read by the relax UDF only)
};
VData to_vdata(const gg_vertex_data *vd);

// ---- graph.cu
// Stream-ordered device allocation from the library's own memory pool (one
// per device).  The pool keeps freed memory for reuse instead of handing it
// back to the driver at every synchronisation, so a graph or batch created
// after another one was released maps no new pages; gg_memory_trim returns it.
cudaError_t dev_alloc(void **p, size_t bytes, cudaStream_t st);
template <typename T>
inline cudaError_t dev_alloc(T **p, size_t bytes, cudaStream_t st) {
  return dev_alloc(reinterpret_cast<void **>(p), bytes, st);
}
gg_status ensure_transpose(gg_graph *g);
gg_status ensure_coo(GraphStore &s, cudaStream_t st);
gg_status ensure_blocked(gg_graph *g, bool reverse, int32_t block_size, const GraphStore **out);
gg_status check_device_error(gg_graph *g, const char *what);
gg_status scratch_get(gg_graph *g, int slot, size_t bytes, void **p);
gg_status scratch_get_app(gg_graph *g, int slot, size_t bytes, void **p);
// stats->vertices_reached / edges_traversed of a result array (reached: >= 0
// and != INT_MAX).
gg_status app_reach_stats(gg_graph *g, const int32_t *val, gg_stats *st);
int resident_grid(const void *kernel, int cta, size_t smem, int sm_count);

// ---- cc_uf.cu
gg_status cc_union_find(gg_graph *g, int32_t *labels, int32_t *parent);

// ---- relabel.cu
gg_status ensure_relabel(gg_graph *g);
gg_status ensure_relabel_csc(gg_graph *g);  // rel->csc for directed graphs (after ensure_relabel)
void free_relabel(gg_graph *g);

// ---- pagerank.cu
gg_status pagerank_pull_twc(gg_graph *g, int32_t iters, float damping, float *rank, float *contrib2);

// ---- frontier.cu
gg_status frontier_prepare_sparse(gg_frontier *f);
gg_status frontier_prepare_bitmap(gg_frontier *f);
gg_status frontier_prepare_boolmap(gg_frontier *f);
gg_status frontier_swap(gg_frontier *f, int32_t creation);   // after apply_modified
gg_status frontier_size(gg_frontier *f, int32_t *n);
gg_status frontier_reset_out(gg_frontier *f, int32_t creation);
DIn frontier_in_view(const gg_frontier *f);
DOut frontier_out_view(gg_frontier *f, int32_t creation, bool dedup);
gg_status reverse_frontier(gg_graph *g, int32_t filter, const VData &vd, int32_t **q, int32_t **cnt);
gg_status frontier_dedup(gg_frontier *f);


// ---- edgeset dispatch (one instantiation set per UDF)
struct EdgeLaunch {
  DGraph g;          // graph to traverse (forward or transposed / blocked)
  Enum en;           // enumerated vertices
  int32_t n_host;    // host-known count for grid sizing (-1 if unknown)
  DIn in_src, in_dst;
  bool pull;
  bool filter;       // to() filter active
  DOut out;
  VData vd;
  int32_t prio_cutoff;
  int32_t lb;
  int32_t cta;
  int32_t max_cta;
  bool edge_only_all; // EDGE_ONLY: iterate all edges (blocked or not)
  gg_graph *graph;   // for scratch, stream, sm count
};
gg_status launch_bfs(const EdgeLaunch &L);
gg_status launch_sssp(const EdgeLaunch &L);
gg_status launch_pr(const EdgeLaunch &L);
gg_status launch_cc(const EdgeLaunch &L);
gg_status launch_bcf(const EdgeLaunch &L);
gg_status launch_bcb(const EdgeLaunch &L);

gg_status edgeset_apply_impl(gg_graph *g, const gg_schedule *s, int32_t udf, int32_t filter,
                             gg_frontier *from, gg_frontier *out, bool allow_dupes,
                             const VData &vd, int32_t prio_cutoff, bool on_device_dedup);
gg_status vertexset_apply_impl(gg_graph *g, gg_frontier *set, int32_t vudf, const VData &vd);

// ---- pq.cu
gg_status pq_finished(gg_pq *pq, bool *fin);
gg_status pq_dequeue(gg_pq *pq);
gg_status pq_reset(gg_pq *pq, int32_t init_priority, int32_t delta, int32_t src);
int32_t pq_cutoff(const gg_pq *pq);
DFar pq_far(const gg_pq *pq);  // far piles the relax parks into

// ---- fused.cu: whole-loop persistent kernels (fuse_kernel, operators.cpp:652-672).
// *ran is false when the schedule has no device-side form (the caller then
// runs the loop unfused).
bool fused_supported(const gg_schedule *s);
// Multi-source BFS (depth, parent scratch) or SSSP (dist) with the TWCE fused
// loop, every step on the device (capturable); sources in device memory.
// SSSP uses the bucket-queue buffers *bq; *stats receives the device address of
// the run's {iterations, bucket advances}.
gg_status fused_multi_enqueue(gg_graph *g, cudaStream_t st, bool sssp, const int32_t *dsrc, int32_t n,
                              int32_t delta, int32_t *parent, int32_t *out, const BqBuffers *bq,
                              const int32_t **stats);
gg_status fused_bfs(gg_graph *g, const gg_schedule *s, int32_t n0, const VData &vd,
                    gg_frontier *f, int32_t *iters, bool *ran);
// Direction-optimising fused BFS (fused.cu k_bfs_do): each level pushes with
// `push` (a fused-supported LB) or pulls over the in-lists, as `mode` decides
// on the device -- the hybrid rule (pull when the frontier is small iff
// small_pull; small = n <= threshold * V), the selector's direction head, or a
// forced direction.  Optional logs: features of level l (feat_log[l][12]) and
// the start time of each level plus the end time (time_log, max_log + 1).
enum : int32_t { DO_RULE = 0, DO_SELECTOR = 1, DO_FORCE_PUSH = 2, DO_FORCE_PULL = 3 };
constexpr int kBfsDoMaxCta = 512;  // the loop is compiled for CTAs of at most 512 threads, 4 per SM
struct BfsDoPlan {
  const gg_schedule *push = nullptr;
  int32_t mode = DO_RULE;
  float threshold = 0.f;
  int32_t small_pull = 0;
  const gg_selector *sel = nullptr;
  float *feat_log = nullptr;
  unsigned long long *time_log = nullptr;
  int32_t max_log = 0;
};
gg_status fused_bfs_do(gg_graph *g, const BfsDoPlan &p, int32_t n0, const VData &vd, gg_frontier *f,
                       int32_t *iters, int32_t *pulls);
gg_status fused_sssp(gg_graph *g, const gg_schedule *s, int32_t n0, int32_t delta, const VData &vd,
                     gg_pq *pq, int32_t *iters, int64_t *advances, bool *ran);
// Bucket-queue buffers for V vertices (pool memory on the graph's stream), their
// release, and the reset at the start of a run with n0 sources on the frontier.
gg_status bq_alloc(gg_graph *g, BqBuffers *b);
void bq_free(gg_graph *g, BqBuffers *b);
gg_status bq_start(const BqBuffers &b, int32_t n0, cudaStream_t st);
uint64_t barrier_timeout_ns();
uint64_t loop_timeout_ns();  // wall-clock bound of one persistent loop (GG_LOOP_TIMEOUT_MS)

}  // namespace gg
