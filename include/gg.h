/*
 * gg.h -- C ABI of libgg.so, the GB300 (sm_103a) edge-traversal engine that
 * stands in for GraphIt's GPU runtime (easy_graphit `runtime/gpu_intrinsics.h`
 * and the `runtime/infra_gpu/` headers) behind the GraphIt operator/schedule API
 * (`include/graphit/operators.h`, `include/graphit/schedule.h`).
 *
 * Conventions (reference behaviour -> this ABI):
 *  - The reference reports errors with exit(-1)/assert (support.h:4-10,
 *    graph.h:251-253, operators.cpp:543,646).  Every entry point here returns a
 *    gg_status instead; gg_last_error() gives the message of the calling thread.
 *  - The reference owns all device memory (cudaMalloc, never freed).  Here each
 *    handle owns its device memory and releases it in its *_destroy call.  Input
 *    pointers may be host or device memory (copied with cudaMemcpyDefault); the
 *    caller keeps ownership of what it passes.
 *  - The reference runs one host thread on the default stream with synchronous
 *    copies.  Here every gg_graph is bound to one CUDA stream (gg_graph_set_stream)
 *    and is not thread-safe; different graphs may be driven from different threads.
 *  - Device-side waits (grid barriers of fused kernels) are bounded; a wait that
 *    gives up returns GG_ERR_TIMEOUT and leaves the CUDA context usable.
 */
#ifndef GG_H
#define GG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
typedef enum gg_status {
  GG_OK = 0,
  GG_ERR_INVALID = 1,     /* bad argument (reference: assert)                      */
  GG_ERR_CUDA = 2,        /* CUDA runtime error (reference: cudaCheckLastError)    */
  GG_ERR_OOM = 3,         /* device or host allocation failed                      */
  GG_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up                    */
  GG_ERR_OVERFLOW = 5,    /* frontier queue capacity exceeded                      */
  GG_ERR_UNSUPPORTED = 6, /* schedule not supported (reference: assert, ops.cpp:646) */
  GG_ERR_IO = 7,          /* graph file missing / truncated / corrupt              */
  GG_ERR_STATE = 8        /* call out of order (e.g. frontier list popped empty)   */
} gg_status;

/* Copies the calling thread's last error message into buf (always
 * NUL-terminated when n > 0) and returns its full length. */
size_t gg_last_error(char *buf, size_t n);
/* Library version string. */
const char *gg_version(void);

/* ---------------------------------------------------------------- schedule
 * POD mirror of graphit::SimpleGPUSchedule (include/graphit/schedule.h:26-118).
 * Enumerator values follow the reference enum order (schedule.h:30-71);
 * GG_LB_ETWC is new (the reference has no ETWC). */
enum { GG_PUSH = 0, GG_PULL = 1 };                         /* direction_type          */
enum { GG_PULL_BITMAP = 0, GG_PULL_BOOLMAP = 1 };          /* pull_frontier_rep_type  */
enum { GG_FC_SPARSE = 0, GG_FC_BITMAP = 1, GG_FC_BOOLMAP = 2 }; /* frontier_creation_type */
enum { GG_DEDUP_DISABLED = 0, GG_DEDUP_ENABLED = 1 };      /* deduplication_type      */
enum { GG_DEDUP_FUSED = 0, GG_DEDUP_UNFUSED = 1 };         /* deduplication_strategy  */
enum {                                                     /* load_balancing_type     */
  GG_LB_VERTEX_BASED = 0, GG_LB_TWC = 1, GG_LB_TWCE = 2, GG_LB_WM = 3,
  GG_LB_CM = 4, GG_LB_STRICT = 5, GG_LB_EDGE_ONLY = 6, GG_LB_ETWC = 7
};
enum { GG_BLOCKED = 0, GG_UNBLOCKED = 1 };                 /* edge_blocking_type      */
enum { GG_FUSION_DISABLED = 0, GG_FUSION_ENABLED = 1 };    /* kernel_fusion_type      */

typedef struct gg_schedule {
  int32_t direction;
  int32_t pull_frontier_rep;
  int32_t frontier_creation;
  int32_t deduplication;
  int32_t deduplication_strategy;
  int32_t load_balancing;
  int32_t edge_blocking;
  int32_t block_size;
  int32_t kernel_fusion;
  int32_t max_cta;   /* reference default 60  (schedule.cpp:6) */
  int32_t cta_size;  /* reference default 512 (schedule.cpp:5) */
} gg_schedule;

/* Fills *s like the SimpleGPUSchedule() constructor (schedule.h:87-97):
 * PUSH, VERTEX_BASED, UNBLOCKED, SPARSE creation, BOOLMAP pull rep,
 * block_size -1, max_cta/cta_size from the process defaults. */
void gg_schedule_init(gg_schedule *s);
/* SimpleGPUSchedule::default_max_cta / default_cta_size (schedule.cpp:5-6). */
void gg_set_default_launch(int32_t max_cta, int32_t cta_size);

/* App-level schedule: a SimpleGPUSchedule, a HybridGPUSchedule(s1, s2) with its
 * runtime threshold (schedule.h:122-139; "use s1 when |frontier| <= t*V",
 * operators.cpp:526), or a learned selector with the simple schedule as its
 * fallback.  `fuse` is the app's fuse_kernel(to_fuse, ...) flag
 * (operators.cpp:652-672). */
enum { GG_SCHED_SIMPLE = 0, GG_SCHED_HYBRID = 1, GG_SCHED_LEARNED = 2 };
struct gg_selector;
typedef struct gg_app_schedule {
  int32_t kind;
  int32_t fuse;
  float threshold;
  gg_schedule s1;
  gg_schedule s2;
  const struct gg_selector *selector;
} gg_app_schedule;

/* ------------------------------------------------------------- host graphs
 * Host-side CSR (int32 offsets[V+1], dst[E], weights[E]), built like GAPBS's
 * BuilderBase::MakeGraph + SquishGraph (runtime/infra_gapbs/builder.h:165-246):
 * neighbour lists sorted ascending, duplicate edges merged keeping the smallest
 * weight, self-loops removed. */
typedef struct gg_host_graph gg_host_graph;

/* R-MAT edge list with the Graph500 bit recursion and GAPBS's per-2^18-edge
 * reseeding, id permutation and U[wmin,wmax] weights
 * (runtime/infra_gapbs/generator.h:45-55,74-107,125-139).  a,b,c are the
 * quadrant probabilities (0.57/0.19/0.19 in the reference); seed 27491095 is
 * GAPBS's kRandSeed (util.h:22). */
gg_status gg_host_graph_rmat(int32_t scale, int32_t degree, float a, float b,
                             float c, int64_t seed, int32_t symmetrize,
                             int32_t wmin, int32_t wmax, gg_host_graph **out);
/* rows x cols 4-neighbour grid, every edge directed both ways, each directed
 * edge weighted U[wmin,wmax] (project-defined generator; no reference one). */
gg_status gg_host_graph_grid(int32_t rows, int32_t cols, int64_t seed,
                             int32_t wmin, int32_t wmax, gg_host_graph **out);
/* Builds a squished CSR from an edge list (u[i] -> v[i], weight w[i] or 1). */
gg_status gg_host_graph_from_edges(int32_t num_vertices, int64_t num_edges,
                                   const int32_t *u, const int32_t *v,
                                   const int32_t *w, int32_t symmetrize,
                                   gg_host_graph **out);
/* Wraps a copy of an existing CSR (no squish). */
gg_status gg_host_graph_from_csr(int32_t num_vertices, int64_t num_edges,
                                 const int32_t *offsets, const int32_t *dst,
                                 const int32_t *weights, gg_host_graph **out);
/* Loads .graphit_bin (graph.h:255-270), .el / .wel text edge lists
 * (infra_gapbs/reader.h:55-100), .gr (DIMACS), .mtx (MatrixMarket), or a GAPBS
 * serialized graph .sg / .wsg (reader.h:322-369; the stored out-lists are
 * taken as they are, symmetrize is ignored). */
gg_status gg_host_graph_load(const char *path, int32_t symmetrize,
                             gg_host_graph **out);
/* Writes a GAPBS serialized graph (writer.h:39-70): .sg (ids only) or .wsg
 * (id, weight pairs) by the path's suffix; `directed` also stores the
 * in-lists, as GAPBS does for a directed graph. */
gg_status gg_host_graph_save_sg(const gg_host_graph *g, const char *path,
                                int32_t directed);
/* Writes the .graphit_bin cache format of graph.h:295-302:
 * [i32 V][i32 E][i32 src[E]][i32 dst[E]][i32 w[E]][i32 offsets[V+1]]. */
gg_status gg_host_graph_save_bin(const gg_host_graph *g, const char *path);
gg_status gg_host_graph_info(const gg_host_graph *g, int32_t *num_vertices,
                             int64_t *num_edges);
/* Disjoint union of n host graphs (part i's vertex v becomes
 * vertex_offsets[i] + v; vertex_offsets may be NULL, else n+1 entries).  Used
 * to run many graphs of uneven size in one traversal (gg_bfs_multi /
 * gg_sssp_multi with one source per part). */
gg_status gg_host_graph_union(const gg_host_graph *const *parts, int32_t n,
                              int32_t *vertex_offsets, gg_host_graph **out);
/* n sources as GAPBS's SourcePicker draws them (infra_gapbs/benchmark.h:50-71):
 * uniform ids from std::mt19937(seed), skipping vertices with no out-edges. */
gg_status gg_host_graph_pick_sources(const gg_host_graph *g, int32_t n,
                                     int64_t seed, int32_t *out);
/* The batched mode's mix of uneven graphs (no reference counterpart): count
 * graphs drawn from std::mt19937(seed), each a 2-D grid with probability 1/4
 * (side 256, 512, 1024 or 2048) or else an R-MAT graph with scale in [12, 20]
 * and edge factor in [4, 32].  spec[i] = {0 R-MAT | 1 grid, scale | side,
 * edge factor | 0}; graph i is generated with seed + 1 + i. */
gg_status gg_host_graph_mix_spec(int64_t seed, int32_t count, int32_t *spec);
const int32_t *gg_host_graph_offsets(const gg_host_graph *g);
const int32_t *gg_host_graph_dst(const gg_host_graph *g);
const int32_t *gg_host_graph_weights(const gg_host_graph *g);
void gg_host_graph_destroy(gg_host_graph *g);

/* ----------------------------------------------------------- device graphs
 * graphit_runtime::GraphT<int> (runtime/infra_gpu/graph.h:17-88) resident in
 * HBM.  load_graph's H2D upload (graph.h:310-320) is gg_graph_create;
 * get_transposed_graph (graph.h:165-234) and get_blocked_graph
 * (graph.h:105-163) run on the GPU here and are cached in the handle. */
typedef struct gg_graph gg_graph;
/* GG_GRAPH_SYMMETRIC promises that every edge (u, v, w) has its reverse
 * (v, u, w) with the same weight: the graph is then its own transpose and
 * pull schedules use it as such. */
enum { GG_GRAPH_SYMMETRIC = 1 };
gg_status gg_graph_create(const int32_t *offsets, const int32_t *dst,
                          const int32_t *weights, int32_t num_vertices,
                          int64_t num_edges, uint32_t flags, gg_graph **out);
/* Frontiers, priority queues, frontier lists and batch plans made on g hold
 * pointers into it: destroy them before the graph. */
gg_status gg_graph_destroy(gg_graph *g);
gg_status gg_graph_info(const gg_graph *g, int32_t *num_vertices,
                        int64_t *num_edges);
/* Binds the graph (and everything run on it) to a CUDA stream (cudaStream_t).
 * NULL selects the library's own non-blocking stream. */
gg_status gg_graph_set_stream(gg_graph *g, void *stream);
gg_status gg_graph_sync(gg_graph *g);
gg_status gg_graph_transpose(gg_graph *g);
gg_status gg_graph_blocked(gg_graph *g, int32_t block_size);
gg_status gg_graph_device_arrays(const gg_graph *g, const int32_t **offsets,
                                 const int32_t **dst, const int32_t **weights);

/* -------------------------------------------------------------- frontiers
 * graphit_runtime::VertexFrontier (= vertexsubset, vertex_frontier.h:26-166):
 * double-buffered sparse queues (capacity 6*V, FRONTIER_MULTIPLIER), bitmaps
 * (uint32 words), boolmaps (bytes), dedup counters and device counts. */
typedef struct gg_frontier gg_frontier;
enum { GG_FMT_SPARSE = 0, GG_FMT_BITMAP = 1, GG_FMT_BOOLMAP = 2 };
gg_status gg_frontier_create(gg_graph *g, int32_t init_all, gg_frontier **out);
gg_status gg_frontier_destroy(gg_frontier *f);
gg_status gg_frontier_add(gg_frontier *f, int32_t v);          /* addVertex   */
gg_status gg_frontier_size(gg_frontier *f, int32_t *n);        /* size_host   */
gg_status gg_frontier_clear(gg_frontier *f);
gg_status gg_frontier_format(const gg_frontier *f, int32_t *fmt);
gg_status gg_frontier_to_sparse(gg_frontier *f);               /* to_sparse_host */
gg_status gg_frontier_to_bitmap(gg_frontier *f);               /* to_bitmap   */
gg_status gg_frontier_to_boolmap(gg_frontier *f);              /* to_boolmap  */
gg_status gg_frontier_dedup(gg_frontier *f);                   /* dedup_frontier_perfect */
/* Copies the members (in ascending vertex order) into out (host or device
 * memory, capacity cap); *n receives the member count. */
gg_status gg_frontier_read(gg_frontier *f, int32_t *out, int32_t cap,
                           int32_t *n);

/* ------------------------------------------------------------ vertex data
 * The VertexData<T> arrays the apps' UDFs touch (the apps/ sources), as device
 * pointers.  Unused members may be NULL. */
typedef struct gg_vertex_data {
  int32_t *parent;      /* bfs.cpp:19            (-1 = unvisited)        */
  int32_t *depth;       /* BFS level, written with parent (optional)     */
  int32_t *dist;        /* sssp.cpp:20 SP         (INT_MAX = unreached)  */
  int32_t *ids;         /* cc.cpp:18 ID                                  */
  int32_t *updates;     /* cc.cpp:21 update[2]                           */
  float *old_rank;      /* pr.cpp:19                                     */
  float *new_rank;      /* pr.cpp:20                                     */
  float *contrib;       /* pr.cpp:21                                     */
  double *num_paths;    /* bc.cpp:20                                     */
  float *dependences;   /* bc.cpp:21                                     */
  uint8_t *visited;     /* bc.cpp:22                                     */
  int32_t level;        /* BFS level written into depth                  */
  int32_t src;          /* source vertex for the reset UDFs              */
  float damping;        /* pr.cpp:23                                     */
} gg_vertex_data;

/* Edge UDFs of the five apps and their to() filters. */
enum {
  GG_UDF_BFS_PARENT = 0,  /* bfs.cpp:23-25  parent[dst]=src  (CAS, graphit.cpp:96-111) */
  GG_UDF_SSSP_RELAX = 1,  /* sssp.cpp:24-27 pq.updatePriorityMin(dst, SP[src]+w)      */
  GG_UDF_PR_ADD = 2,      /* pr.cpp:32-34   new_rank[dst] += contrib[src]             */
  GG_UDF_CC_HOOK = 3,     /* cc.cpp:23-36                                              */
  GG_UDF_BC_FORWARD = 4,  /* bc.cpp:34-36   num_paths[dst] += num_paths[src]          */
  GG_UDF_BC_BACKWARD = 5  /* bc.cpp:52-54   dependences[dst] += dependences[src]      */
};
enum {
  GG_FILTER_NONE = 0,
  GG_FILTER_PARENT_UNSET = 1, /* bfs.cpp:27-29 parent[v] == -1    */
  GG_FILTER_UNVISITED = 2     /* bc.cpp:38-40  visited[v] == false */
};
/* Vertex UDFs of the five apps (vertexset_apply, operators.cpp:10-65). */
enum {
  GG_VUDF_BFS_RESET = 0,         /* bfs.cpp:31-33 (+ parent[src]=src)     */
  GG_VUDF_SSSP_RESET = 1,        /* sssp.cpp:29-31 (+ SP[src]=0)          */
  GG_VUDF_PR_RESET = 2,          /* pr.cpp:43-46                          */
  GG_VUDF_PR_CONTRIB = 3,        /* pr.cpp:28-30                          */
  GG_VUDF_PR_UPDATE = 4,         /* pr.cpp:36-41                          */
  GG_VUDF_CC_INIT = 5,           /* cc.cpp:37-39                          */
  GG_VUDF_CC_PJUMP = 6,          /* cc.cpp:41-49                          */
  GG_VUDF_BC_RESET = 7,          /* bc.cpp:28-32                          */
  GG_VUDF_BC_MARK_VISITED = 8,   /* bc.cpp:42-44                          */
  GG_VUDF_BC_MARK_UNVISITED = 9, /* bc.cpp:45-47                          */
  GG_VUDF_BC_BACKWARD_VERTEX = 10, /* bc.cpp:48-51                        */
  GG_VUDF_BC_FINAL = 11          /* bc.cpp:56-61                          */
};

/* edgeset_apply(s).from(from).to(filter).apply(g, udf)            (from != NULL, out == NULL)
 * edgeset_apply(s).from(from).to(filter).apply_modified(g, out, tracked, udf, allow_dupes)
 *                                                                  (out != NULL)
 * from == NULL enumerates every vertex (operators.cpp:551-556,583-590).
 * Implements the dispatch of operators.cpp:513-650 and operators.h:105-173. */
gg_status gg_edgeset_apply(gg_graph *g, const gg_schedule *s, int32_t udf,
                           int32_t to_filter, gg_frontier *from,
                           gg_frontier *out, int32_t allow_dupes,
                           const gg_vertex_data *vd);
/* vertexset_apply(set, udf); set == NULL applies to every vertex. */
gg_status gg_vertexset_apply(gg_graph *g, gg_frontier *set, int32_t vudf,
                             const gg_vertex_data *vd);

/* --------------------------------------------------- delta-stepping queue
 * graphit_runtime::GPUPriorityQueue<int> (gpu_priority_queue.h:21-247) and
 * PriorityQueue::updatePriorityMin (graphit_types.h:426-430). */
typedef struct gg_pq gg_pq;
gg_status gg_pq_create(gg_graph *g, int32_t *priorities, int32_t init_priority,
                       int32_t delta, int32_t src, gg_pq **out);
gg_status gg_pq_destroy(gg_pq *pq);
gg_status gg_pq_finished(gg_pq *pq, int32_t *finished);
/* dequeue(): returns the queue's frontier (owned by the queue: released by
 * gg_pq_destroy; gg_frontier_destroy refuses it with GG_ERR_STATE). */
gg_status gg_pq_dequeue(gg_pq *pq, gg_frontier **frontier);
/* edgeset_apply(s).from(pq frontier).apply_priority(g, relax, pq)
 * (operators.h:73-103). */
gg_status gg_edgeset_apply_priority(gg_graph *g, const gg_schedule *s,
                                    gg_pq *pq, const gg_vertex_data *vd);

/* ------------------------------------------------------------ frontier list
 * graphit_runtime::VertexFrontierList (list.h:18-116), the BC level stack. */
typedef struct gg_frontier_list gg_frontier_list;
gg_status gg_frontier_list_create(gg_graph *g, gg_frontier_list **out);
gg_status gg_frontier_list_destroy(gg_frontier_list *l);
gg_status gg_frontier_list_insert(gg_frontier_list *l, gg_frontier *f);
gg_status gg_frontier_list_retrieve(gg_frontier_list *l, gg_frontier *f);

/* --------------------------------------------------------------- whole apps
 * The testcase() bodies of apps/bfs.cpp, sssp.cpp, pr.cpp, cc.cpp, bc.cpp
 * for one trial.  Output pointers may be host or device memory. */
typedef struct gg_stats {
  int32_t iterations;       /* frontier iterations (BFS levels, SSSP rounds, ...) */
  int32_t push_iterations;  /* iterations run with a PUSH schedule                 */
  int32_t pull_iterations;  /* iterations run with a PULL schedule                 */
  int32_t bucket_advances;  /* SSSP: priority-queue bucket advances                */
  int64_t vertices_reached;
  int64_t edges_traversed;  /* algorithmic edges: sum of out-degree of reached v   */
  float device_ms;          /* CUDA-event time of the trial on the graph's stream  */
  float loop_ms;            /* CUDA-event time of the traversal loop alone (the
                               fused kernel, or the unfused iterations)            */
  int32_t fused;            /* 1 when the loop ran as one persistent kernel        */
  int32_t launches;         /* kernels this call launched                           */
} gg_stats;

/* Number of kernels libgg.so has launched in this process. */
uint64_t gg_kernel_launches(void);

/* Device memory released by graphs, frontiers and batches stays in the
 * library's stream-ordered pool for reuse (a new graph maps no new pages).
 * gg_memory_trim hands the unused part back to the driver, keeping at most
 * keep_bytes reserved per device. */
gg_status gg_memory_trim(size_t keep_bytes);

/* BFS from src: depth_out[v] = hop distance (-1 unreached); parent_out (may be
 * NULL) = the parent array of bfs.cpp (parent[src] = src).
 * With fuse = 1, a hybrid schedule of one push schedule (VERTEX_BASED, TWCE,
 * CM or WM, SPARSE creation) and one PULL schedule, or a learned schedule with
 * a selector, runs as ONE persistent kernel that picks each level's direction
 * on the device: the hybrid rule of operators.cpp:516-532, or the network's
 * direction head on the frontier statistics (no host round trip per level;
 * the reference runs bfs.cpp's hybrid "power" schedule unfused).  Pull levels
 * scan the in-lists of unvisited vertices, stopping at the first in-neighbour
 * on the previous level.  Depths are the same whatever the directions;
 * parents are a valid BFS tree. */
gg_status gg_bfs(gg_graph *g, const gg_app_schedule *s, int32_t src,
                 int32_t *depth_out, int32_t *parent_out, gg_stats *stats);
/* Training data of that loop's direction (no reference counterpart): BFS from
 * src with every level pushed (PUSH TWCE), then every level pulled, twice
 * each.  feats[l][12] = the selector's features of level l; times[l][2] = its
 * best time in ms (push, pull); *nrows = levels recorded (at most max_rows). */
gg_status gg_bfs_collect_directions(gg_graph *g, int32_t src, int32_t max_rows,
                                    float *feats, float *times, int32_t *nrows);
/* Delta-stepping SSSP from src: dist_out[v] (INT_MAX unreached). */
gg_status gg_sssp(gg_graph *g, const gg_app_schedule *s, int32_t src,
                  int32_t delta, int32_t *dist_out, gg_stats *stats);
/* PageRank, `iters` iterations of pr.cpp:60-64; rank_out = old_rank. */
gg_status gg_pagerank(gg_graph *g, const gg_app_schedule *s, int32_t iters,
                      float damping, float *rank_out, gg_stats *stats);
/* Connected components (cc.cpp); labels_out[v] = min vertex id of v's component.
 * With s->fuse set (cc.cpp's main leaves it off) the hook / pointer-jump rounds
 * are fused into one pass over the edges: a lock-free union-find whose roots
 * are the smallest ids of their trees, giving the same labels. */
gg_status gg_cc(gg_graph *g, const gg_app_schedule *s, int32_t *labels_out,
                gg_stats *stats);
/* Single-source betweenness dependencies (bc.cpp) from src. */
gg_status gg_bc(gg_graph *g, const gg_app_schedule *s, int32_t src,
                float *dep_out, gg_stats *stats);

/* ------------------------------------------------- learned schedule selector
 * No reference counterpart.  A bf16 MLP (12 features -> 64 -> 64 -> 11 logits)
 * whose heads choose, per iteration, the direction (push/pull), the load
 * balancing (TWCE, ETWC, CM, WM, VERTEX_BASED, EDGE_ONLY) and the output frontier type
 * (queue, bitmap, boolmap).  Forward and backward are hand-written tensor-core
 * kernels (mma.sync bf16, fp32 accumulation); training is full-batch Adam on
 * fp32 master weights.  Used by app schedules of kind GG_SCHED_LEARNED, whose
 * s1 is the fallback when no selector is attached.
 * Features (per iteration): log2 of frontier vertices, frontier edges,
 * unvisited vertices and edges, frontier degree mean/max/variance; iteration
 * index; log2 V and E; frontier share of V and of E.
 * Labels: int32 triples (direction 0..1, load balancing 0..5, frontier 0..2). */
enum { GG_SEL_BFS = 0, GG_SEL_SSSP = 1, GG_SEL_CC = 2 };
typedef struct gg_selector gg_selector;
gg_status gg_selector_create(int64_t seed, gg_selector **out);
gg_status gg_selector_destroy(gg_selector *s);
int32_t gg_selector_num_params(void);
gg_status gg_selector_get_params(const gg_selector *s, float *out, int32_t n);
gg_status gg_selector_set_params(gg_selector *s, const float *in, int32_t n);
/* logits[n][11] of features x[n][12] (host or device memory). */
gg_status gg_selector_forward(gg_selector *s, const float *x, int32_t n, float *logits);
/* Gradient (all parameters) and loss of the mean summed cross-entropy. */
gg_status gg_selector_grad(gg_selector *s, const float *x, const int32_t *labels,
                           int32_t n, float *grad, float *loss);
gg_status gg_selector_train(gg_selector *s, const float *x, const int32_t *labels,
                            int32_t n, int32_t epochs, float lr, float *final_loss);
gg_status gg_selector_save(const gg_selector *s, const char *path);
gg_status gg_selector_load(const char *path, gg_selector **out);
/* Training data generated by the engine: runs `app` from src (delta for SSSP)
 * with the fallback schedule and, at each iteration, times all 36 candidate
 * schedules (candidate c = direction*18 + lb*3 + frontier) on the same state.
 * feats[max_rows][12], times[max_rows][36] in ms (INFINITY if a candidate
 * failed); *nrows = iterations recorded. */
gg_status gg_selector_collect(gg_graph *g, int32_t app, int32_t src, int32_t delta,
                              int32_t max_rows, float *feats, float *times,
                              int32_t *nrows);

/* ----------------------------------------------------- allocation-free BFS
 * No counterpart in the reference: an extra entry point for callers that may
 * not allocate device memory while they run (code inside someone else's
 * pre-sized memory pool or arena, real-time loops that cannot risk an
 * allocation stall or failure, hosts that keep their allocator to
 * themselves).  BFS from src over a CSR the caller already holds on the device;
 * depth_out (device, num_vertices entries) receives the hop distance or -1.
 * The library allocates nothing here: its scratch is one static device array
 * sized for at most 1,048,576 vertices (about 8 MiB, held on every GPU that
 * loads the library until the process exits); larger graphs are rejected with
 * GG_ERR_INVALID.  The first call on a device (and the first after the calling
 * thread's current context changes) looks up that array's address with
 * cudaGetSymbolAddress, which allocates nothing.  All calls share the array:
 * calls that overlap on the GPU race and must be serialised by the caller.
 * Runs on `stream` (NULL = legacy default stream), reads its status word back
 * and synchronises `stream` before it returns, with the result in depth_out. */
gg_status gg_bfs_noalloc(const int32_t *offsets, const int32_t *dst,
                         int32_t num_vertices, int32_t num_edges, int32_t src,
                         int32_t *depth_out, void *stream);

/* ------------------------------------------------------------ batched mode
 * Many sources in one persistent launch (no reference counterpart: the
 * reference runs one source per testcase() trial).  Results equal nsrc
 * independent runs of gg_bfs / gg_sssp.
 *  gg_bfs_batch: bit-parallel multi-source BFS, 64 sources per pass;
 *    depth_out[s*V + v] (host or device memory, nsrc*V int32).
 *  gg_sssp_batch: 32 sources per pass with per-source delta-stepping windows
 *    (gpu_priority_queue.h semantics) and a far pile instead of O(V) bucket
 *    scans; dist_out[s*V + v] (INT_MAX unreached).
 *  gg_bc_batch: BC dependencies of apps/bc.cpp for 64 sources per pass (the
 *    levels of one bit-parallel BFS shared by all sources; sigma and
 *    dependencies gathered per source in fp64); dep_out[s*V + v] (fp32, host
 *    or device memory, 0 where unreached).  Needs 64*V < 2^31.
 *    stats->edges_traversed = 2 * sum over sources of the reached out-edges. */
gg_status gg_bfs_batch(gg_graph *g, const int32_t *sources, int32_t nsrc,
                       int32_t *depth_out, gg_stats *stats);
gg_status gg_bc_batch(gg_graph *g, const int32_t *sources, int32_t nsrc,
                      float *dep_out, gg_stats *stats);
/* Batch plans: a whole gg_bfs_batch / gg_sssp_batch / gg_bc_batch captured
 * once into a CUDA graph (every persistent launch of every group of sources)
 * and replayed with one graph launch per run.  `out` must be device memory:
 * nsrc*V int32 (BFS depths, SSSP distances) or float (BC dependencies).  The
 * plan copies the sources and owns its device state; delta is used by SSSP.
 * GG_BATCH_BFS_MULTI / GG_BATCH_SSSP_MULTI capture one multi-source traversal
 * (gg_bfs_multi / gg_sssp_multi with the TWCE fused loop; one persistent
 * launch) writing V int32 into `out`: over a disjoint union of graphs with one
 * source per part, every part's own BFS / SSSP. */
typedef struct gg_batch_plan gg_batch_plan;
enum { GG_BATCH_BFS = 0, GG_BATCH_SSSP = 1, GG_BATCH_BC = 2,
       GG_BATCH_BFS_MULTI = 3, GG_BATCH_SSSP_MULTI = 4 };
gg_status gg_batch_plan_create(gg_graph *g, int32_t app, const int32_t *sources,
                               int32_t nsrc, int32_t delta, void *out,
                               gg_batch_plan **plan);
gg_status gg_batch_plan_run(gg_batch_plan *plan, gg_stats *stats);
gg_status gg_batch_plan_destroy(gg_batch_plan *plan);
/* Launch shape of a graph's batched kernels (no reference counterpart).
 * Zero fields take the built-in default.  Results never depend on it.
 *  blocks_per_sm      persistent CTAs per SM, capped at what fits (default:
 *                     all that fit);
 *  chunk              edges per work item of batched SSSP and BC, a power of
 *                     two in [32, 4096] (default 256);
 *  edge_parallel_max  batched SSSP: work items active for at most this many
 *                     sources map lanes to edges, the others lanes to sources
 *                     (default 6; -1 = never edge-parallel; at most 32);
 *  bottom_up_div      batched BFS: a level whose frontier holds more than
 *                     V / bottom_up_div vertices runs bottom-up over in-lists
 *                     (default 16; -1 = always top-down; at most 4096);
 *  per_source_cta     batched SSSP: 1 = every source runs the delta-stepping
 *                     loop in a CTA of its own (the single-source bucket queue,
 *                     no grid barriers; for meshes and road-like graphs),
 *                     -1 = the lane-per-source kernel, 0 = by the graph: a CTA
 *                     per source when no vertex has more than 32 out-edges.
 * The tuning of `app` (GG_BATCH_*) applies to the batched calls and to plans
 * created after it is set. */
typedef struct gg_batch_tuning {
  int32_t blocks_per_sm;
  int32_t chunk;
  int32_t edge_parallel_max;
  int32_t bottom_up_div;
  int32_t per_source_cta;
} gg_batch_tuning;
gg_status gg_batch_set_tuning(gg_graph *g, int32_t app, const gg_batch_tuning *t);
gg_status gg_batch_get_tuning(const gg_graph *g, int32_t app, gg_batch_tuning *t);
/* Autotuner: times candidate launch shapes of `app` on the graph (one pass
 * over the first min(nsrc, pass width) sources per candidate, best of two
 * timed runs of the persistent kernel), by coordinate descent over
 * blocks_per_sm, then chunk (SSSP, BC), edge_parallel_max (SSSP) or
 * bottom_up_div (BFS); sets the fastest as the
 * graph's tuning and returns it in *best.  Every trial goes to rows (at most
 * max_rows; *nrows = trials run).  delta is used by SSSP. */
typedef struct gg_tune_row {
  gg_batch_tuning tuning;
  float ms;
} gg_tune_row;
gg_status gg_batch_autotune(gg_graph *g, int32_t app, const int32_t *sources,
                            int32_t nsrc, int32_t delta, gg_batch_tuning *best,
                            gg_tune_row *rows, int32_t max_rows, int32_t *nrows);
/* Multi-source traversal with the app schedule: every source starts at 0 and
 * out[v] is the distance to the nearest source.  With one source per part of a
 * gg_host_graph_union this runs many graphs of uneven size in one persistent
 * launch (fuse=1), load-balanced across graphs by the schedule's LB. */
gg_status gg_bfs_multi(gg_graph *g, const gg_app_schedule *s,
                       const int32_t *sources, int32_t n, int32_t *depth_out,
                       int32_t *parent_out, gg_stats *stats);
gg_status gg_sssp_multi(gg_graph *g, const gg_app_schedule *s,
                        const int32_t *sources, int32_t n, int32_t delta,
                        int32_t *dist_out, gg_stats *stats);
gg_status gg_sssp_batch(gg_graph *g, const int32_t *sources, int32_t nsrc,
                        int32_t delta, int32_t *dist_out, gg_stats *stats);
/* SSSP on a disjoint union of graphs (gg_host_graph_union) with one source per
 * part, every part's delta-stepping loop in a CTA of its own (no reference
 * counterpart; the batched mode's path for many high-diameter graphs, whose
 * loops are barrier-bound on the whole GPU).  Part p holds the vertices
 * [part_begin[p], part_begin[p+1]) and sources[p] (a vertex of the union) lies
 * in it; an edge that leaves its part gives GG_ERR_INVALID.  dist_out: V int32
 * (INT_MAX unreached), each part's values equal to its own gg_sssp. */
gg_status gg_sssp_parts(gg_graph *g, const int32_t *part_begin, int32_t nparts,
                        const int32_t *sources, int32_t delta, int32_t *dist_out,
                        gg_stats *stats);

/* Learned per-level schedule of the batched kernels (no reference
 * counterpart): with a selector attached, batched BFS (GG_BATCH_BFS, the only
 * app that takes one) picks each level's direction -- top-down or bottom-up --
 * with the network's direction head on that level's frontier statistics,
 * computed on the device inside the persistent loop (no host round trip).
 * NULL detaches it (the bottom_up_div rule decides again).  The selector must
 * outlive the calls and plans that use it.  Results never depend on it. */
gg_status gg_batch_set_selector(gg_graph *g, int32_t app, const gg_selector *sel);
/* Its training data, made by the engine: the first min(nsrc, 64) sources
 * traversed with every level forced top-down and then bottom-up (a level's
 * result does not depend on its direction, so level l starts from the same
 * state in every run).  feats[l][12] (the selector's features of level l),
 * times[l][2] (ms top-down, bottom-up); *nrows = levels recorded. */
gg_status gg_batch_collect(gg_graph *g, int32_t app, const int32_t *sources, int32_t nsrc,
                           int32_t max_rows, float *feats, float *times, int32_t *nrows);

/* ------------------------------------------------------------ diagnostics
 * Runs a grid barrier that can never complete (it waits for one block more
 * than were launched) with the given time limit, to exercise the bounded-wait
 * path; returns GG_ERR_TIMEOUT when the wait gave up as designed. */
gg_status gg_debug_barrier_timeout(int32_t timeout_us);

#ifdef __cplusplus
}
#endif
#endif /* GG_H */
