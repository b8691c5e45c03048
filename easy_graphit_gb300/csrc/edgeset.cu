// edgeset.apply dispatch: the host logic of edgeset_apply::apply
// (src/graphit/operators.cpp:513-650) and apply_modified / apply_priority
// (include/graphit/operators.h:73-173).
//
// PUSH enumerates the from-frontier (sparse) or every vertex; the to() filter
// guards destinations.  PULL converts the from-frontier to a bitmap or boolmap,
// enumerates the reverse frontier (vertices passing to()) over the transposed
// graph, tests neighbours for membership, and calls the UDF with swapped
// endpoints.  EDGE_ONLY walks every COO edge (optionally the dst-blocked copy).
// apply_modified writes the tracked vertices into the output side of `out` in
// the schedule's frontier_creation format and swaps it in afterwards.
#include "engine.h"

namespace gg {

static gg_status validate(const gg_schedule *s) {
  if (!s) return set_error(GG_ERR_INVALID, "schedule is NULL");
  if (s->direction != GG_PUSH && s->direction != GG_PULL)
    return set_error(GG_ERR_INVALID, "bad direction %d", s->direction);
  if (s->load_balancing < GG_LB_VERTEX_BASED || s->load_balancing > GG_LB_ETWC)
    return set_error(GG_ERR_INVALID, "bad load balancing %d", s->load_balancing);
  if (s->frontier_creation < GG_FC_SPARSE || s->frontier_creation > GG_FC_BOOLMAP)
    return set_error(GG_ERR_INVALID, "bad frontier creation %d", s->frontier_creation);
  if (s->cta_size < 64 || s->cta_size > 1024 || s->cta_size % 32)
    return set_error(GG_ERR_INVALID, "cta_size %d must be a multiple of 32 in [64,1024]",
                     s->cta_size);
  if (s->load_balancing == GG_LB_EDGE_ONLY && s->edge_blocking == GG_BLOCKED && s->block_size <= 0)
    return set_error(GG_ERR_INVALID, "Invalid block size value");  // operators.cpp:624
  return GG_OK;
}

static gg_status check_udf(int32_t udf, const VData &vd) {
  bool ok = true;
  switch (udf) {
    case GG_UDF_BFS_PARENT: ok = vd.parent; break;
    case GG_UDF_SSSP_RELAX: ok = vd.dist; break;
    case GG_UDF_PR_ADD: ok = vd.contrib && vd.new_rank; break;
    case GG_UDF_CC_HOOK: ok = vd.ids && vd.updates; break;
    case GG_UDF_BC_FORWARD: ok = vd.num_paths && vd.visited; break;
    case GG_UDF_BC_BACKWARD: ok = (vd.dependences || vd.dep64) && vd.visited; break;
    default: return set_error(GG_ERR_INVALID, "unknown edge UDF %d", udf);
  }
  if (!ok) return set_error(GG_ERR_INVALID, "vertex data needed by UDF %d is NULL", udf);
  return GG_OK;
}

gg_status edgeset_apply_impl(gg_graph *g, const gg_schedule *s, int32_t udf, int32_t filter,
                             gg_frontier *from, gg_frontier *out, bool allow_dupes,
                             const VData &vd, int32_t prio_cutoff, bool) {
  GG_TRY(validate(s));
  GG_TRY(check_udf(udf, vd));
  if (filter == GG_FILTER_PARENT_UNSET && !vd.parent)
    return set_error(GG_ERR_INVALID, "parent filter needs vertex data parent");
  if (filter == GG_FILTER_UNVISITED && !vd.visited)
    return set_error(GG_ERR_INVALID, "visited filter needs vertex data visited");
  const int32_t V = g->csr.V;
  const bool edge_only = s->load_balancing == GG_LB_EDGE_ONLY;
  EdgeLaunch L{};
  L.graph = g;
  L.cta = s->cta_size;
  L.max_cta = s->max_cta;
  L.lb = s->load_balancing;
  L.vd = vd;
  L.prio_cutoff = prio_cutoff;
  L.filter = filter != GG_FILTER_NONE;
  L.in_src = DIn{IN_ALL, nullptr, nullptr};
  L.in_dst = DIn{IN_ALL, nullptr, nullptr};
  L.en = Enum{nullptr, nullptr, V};
  L.n_host = V;
  const GraphStore *gs = &g->csr;
  bool skip = false;
  if (s->direction == GG_PUSH) {
    if (from) {
      int32_t n = 0;
      if (edge_only) {
        GG_TRY(frontier_prepare_bitmap(from));
        L.in_src = frontier_in_view(from);
        GG_TRY(frontier_size(from, &n));
      } else {
        GG_TRY(frontier_prepare_sparse(from));
        GG_TRY(frontier_size(from, &n));
        L.en = Enum{from->q_in, from->cnt_in, n};
        L.n_host = n;
      }
      skip = n == 0;
    }
  } else {
    L.pull = true;
    if (from) {
      if (s->pull_frontier_rep == GG_PULL_BITMAP)
        GG_TRY(frontier_prepare_bitmap(from));
      else
        GG_TRY(frontier_prepare_boolmap(from));
      L.in_dst = frontier_in_view(from);
      int32_t n = 0;
      GG_TRY(frontier_size(from, &n));
      skip = n == 0;
      if (!edge_only && !skip) {
        int32_t *rq = nullptr, *rc = nullptr;
        GG_TRY(reverse_frontier(g, filter, vd, &rq, &rc));
        L.en = Enum{rq, rc, -1};
        L.n_host = -1;
        if (s->load_balancing == GG_LB_STRICT) {  // STRICT sizes its scan on the host
          GG_CUDA(cudaMemcpyAsync(g->h_pinned + 4, rc, sizeof(int32_t), cudaMemcpyDeviceToHost, g->stream));
          GG_CUDA(cudaStreamSynchronize(g->stream));
          L.n_host = g->h_pinned[4];
          L.en.n = L.n_host;
        }
      }
    }
    GG_TRY(ensure_transpose(g));
    if (g->csc) gs = g->csc.get();
  }
  if (edge_only && s->edge_blocking == GG_BLOCKED)
    GG_TRY(ensure_blocked(g, L.pull && !g->symmetric, s->block_size, &gs));
  else if (edge_only && gs == &g->csr)
    GG_TRY(ensure_coo(g->csr, g->stream));  // EDGE_ONLY walks the COO source column
  L.g = gs->view();
  if (!edge_only) L.g.nbuckets = 0;
  const bool sparse_out = s->frontier_creation == GG_FC_SPARSE;
  const bool dedup = !allow_dupes && sparse_out;
  const bool fused_dedup = dedup && s->deduplication_strategy != GG_DEDUP_UNFUSED;
  if (out) {
    if (dedup) out->epoch++;  // curr_dedup_counter + 1, operators.h:147-149
    L.out = frontier_out_view(out, s->frontier_creation, fused_dedup);
  } else {
    L.out = DOut{};
    L.out.mode = OUT_NONE;
  }
  if (!skip) {
    switch (udf) {
      case GG_UDF_BFS_PARENT: GG_TRY(launch_bfs(L)); break;
      case GG_UDF_SSSP_RELAX: GG_TRY(launch_sssp(L)); break;
      case GG_UDF_PR_ADD: GG_TRY(launch_pr(L)); break;
      case GG_UDF_CC_HOOK: GG_TRY(launch_cc(L)); break;
      case GG_UDF_BC_FORWARD: GG_TRY(launch_bcf(L)); break;
      case GG_UDF_BC_BACKWARD: GG_TRY(launch_bcb(L)); break;
    }
  }
  if (out) {
    GG_TRY(frontier_swap(out, s->frontier_creation));
    if (dedup && !fused_dedup) GG_TRY(frontier_dedup(out));  // dedup_frontier_perfect
  }
  return GG_OK;
}

}  // namespace gg

using namespace gg;

extern "C" gg_status gg_edgeset_apply(gg_graph *g, const gg_schedule *s, int32_t udf,
                                      int32_t to_filter, gg_frontier *from, gg_frontier *out,
                                      int32_t allow_dupes, const gg_vertex_data *vd) {
  GG_CHECK_ARG(g && vd, "bad arguments");
  GG_CHECK_ARG(to_filter >= GG_FILTER_NONE && to_filter <= GG_FILTER_UNVISITED, "bad to() filter");
  GG_TRY(edgeset_apply_impl(g, s, udf, to_filter, from, out, allow_dupes != 0, to_vdata(vd), INT_MAX,
                            false));
  return check_device_error(g, "edgeset_apply");
}
