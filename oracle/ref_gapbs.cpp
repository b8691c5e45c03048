// ORACLE -- test infrastructure only.
//
// Driver that runs the reference's own CPU code (the vendored GAPBS headers of
// easy_graphit, runtime/infra_gapbs/) to produce golden data.  It is compiled
// by `make -C oracle ref` with those headers included where they lie in the
// reference tree; the binary goes to oracle/_ref/ and is never shipped.
//
//   ref_gapbs graph <scale> <degree> <symmetrize> <out.bin>
//       Generator::MakeRMatEL + InsertWeights (generator.h:74-139), then
//       BuilderBase::MakeGraphFromEL + SquishGraph (builder.h:165-226).
//       Writes [i32 V][i64 E][i32 offsets[V+1]][i32 dst[E]][i32 w[E]].
//   ref_gapbs sssp <scale> <degree> <symmetrize> <unit_weights> <delta> <out.bin> <src>...
//       Same graph, then OrderedProcessingOperatorNoMerge with the
//       updatePriorityMin edge function (ordered_processing.h:15-143) per
//       source.  Writes [i32 nsrc][i32 V] then nsrc rows of i32 dist[V]
//       (INT_MAX = unreached).
#include "benchmark.h"
#include "ordered_processing.h"

#include <climits>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

namespace {

// CLBase only carries the symmetrize flag here; generation is driven directly.
struct SymCL : public CLBase {
  explicit SymCL(bool sym) : CLBase(std::string("")) { symmetrize_ = sym; }
};

WGraph make_graph(int scale, int degree, bool sym) {
  SymCL cli(sym);
  WeightedBuilder b(cli);
  Generator<NodeID, WNode> gen(scale, degree);
  pvector<EdgePair<NodeID, WNode>> el = gen.GenerateEL(false);
  Generator<NodeID, WNode>::InsertWeights(el);
  WGraph g = b.MakeGraphFromEL(el);
  return b.SquishGraph(g);
}

void csr_of(const WGraph &g, bool unit, std::vector<int32_t> &off,
            std::vector<int32_t> &dst, std::vector<int32_t> &w) {
  const int32_t V = g.num_nodes();
  off.assign(V + 1, 0);
  dst.clear();
  w.clear();
  for (int32_t u = 0; u < V; ++u) {
    for (WNode wn : g.out_neigh(u)) {
      dst.push_back(wn.v);
      w.push_back(unit ? 1 : wn.w);
    }
    off[u + 1] = (int32_t)dst.size();
  }
}

}  // namespace

int main(int argc, char **argv) {
  if (argc < 2) return 2;
  const std::string mode = argv[1];
  if (mode == "graph" && argc == 6) {
    WGraph g = make_graph(atoi(argv[2]), atoi(argv[3]), atoi(argv[4]) != 0);
    std::vector<int32_t> off, dst, w;
    csr_of(g, false, off, dst, w);
    FILE *f = fopen(argv[5], "wb");
    if (!f) return 3;
    const int32_t V = g.num_nodes();
    const int64_t E = (int64_t)dst.size();
    fwrite(&V, 4, 1, f);
    fwrite(&E, 8, 1, f);
    fwrite(off.data(), 4, off.size(), f);
    fwrite(dst.data(), 4, dst.size(), f);
    fwrite(w.data(), 4, w.size(), f);
    fclose(f);
    return 0;
  }
  if (mode == "sssp" && argc >= 9) {
    WGraph g = make_graph(atoi(argv[2]), atoi(argv[3]), atoi(argv[4]) != 0);
    const bool unit = atoi(argv[5]) != 0;
    const int32_t delta = atoi(argv[6]);
    if (unit) {
      // Rebuild with unit weights so delta-stepping yields hop distances.
      for (NodeID u = 0; u < g.num_nodes(); ++u)
        for (WNode &wn : g.out_neigh(u)) wn.w = 1;
    }
    const int32_t V = g.num_nodes();
    const int32_t nsrc = argc - 8;
    FILE *f = fopen(argv[7], "wb");
    if (!f) return 3;
    fwrite(&nsrc, 4, 1, f);
    fwrite(&V, 4, 1, f);
    std::vector<int32_t> SP(V);
    for (int i = 0; i < nsrc; ++i) {
      const NodeID src = atoi(argv[8 + i]);
      for (int32_t v = 0; v < V; ++v) SP[v] = INT_MAX;
      SP[src] = 0;
      EagerPriorityQueue<int32_t> pq(SP.data(), delta);
      auto while_cond = [&]() { return !pq.finished(); };
      auto edge_apply = [&](std::vector<std::vector<NodeID>> &local_bins, NodeID s,
                            NodeID d, WeightT wt) {
        updatePriorityMin<int32_t>()(&pq, local_bins, d, SP[d], SP[s] + wt);
      };
      OrderedProcessingOperatorNoMerge(&pq, g, while_cond, edge_apply, src);
      fwrite(SP.data(), 4, V, f);
    }
    fclose(f);
    return 0;
  }
  fprintf(stderr, "usage: ref_gapbs graph|sssp ...\n");
  return 2;
}
