// edgeset.apply kernels of the PageRank edge UDF (apps/pr.cpp:32-34): every load-balancing
// strategy in both directions.
#include "lb_launch.cuh"

namespace gg {

gg_status launch_pr(const EdgeLaunch &L) {
  UPr u{L.vd.contrib, L.vd.new_rank};
  return launch_dir(L, u);
}

}  // namespace gg
