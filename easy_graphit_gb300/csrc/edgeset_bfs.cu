// edgeset.apply kernels of the BFS parent UDF (apps/bfs.cpp:23-29): every load-balancing
// strategy in both directions.
#include "lb_launch.cuh"

namespace gg {

gg_status launch_bfs(const EdgeLaunch &L) {
  UBfs u{L.vd.parent, L.vd.depth, L.vd.level};
  return launch_dir(L, u);
}

}  // namespace gg
