// edgeset.apply kernels of the BC forward UDF (apps/bc.cpp:34-36): every load-balancing
// strategy in both directions.
#include "lb_launch.cuh"

namespace gg {

gg_status launch_bcf(const EdgeLaunch &L) {
  UBcF u{L.vd.num_paths, L.vd.visited};
  return launch_dir(L, u);
}

}  // namespace gg
