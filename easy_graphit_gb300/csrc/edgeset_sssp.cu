// edgeset.apply kernels of the SSSP relax UDF (apps/sssp.cpp:24-27): every load-balancing
// strategy in both directions.
#include "lb_launch.cuh"

namespace gg {

gg_status launch_sssp(const EdgeLaunch &L) {
  USssp u{L.vd.dist, L.prio_cutoff, L.vd.far};
  return launch_dir(L, u);
}

}  // namespace gg
