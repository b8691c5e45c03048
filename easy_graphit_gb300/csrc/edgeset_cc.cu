// edgeset.apply kernels of the CC hook UDF (apps/cc.cpp:23-36): every load-balancing
// strategy in both directions.
#include "lb_launch.cuh"

namespace gg {

gg_status launch_cc(const EdgeLaunch &L) {
  UCc u{L.vd.ids, L.vd.updates};
  return launch_dir(L, u);
}

}  // namespace gg
