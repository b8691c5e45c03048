// edgeset.apply kernels of the BC backward UDF (apps/bc.cpp:52-54): every load-balancing
// strategy in both directions.
#include "lb_launch.cuh"

namespace gg {

gg_status launch_bcb(const EdgeLaunch &L) {
  if (L.vd.dep64) {
    UBcB<double> u{L.vd.dep64, L.vd.visited};
    return launch_dir(L, u);
  }
  UBcB<float> u{L.vd.dependences, L.vd.visited};
  return launch_dir(L, u);
}

}  // namespace gg
