// gg_app: the apps' testcase() trial loops (apps/{bfs,sssp,pr,cc,bc}.cpp) as one
// command-line driver over the C ABI, so runs behave like the reference apps:
//
//   gg_app <bfs|sssp|pr|cc|bc> <graph> [src] [delta | threshold]
//          [--max-cta N] [--cta-size N] [--power] [--trials N] [--out FILE]
//
// <graph> is a file gg_host_graph_load reads (.graphit_bin, .el, .wel, .gr,
// .mtx) or a generator: rmat:SCALE[:DEGREE][:sym] (GAPBS R-MAT) or
// grid:ROWS:COLS.  --max-cta / --cta-size set the schedules' launch defaults
// (SimpleGPUSchedule::default_max_cta / default_cta_size, the apps' argv[1]
// and argv[2]); --power selects each app's alternative schedule (argv[3] ==
// "power").  The source defaults to GAPBS's SourcePicker's first pick; the
// SSSP delta defaults to 32 and the hybrid threshold of BFS / BC to 0.12.
// Each trial prints its wall time in seconds, one per line, as print_time does
// (PageRank prints t / 20); trial counts follow the apps (4, 5, 10, 10, 3).
// --out writes the last trial's result array (raw int32 or float32, V values).
#include <sys/time.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gg.h"

namespace {

[[noreturn]] void die(const char *what) {
  char buf[1024];
  gg_last_error(buf, sizeof(buf));
  std::fprintf(stderr, "gg_app: %s: %s\n", what, buf);
  std::exit(1);
}

void check(gg_status s, const char *what) {
  if (s != GG_OK) die(what);
}

double now_s() {
  timeval t{};
  gettimeofday(&t, nullptr);
  return t.tv_sec + t.tv_usec / 1e6;
}

gg_host_graph *load(const std::string &spec, bool *sym) {
  gg_host_graph *hg = nullptr;
  if (spec.rfind("rmat:", 0) == 0) {
    int scale = 0, degree = 16;
    char tail[16] = {0};
    const int n = std::sscanf(spec.c_str() + 5, "%d:%d:%15s", &scale, &degree, tail);
    if (n < 1) {
      std::fprintf(stderr, "gg_app: bad generator %s\n", spec.c_str());
      std::exit(2);
    }
    *sym = std::strcmp(tail, "sym") == 0;
    check(gg_host_graph_rmat(scale, degree, 0.57f, 0.19f, 0.19f, 27491095, *sym, 1, 255, &hg), "rmat");
  } else if (spec.rfind("grid:", 0) == 0) {
    int rows = 0, cols = 0;
    if (std::sscanf(spec.c_str() + 5, "%d:%d", &rows, &cols) != 2) {
      std::fprintf(stderr, "gg_app: bad generator %s\n", spec.c_str());
      std::exit(2);
    }
    *sym = true;
    check(gg_host_graph_grid(rows, cols, 27491095, 1, 1000, &hg), "grid");
  } else {
    check(gg_host_graph_load(spec.c_str(), 0, &hg), "load");
  }
  return hg;
}

// The schedules each app's main() builds (apps/*.cpp), default or "power".
gg_app_schedule app_schedule(const std::string &app, bool power, float threshold) {
  gg_app_schedule s{};
  s.kind = GG_SCHED_SIMPLE;
  gg_schedule_init(&s.s1);
  gg_schedule_init(&s.s2);
  s.threshold = threshold;
  if (app == "bfs") {  // bfs.cpp:69-92
    s.s1.load_balancing = GG_LB_TWCE;
    if (power) {
      s.kind = GG_SCHED_HYBRID;
      s.s2.direction = GG_PULL;
      s.s2.pull_frontier_rep = GG_PULL_BITMAP;
      s.s2.load_balancing = GG_LB_VERTEX_BASED;
      s.s2.frontier_creation = GG_FC_BITMAP;
    } else {
      s.fuse = 1;
    }
  } else if (app == "sssp") {  // sssp.cpp:65-83
    if (power) {
      s.s1.load_balancing = GG_LB_TWCE;
      s.s1.frontier_creation = GG_FC_BOOLMAP;
    } else {
      s.s1.frontier_creation = GG_FC_SPARSE;
      s.fuse = 1;
    }
  } else if (app == "pr") {  // pr.cpp:79-81
    s.s1.direction = GG_PULL;
    s.s1.load_balancing = GG_LB_EDGE_ONLY;
    s.s1.edge_blocking = GG_BLOCKED;
    s.s1.block_size = 0x42000;
  } else if (app == "cc") {  // cc.cpp:86-88
    s.s1.load_balancing = GG_LB_EDGE_ONLY;
  } else if (app == "bc") {  // bc.cpp:131-156
    s.s1.load_balancing = GG_LB_TWCE;
    if (power) {
      s.kind = GG_SCHED_HYBRID;
      s.s2.direction = GG_PULL;
      s.s2.pull_frontier_rep = GG_PULL_BITMAP;
      s.s2.load_balancing = GG_LB_TWCE;
      s.s2.frontier_creation = GG_FC_BITMAP;
    } else {
      s.fuse = 1;
    }
  }
  return s;
}

void usage() {
  std::fprintf(stderr,
               "usage: gg_app <bfs|sssp|pr|cc|bc> <graph file | rmat:S[:D][:sym] | grid:R:C> [src] "
               "[delta|threshold]\n              [--max-cta N] [--cta-size N] [--power] [--trials N] "
               "[--out FILE]\n");
  std::exit(2);
}

}  // namespace

int main(int argc, char **argv) {
  std::vector<std::string> pos;
  int max_cta = 60, cta_size = 512, trials = -1;  // schedule.cpp:5-6 defaults
  bool power = false;
  const char *out_path = nullptr;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    auto next = [&]() -> const char * {
      if (i + 1 >= argc) usage();
      return argv[++i];
    };
    if (a == "--max-cta") max_cta = std::atoi(next());
    else if (a == "--cta-size") cta_size = std::atoi(next());
    else if (a == "--trials") trials = std::atoi(next());
    else if (a == "--out") out_path = next();
    else if (a == "--power" || a == "power") power = true;
    else if (a == "-h" || a == "--help") usage();
    else pos.push_back(a);
  }
  if (pos.size() < 2) usage();
  const std::string app = pos[0];
  if (app != "bfs" && app != "sssp" && app != "pr" && app != "cc" && app != "bc") usage();
  if (trials < 0) trials = app == "bfs" ? 4 : app == "sssp" ? 5 : app == "bc" ? 3 : 10;
  gg_set_default_launch(max_cta, cta_size);

  bool sym = false;
  gg_host_graph *hg = load(pos[1], &sym);
  int32_t V = 0;
  int64_t E = 0;
  check(gg_host_graph_info(hg, &V, &E), "info");
  int32_t src = 0;
  if (pos.size() > 2) {
    src = std::atoi(pos[2].c_str());
  } else if (app != "pr" && app != "cc") {
    check(gg_host_graph_pick_sources(hg, 1, 27491095, &src), "source");
  }
  if (src < 0 || src >= V) {
    std::fprintf(stderr, "gg_app: source %d out of range [0, %d)\n", src, V);
    return 2;
  }
  const int32_t delta = (app == "sssp" && pos.size() > 3) ? std::atoi(pos[3].c_str()) : 32;
  const float threshold = ((app == "bfs" || app == "bc") && pos.size() > 3) ? (float)std::atof(pos[3].c_str()) : 0.12f;
  gg_graph *g = nullptr;
  check(gg_graph_create(gg_host_graph_offsets(hg), gg_host_graph_dst(hg), gg_host_graph_weights(hg), V, E,
                        sym ? GG_GRAPH_SYMMETRIC : 0, &g),
        "graph");
  const gg_app_schedule s = app_schedule(app, power, threshold);
  std::vector<int32_t> iout(V);
  std::vector<float> fout(V);
  gg_stats st{};
  for (int t = 0; t < trials; ++t) {
    const double t0 = now_s();
    if (app == "bfs") check(gg_bfs(g, &s, src, iout.data(), nullptr, &st), "bfs");
    else if (app == "sssp") check(gg_sssp(g, &s, src, delta, iout.data(), &st), "sssp");
    else if (app == "pr") check(gg_pagerank(g, &s, 20, 0.85f, fout.data(), &st), "pagerank");
    else if (app == "cc") check(gg_cc(g, &s, iout.data(), &st), "cc");
    else check(gg_bc(g, &s, src, fout.data(), &st), "bc");
    const double t1 = now_s() - t0;
    std::printf("%g\n", app == "pr" ? t1 / 20 : t1);
  }
  std::fprintf(stderr, "gg_app %s V=%d E=%lld src=%d: %d iterations, %lld edges, device %.3f ms, %.2f GTEPS\n",
               app.c_str(), V, (long long)E, src, st.iterations, (long long)st.edges_traversed, st.device_ms,
               st.device_ms > 0 ? st.edges_traversed / (st.device_ms * 1e6) : 0.0);
  if (out_path) {
    FILE *f = std::fopen(out_path, "wb");
    if (!f) {
      std::perror(out_path);
      return 1;
    }
    const bool fl = app == "pr" || app == "bc";
    std::fwrite(fl ? (const void *)fout.data() : (const void *)iout.data(), 4, V, f);
    std::fclose(f);
  }
  gg_graph_destroy(g);
  gg_host_graph_destroy(hg);
  return 0;
}
