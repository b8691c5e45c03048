// Thread-local error reporting for the C ABI.  The reference prints and calls
// exit(-1) (runtime/infra_gpu/support.h:4-10); here the status is returned and
// the message is kept for gg_last_error().
#include <atomic>
#include <cstdio>
#include <cstring>

#include "gg_internal.h"

namespace gg {

static thread_local std::string t_last_error;

int32_t g_default_max_cta = 60;   // schedule.cpp:6
int32_t g_default_cta_size = 512; // schedule.cpp:5

gg_status set_error(gg_status s, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  t_last_error = buf;
  return s;
}

void clear_error() { t_last_error.clear(); }

static std::atomic<uint64_t> g_launch_count{0};
void note_launch() { g_launch_count.fetch_add(1, std::memory_order_relaxed); }
uint64_t launches() { return g_launch_count.load(std::memory_order_relaxed); }

}  // namespace gg

extern "C" uint64_t gg_kernel_launches(void) { return gg::launches(); }

extern "C" size_t gg_last_error(char *buf, size_t n) {
  const std::string &e = gg::t_last_error;
  if (buf && n > 0) {
    size_t k = e.size() < n - 1 ? e.size() : n - 1;
    std::memcpy(buf, e.data(), k);
    buf[k] = 0;
  }
  return e.size();
}

extern "C" const char *gg_version(void) { return "easy_graphit_gb300 0.1 (sm_103a)"; }

extern "C" void gg_set_default_launch(int32_t max_cta, int32_t cta_size) {
  if (max_cta > 0) gg::g_default_max_cta = max_cta;
  if (cta_size >= 32 && cta_size <= 1024 && cta_size % 32 == 0)
    gg::g_default_cta_size = cta_size;
}

extern "C" void gg_schedule_init(gg_schedule *s) {
  if (!s) return;
  // SimpleGPUSchedule() constructor, include/graphit/schedule.h:87-97.
  s->direction = GG_PUSH;
  s->pull_frontier_rep = GG_PULL_BOOLMAP;
  s->frontier_creation = GG_FC_SPARSE;
  s->deduplication = GG_DEDUP_DISABLED;
  s->deduplication_strategy = GG_DEDUP_FUSED;
  s->load_balancing = GG_LB_VERTEX_BASED;
  s->edge_blocking = GG_UNBLOCKED;
  s->block_size = -1;
  s->kernel_fusion = GG_FUSION_DISABLED;
  s->max_cta = gg::g_default_max_cta;
  s->cta_size = gg::g_default_cta_size;
}
