// Internal declarations shared by the host (.cpp) and device (.cu) parts of
// libgg.so.  Nothing here is part of the C ABI.
#pragma once

#include <cstdarg>
#include <cstdint>
#include <string>

#include "../../include/gg.h"

namespace gg {

// Records `fmt` as the calling thread's last error and returns `s`.
gg_status set_error(gg_status s, const char *fmt, ...)
    __attribute__((format(printf, 2, 3)));
void clear_error();

// Process-wide launch defaults (SimpleGPUSchedule::default_max_cta/_cta_size).
extern int32_t g_default_max_cta;
extern int32_t g_default_cta_size;

// Counts kernel launches issued by the library (gg_kernel_launches()).
void note_launch();
uint64_t launches();

}  // namespace gg

// The host CSR graph (gg_host_graph in the ABI).
struct gg_host_graph {
  int32_t V = 0;
  int64_t E = 0;
  std::basic_string<int32_t> offsets;  // V+1
  std::basic_string<int32_t> dst;      // E
  std::basic_string<int32_t> w;        // E
};

#define GG_CHECK_ARG(cond, msg)                                   \
  do {                                                            \
    if (!(cond)) return gg::set_error(GG_ERR_INVALID, "%s", msg); \
  } while (0)
