// yh_threads.cpp -- process-wide limit on the host threads of the host producers
// (yh_bvh_build, yh_cache_*) and of the scene repack inside yc_upload_scene. Their
// outputs do not depend on it: work is split into chunks whose partial results are
// combined in a fixed order.
#include "yh_threads.h"

#include <algorithm>
#include <atomic>
#include <thread>

#include "yune_host.h"

namespace {
std::atomic<int> g_limit{0};   // 0: every core the host reports
}  // namespace

namespace yh {
int host_threads() {
  const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
  const int lim = g_limit.load(std::memory_order_relaxed);
  return lim > 0 ? lim : hw;
}
}  // namespace yh

extern "C" int yh_set_host_threads(int n) {
  if (n < 0 || n > 4096) return YH_E_INVALID;
  g_limit.store(n, std::memory_order_relaxed);
  return YH_OK;
}

extern "C" int yh_get_host_threads(void) { return yh::host_threads(); }
