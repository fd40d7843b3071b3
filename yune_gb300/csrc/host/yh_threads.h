// yh_threads.h -- the number of host threads the host producers and the scene repack
// use (yh_set_host_threads; all cores unless a caller sets a limit).
#pragma once

namespace yh {
int host_threads();
}  // namespace yh
