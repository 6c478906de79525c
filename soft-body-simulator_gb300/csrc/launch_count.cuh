// Host-side count of the kernel launches this library enqueues, per host
// thread.  Every launcher adds the kernels it enqueues; the handle reads the
// difference around a frame (and, for a CUDA graph, around its capture, whose
// kernels then run on every replay).
#pragma once

#include <stdint.h>

namespace sbs {

uint64_t& launch_counter();
inline void count_launch(uint64_t n = 1) { launch_counter() += n; }

}  // namespace sbs
