// Shared host-side helpers of the C ABI: per-thread last-error text and status plumbing.
#pragma once

#include <cstdarg>
#include <cstdio>
#include <string>

#include "phe_gb300.h"

namespace phe_gb300 {

// Records `msg` as this thread's last error and returns `status`. The reference logs and
// continues on errors (cuda_ray_tracer/CudaHelpers.hpp:13-25); this library reports them instead.
phe_status fail(phe_status status, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
void clear_error();

} // namespace phe_gb300
