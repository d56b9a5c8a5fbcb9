// Shared host-side helpers of the C ABI: per-thread last-error text and status plumbing.
#pragma once

#include <cstdarg>
#include <cstdio>
#include <string>

#include <nvtx3/nvToolsExt.h>

#include "phe_gb300.h"

namespace phe_gb300 {

// NVTX range around one library operation (frame, batch launch, serving wave, scene upload, BVH
// build): visible in Nsight timelines, a no-op costing one branch when no tool is attached.
struct NvtxRange {
	explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
	~NvtxRange() { nvtxRangePop(); }
	NvtxRange(const NvtxRange&) = delete;
	NvtxRange& operator=(const NvtxRange&) = delete;
};

// Records `msg` as this thread's last error and returns `status`. The reference logs and
// continues on errors (cuda_ray_tracer/CudaHelpers.hpp:13-25); this library reports them instead.
phe_status fail(phe_status status, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
void clear_error();

} // namespace phe_gb300
