// trace_launch.h — host-side launchers of the traversal kernels.
#pragma once

#include <cuda_runtime.h>

#include "../../include/walkray.h"
#include "wr_device.cuh"

namespace wr {

// k_trace_closest over n rays (n x 6 floats on the device).  d_inside /
// d_contact NULL = unfiltered.  d_counter (one u64) and d_err (one u32) are
// device scratch words; d_err gets bit 0 on a stack overflow (never expected:
// the stack is sized from the tree depth).
cudaError_t launch_trace_closest(const DevTree& T, const float* d_rays, uint64_t n, const int32_t* d_inside,
                                 const int32_t* d_contact, wr_hit* d_hits, unsigned long long* d_counter,
                                 unsigned int* d_err, int num_sms, bool prune, cudaStream_t stream,
                                 int* launched_blocks, const TraceTune* tune = nullptr, int ctas_per_sm = 0);

}  // namespace wr
