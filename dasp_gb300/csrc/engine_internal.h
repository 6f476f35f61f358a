// Engine entry points for the native runtime parts of the library (the
// serving loop) that drive handles directly, below the C ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/shwfs.h"

namespace shwfs {

// one frame through the integration state machine (py_run,
// cmod/src/centmodule.c:3188-3229) with the phase at a device pointer and the
// handle's own device-resident cents/bimg; queued on st, not waited for.
// *readout = 1 when the frame was a readout frame (outputs written).
shwfs_status engine_frame(shwfs_handle* h, const float* phs_dev, cudaStream_t st, int* readout);
// bytes of device memory the handle holds
int64_t engine_device_bytes(const shwfs_handle* h);
// device status word of the handle's kernels (bit 1: reference sampler
// limit, bit 2: tensor-core wait timed out)
const int* engine_status_ptr(const shwfs_handle* h);
int engine_nsubaps(const shwfs_handle* h);
// set the calling thread's shwfs_last_error() message; returns st
shwfs_status engine_fail(shwfs_status st, const char* msg);

}  // namespace shwfs
