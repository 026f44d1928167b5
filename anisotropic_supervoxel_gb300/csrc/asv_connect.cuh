// asv_connect.cuh -- 3D connectivity enforcement on the device (asv_connect.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

// device scratch bytes for a W*H*D = n volume
size_t asv_connect_scratch_bytes(long long n);

// Connected segments of `lab` (device, n = W*H*D) relabelled as
// Image::EnforceLabelConnectivity3D does, into `out` (device).  Synchronizes
// `st`.  Returns 0, -1 on a CUDA error, -2 when a union-find retry bound was
// exceeded, -3 for more than 2^30 segments; *host_R = segments found,
// *host_num = labels after merging.
int asv_launch_connect(const int32_t *lab, int W, int H, int D, int supsz, int32_t *out, void *scratch,
                       cudaStream_t st, int *host_R, int *host_num);
