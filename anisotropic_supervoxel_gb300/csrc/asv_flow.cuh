// asv_flow.cuh -- dense optical flow on the device (asv_flow.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

// device scratch bytes for a W x H x D clip
size_t asv_flow_scratch_bytes(int W, int H, int D);

// forward (z -> z+1) and backward (z -> z-1) flow of the RGB8 clip `rgb`
// (device, [D][H][W][3]) into the interleaved volumes fwd / bwd (device,
// [D][H][W] float2; fwd of the last frame and bwd of the first are zero,
// unless keep_first_bwd leaves the first frame's bwd as it is).  Returns 0,
// or -1 on a CUDA error.  Asynchronous on `st`.
int asv_launch_flow(const uint8_t *rgb, int W, int H, int D, float2 *fwd, float2 *bwd, void *scratch,
                    cudaStream_t st, int keep_first_bwd = 0);
