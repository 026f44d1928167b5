// asv_eval.cuh -- supervoxel quality measures on the device (asv_eval.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define EV_MAX_LABELS 32768     // supervoxel labels -1 .. 32767
#define EV_MAX_TRUTH 4096       // truth ids 0 .. 4095

// meta[0] = largest label, meta[1] = largest truth id, meta[2] = 1 when a
// value is out of range.  Asynchronous on st.
int asv_launch_eval_range(const int32_t *lab, const int32_t *gt, long long n, int *meta, cudaStream_t st);

// counts for rows = largest label + 2 (row 0 = label -1) and NG truth ids:
// cnt[rows][NG], zmin/zmax[rows], sb (n bytes scratch), tot[2] = truth
// boundary voxels, recalled ones.  Asynchronous on st.
int asv_launch_eval(const int32_t *lab, const int32_t *gt, int W, int H, int D, int rows, int NG, unsigned *cnt,
                    int *zmin, int *zmax, uint8_t *sb, unsigned long long *tot, cudaStream_t st);
