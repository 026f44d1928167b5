// asv_stream.cuh -- state of the streaming form kept on the device between
// blocks (the seeds carried over, the id maps, counters, label staging).
#pragma once

#include "asv_common.cuh"

enum { STREAM_KEPT = 0, STREAM_PLACED = 1, STREAM_KP = 2, STREAM_NAL = 3, STREAM_CTR_WORDS = 8 };

struct StreamDev {
    float4 *kept_pos;    // seeds carried into the current block: (x, y, z, id in the previous block)
    float4 *kept_next;   // seeds the current block carries into the next one
    int *gmap_prev;      // previous block's block-local -> video id map
    int *gmap_cur;       // current block's map
    int *ctr;            // STREAM_* counters
    int32_t *lab_out;    // video-wide labels of the finished frames
};

void asv_launch_stream_compose(const AsvDev &d, const StreamDev &s, int Kn, int Kcap, cudaStream_t st);
void asv_launch_stream_next(const AsvDev &d, const StreamDev &s, float z_keep, float z_shift, int keep,
                            cudaStream_t st);
void asv_launch_stream_map(const AsvDev &d, const StreamDev &s, long long n, cudaStream_t st);
cudaError_t asv_copy_d2d(void *dst, const void *src, size_t bytes, cudaStream_t st);
