// asv_stream.cu -- device side of the streaming form
// (streamGPU-AS/Render.cpp:348-569): the seeds carried from one block to the
// next, the block-local -> video-wide id map, and the labels of the finished
// frames, all kept on the device between blocks.
#include "asv_common.cuh"
#include "asv_stream.cuh"

#define FULL 0xffffffffu

// Seed table of a block: the kept seeds of the previous block first, then the
// Kn new seeds the density placement wrote to pos0[0..Kn)
// (Render.cpp:434-460), and the id map of the block (block2all, :443-458).
// One block of 1024 threads; uses the (no longer needed) grid array as
// scratch for the new seeds.
__global__ void __launch_bounds__(1024) k_stream_compose(AsvDev d, StreamDev s, int Kn, int Kcap)
{
    const int kept = s.ctr[STREAM_KEPT], placed = s.ctr[STREAM_PLACED];
    SegDesc *seg = const_cast<SegDesc *>(d.segs);           // the block's seed count is set here, on the device
    const bool short_grid = d.post[POST_VALID] != Kn;
    if (short_grid || kept + Kn > Kcap) {
        // fewer placed seeds than the grid, or over capacity: the block runs
        // with no seeds and leaves the stream's state alone; the host reports it
        if (threadIdx.x == 0) {
            s.ctr[STREAM_KP] = short_grid ? -2 : -1;
            seg[0].Kp = 0;
        }
        return;
    }
    float4 *tmp = d.grid;
    for (int i = threadIdx.x; i < Kn; i += blockDim.x) tmp[i] = d.pos0[i];
    __syncthreads();
    for (int i = threadIdx.x; i < kept; i += blockDim.x) {
        float4 k = s.kept_pos[i];
        d.pos0[i] = make_float4(k.x, k.y, k.z, (float)i);
        s.gmap_cur[i] = s.gmap_prev[(int)k.w];
    }
    for (int i = threadIdx.x; i < Kn; i += blockDim.x) {
        float4 p = tmp[i];
        d.pos0[kept + i] = make_float4(p.x, p.y, p.z, (float)(kept + i));
        s.gmap_cur[kept + i] = placed + i;
    }
    if (threadIdx.x == 0) {
        s.ctr[STREAM_KP] = kept + Kn;
        seg[0].Kp = kept + Kn;
    }
}

// After a block: final centroids of the alive seeds
// (streamGPU-AS/Image.cpp:1563-1582), the seeds kept for the next block
// (z > block_size - one_third, shifted by two_third, minimum 1.5;
// Render.cpp:519-541) in seed order, and seeds_num_placed (:514).
__global__ void __launch_bounds__(1024) k_stream_next(AsvDev d, StreamDev s, float z_keep,
                                                      float z_shift, int keep)
{
    if (s.ctr[STREAM_KP] < 0) return;                        // a refused block: the state stays
    const SegDesc &S = d.segs[0];
    const int Kp = S.Kp;
    const unsigned long long *sums = d.sums + 8ull * S.seed_off;
    __shared__ int wt[2][32];
    __shared__ int carry[2];
    const int kept_in = s.ctr[STREAM_KEPT];
    if (threadIdx.x < 2) carry[threadIdx.x] = 0;
    __syncthreads();
    for (int b0 = 0; b0 < Kp; b0 += blockDim.x) {
        const int i = b0 + threadIdx.x;
        int area = 0;
        float c[3] = { 0, 0, 0 };
        if (i < Kp) {
            area = (int)sums[8ull * i + 3];
            if (area >= 1)
                for (int a = 0; a < 3; a++) {
                    float sf = __ull2float_rn(sums[8ull * i + a]) * 0.5f;
                    c[a] = (float)((double)floorf(sf / (float)area) + 0.5);
                }
        }
        const int alive = area >= 1 ? 1 : 0;
        const int kp = (keep && alive && c[2] > z_keep) ? 1 : 0;
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        const unsigned ba = __ballot_sync(FULL, alive), bk = __ballot_sync(FULL, kp);
        if (lane == 0) { wt[0][w] = __popc(ba); wt[1][w] = __popc(bk); }
        __syncthreads();
        if (threadIdx.x < 32) {
            for (int t = 0; t < 2; t++) {
                int v = wt[t][threadIdx.x], incl = v;
                for (int o = 1; o < 32; o <<= 1) {
                    int m = __shfl_up_sync(FULL, incl, o);
                    if (threadIdx.x >= o) incl += m;
                }
                wt[t][threadIdx.x] = incl - v;
            }
        }
        __syncthreads();
        if (kp) {
            const int j = carry[1] + wt[1][w] + __popc(bk & ((1u << lane) - 1u));
            float nz = c[2] - z_shift;
            if (nz < 1) nz = 1.5f;
            s.kept_next[j] = make_float4(c[0], c[1], nz, (float)i);
        }
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) {
            carry[0] += wt[0][w] + __popc(ba & ((1u << lane) - 1u)) + alive;
            carry[1] += wt[1][w] + __popc(bk & ((1u << lane) - 1u)) + kp;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        s.ctr[STREAM_NAL] = carry[0];
        s.ctr[STREAM_PLACED] += carry[0] - kept_in;
        s.ctr[STREAM_KEPT] = keep ? carry[1] : 0;
    }
}

// video-wide labels of the finished frames: block2all[label] (-1 -> 0,
// Render.cpp:559-563)
__global__ void __launch_bounds__(256) k_stream_map(AsvDev d, StreamDev s, long long n)
{
    const SegDesc &S = d.segs[0];
    const int32_t *post = (S.final_buf ? d.labA : d.labB) + S.vox_off;
    long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n || s.ctr[STREAM_KP] < 0) return;
    int l = post[v];
    s.lab_out[v] = (l >= 0 && l < S.Kp) ? s.gmap_cur[l] : 0;
}

void asv_launch_stream_compose(const AsvDev &d, const StreamDev &s, int Kn, int Kcap, cudaStream_t st)
{
    k_stream_compose<<<1, 1024, 0, st>>>(d, s, Kn, Kcap);
}

void asv_launch_stream_next(const AsvDev &d, const StreamDev &s, float z_keep, float z_shift, int keep,
                            cudaStream_t st)
{
    k_stream_next<<<1, 1024, 0, st>>>(d, s, z_keep, z_shift, keep);
}

void asv_launch_stream_map(const AsvDev &d, const StreamDev &s, long long n, cudaStream_t st)
{
    k_stream_map<<<(int)((n + 255) / 256), 256, 0, st>>>(d, s, n);
}

// device-to-device copy of 16-byte words on the SMs
__global__ void __launch_bounds__(256) k_copy16(const uint4 *__restrict__ src, uint4 *__restrict__ dst, size_t n)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

// A block's device-to-device copies (the overlap shift, the staging of fed
// frames) as a kernel when both ends and the size are 16-byte aligned, so
// they do not queue on a copy engine behind the next block's upload from
// the host; a cudaMemcpyAsync otherwise.
cudaError_t asv_copy_d2d(void *dst, const void *src, size_t bytes, cudaStream_t st)
{
    if (!bytes) return cudaSuccess;
    const uintptr_t a = (uintptr_t)dst, b = (uintptr_t)src;
    const bool apart = a + bytes <= b || b + bytes <= a;
    if (apart && ((a | b | bytes) & 15u) == 0) {
        const size_t n = bytes / 16;
        int sms = 0, dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const size_t want = (n + 255) / 256, cap = (size_t)(sms > 0 ? sms : 1) * 8;
        k_copy16<<<(unsigned)(want < cap ? want : cap), 256, 0, st>>>((const uint4 *)src, (uint4 *)dst, n);
        return cudaGetLastError();
    }
    return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st);
}
