// asv_eval.cu -- supervoxel quality measures against a ground-truth
// segmentation (the LIBSVX benchmark the reference is evaluated with,
// README.md:26-28: "3D undersegmentation error", "3D segmentation accuracy",
// "3D boundary recall", mean duration; Xu & Corso, "Evaluation of super-voxel
// methods for early video processing", CVPR 2012).  LIBSVX's own code is not
// available here; the definitions implemented are stated in asv.h.
//
// The device counts: the overlap matrix n[s][g] (supervoxel s, truth segment
// g), each supervoxel's first and last frame, the truth boundary voxels and
// how many of them have a supervoxel boundary within one voxel.  The host
// turns the counts into the measures.
#include "asv_eval.cuh"

#define EV_T 256

#define EV_RANGE_PER_THREAD 8

// label ranges and bounds violations: a block reduces EV_T * 8 voxels (warp
// reductions, then the block's warps through shared memory) and issues one
// atomic per quantity, so the three global words see few updates
__global__ void k_ev_range(const int32_t *__restrict__ lab, const int32_t *__restrict__ gt, long long n, int *meta)
{
    __shared__ int red[3][EV_T / 32];
    const long long base = (long long)blockIdx.x * blockDim.x * EV_RANGE_PER_THREAD + threadIdx.x;
    int ls = -1, lg = -1, bad = 0;
#pragma unroll
    for (int k = 0; k < EV_RANGE_PER_THREAD; k++) {
        const long long v = base + (long long)k * blockDim.x;
        if (v < n) {
            const int a = lab[v], b = gt[v];
            ls = max(ls, a);
            lg = max(lg, b);
            bad |= (a < -1 || a >= EV_MAX_LABELS || b < 0 || b >= EV_MAX_TRUTH) ? 1 : 0;
        }
    }
    ls = __reduce_max_sync(0xffffffffu, ls);
    lg = __reduce_max_sync(0xffffffffu, lg);
    bad = __reduce_or_sync(0xffffffffu, bad);
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        red[0][w] = ls;
        red[1][w] = lg;
        red[2][w] = bad;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 1; i < EV_T / 32; i++) {
            ls = max(ls, red[0][i]);
            lg = max(lg, red[1][i]);
            bad |= red[2][i];
        }
        atomicMax(meta + 0, ls);
        atomicMax(meta + 1, lg);
        if (bad) atomicOr(meta + 2, 1);
    }
}

// overlap counts (label -1 is row 0) and per-supervoxel frame range; lanes
// with the same (s, g) pair form one group, whose leader adds the group's
// count and its frame range once
__global__ void k_ev_overlap(const int32_t *__restrict__ lab, const int32_t *__restrict__ gt, int W, int H, int D,
                             int NG, unsigned *__restrict__ cnt, int *__restrict__ zmin, int *__restrict__ zmax)
{
    const long long fr = (long long)W * H, n = fr * D;
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = v < n;
    const int s = in ? lab[v] + 1 : 0, g = in ? gt[v] : 0;
    const int key = in ? s * NG + g : -1;
    const unsigned grp = __match_any_sync(0xffffffffu, key);
    const unsigned z = in ? (unsigned)(v / fr) : 0u;
    const unsigned zlo = __reduce_min_sync(grp, z), zhi = __reduce_max_sync(grp, z);
    if (in && (int)(threadIdx.x & 31) == __ffs(grp) - 1) {
        atomicAdd(cnt + key, (unsigned)__popc(grp));
        if (s > 0) {
            atomicMin(zmin + s, (int)zlo);
            atomicMax(zmax + s, (int)zhi);
        }
    }
}

// supervoxel boundary flags: a voxel with a 6-neighbour of another label
__global__ void k_ev_sbound(const int32_t *__restrict__ lab, int W, int H, int D, uint8_t *__restrict__ sb)
{
    const long long fr = (long long)W * H, n = fr * D;
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const int z = (int)(v / fr), p = (int)(v - z * fr), y = p / W, x = p - y * W;
    const int l = lab[v];
    bool b = false;
    if (x > 0) b |= lab[v - 1] != l;
    if (x < W - 1) b |= lab[v + 1] != l;
    if (y > 0) b |= lab[v - W] != l;
    if (y < H - 1) b |= lab[v + W] != l;
    if (z > 0) b |= lab[v - fr] != l;
    if (z < D - 1) b |= lab[v + fr] != l;
    sb[v] = b ? 1 : 0;
}

// truth boundary voxels, and those with a supervoxel boundary voxel in their
// 3x3x3 neighbourhood
__global__ void k_ev_recall(const int32_t *__restrict__ gt, const uint8_t *__restrict__ sb, int W, int H, int D,
                            unsigned long long *__restrict__ tot)
{
    const long long fr = (long long)W * H, n = fr * D;
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned isb = 0, rec = 0;
    if (v < n) {
        const int z = (int)(v / fr), p = (int)(v - z * fr), y = p / W, x = p - y * W;
        const int g = gt[v];
        bool b = false;
        if (x > 0) b |= gt[v - 1] != g;
        if (x < W - 1) b |= gt[v + 1] != g;
        if (y > 0) b |= gt[v - W] != g;
        if (y < H - 1) b |= gt[v + W] != g;
        if (z > 0) b |= gt[v - fr] != g;
        if (z < D - 1) b |= gt[v + fr] != g;
        if (b) {
            isb = 1;
            for (int dz = -1; dz <= 1 && !rec; dz++) {
                const int zz = z + dz;
                if (zz < 0 || zz >= D) continue;
                for (int dy = -1; dy <= 1 && !rec; dy++) {
                    const int yy = y + dy;
                    if (yy < 0 || yy >= H) continue;
                    for (int dx = -1; dx <= 1; dx++) {
                        const int xx = x + dx;
                        if (xx < 0 || xx >= W) continue;
                        if (sb[fr * zz + (long long)yy * W + xx]) { rec = 1; break; }
                    }
                }
            }
        }
    }
    isb = __reduce_add_sync(0xffffffffu, isb);
    rec = __reduce_add_sync(0xffffffffu, rec);
    __shared__ unsigned red[2][EV_T / 32];                 // then the block's warps: one atomic pair per block
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        red[0][w] = isb;
        red[1][w] = rec;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 1; i < EV_T / 32; i++) {
            isb += red[0][i];
            rec += red[1][i];
        }
        if (isb) {
            atomicAdd(tot + 0, (unsigned long long)isb);
            atomicAdd(tot + 1, (unsigned long long)rec);
        }
    }
}

static unsigned ev_blocks(long long n) { return (unsigned)((n + EV_T - 1) / EV_T); }

int asv_launch_eval_range(const int32_t *lab, const int32_t *gt, long long n, int *meta, cudaStream_t st)
{
    cudaMemsetAsync(meta, 0xff, 2 * sizeof(int), st);       // -1
    cudaMemsetAsync(meta + 2, 0, sizeof(int), st);
    k_ev_range<<<(unsigned)((n + EV_T * EV_RANGE_PER_THREAD - 1) / (EV_T * EV_RANGE_PER_THREAD)), EV_T, 0, st>>>(
        lab, gt, n, meta);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int asv_launch_eval(const int32_t *lab, const int32_t *gt, int W, int H, int D, int rows, int NG, unsigned *cnt,
                    int *zmin, int *zmax, uint8_t *sb, unsigned long long *tot, cudaStream_t st)
{
    const long long n = (long long)W * H * D;
    cudaMemsetAsync(cnt, 0, sizeof(unsigned) * (size_t)rows * NG, st);
    cudaMemsetAsync(zmin, 0x7f, sizeof(int) * (size_t)rows, st);      // large
    cudaMemsetAsync(zmax, 0xff, sizeof(int) * (size_t)rows, st);      // -1
    cudaMemsetAsync(tot, 0, 2 * sizeof(unsigned long long), st);
    k_ev_overlap<<<ev_blocks(n), EV_T, 0, st>>>(lab, gt, W, H, D, NG, cnt, zmin, zmax);
    k_ev_sbound<<<ev_blocks(n), EV_T, 0, st>>>(lab, W, H, D, sb);
    k_ev_recall<<<ev_blocks(n), EV_T, 0, st>>>(gt, sb, W, H, D, tot);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}
