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

// label ranges and bounds violations
__global__ void k_ev_range(const int32_t *__restrict__ lab, const int32_t *__restrict__ gt, long long n, int *meta)
{
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int ls = -1, lg = -1, bad = 0;
    if (v < n) {
        ls = lab[v];
        lg = gt[v];
        bad = (ls < -1 || ls >= EV_MAX_LABELS || lg < 0 || lg >= EV_MAX_TRUTH) ? 1 : 0;
    }
    ls = __reduce_max_sync(0xffffffffu, ls);
    lg = __reduce_max_sync(0xffffffffu, lg);
    bad = __reduce_or_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31) == 0) {
        atomicMax(meta + 0, ls);
        atomicMax(meta + 1, lg);
        if (bad) atomicOr(meta + 2, 1);
    }
}

// overlap counts (label -1 is row 0) and per-supervoxel frame range; lanes
// with the same (s, g) pair add once per warp
__global__ void k_ev_overlap(const int32_t *__restrict__ lab, const int32_t *__restrict__ gt, int W, int H, int D,
                             int NG, unsigned *__restrict__ cnt, int *__restrict__ zmin, int *__restrict__ zmax)
{
    const long long fr = (long long)W * H, n = fr * D;
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = v < n;
    const int s = in ? lab[v] + 1 : 0, g = in ? gt[v] : 0;
    const int key = in ? s * NG + g : -1;
    const unsigned grp = __match_any_sync(0xffffffffu, key);
    const int lead = __ffs(grp) - 1;
    if (in && (int)(threadIdx.x & 31) == lead) atomicAdd(cnt + key, (unsigned)__popc(grp));
    if (in && s > 0) {
        const int z = (int)(v / fr);
        atomicMin(zmin + s, z);
        atomicMax(zmax + s, z);
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
    if ((threadIdx.x & 31) == 0 && isb) {
        atomicAdd(tot + 0, (unsigned long long)isb);
        atomicAdd(tot + 1, (unsigned long long)rec);
    }
}

static unsigned ev_blocks(long long n) { return (unsigned)((n + EV_T - 1) / EV_T); }

int asv_launch_eval_range(const int32_t *lab, const int32_t *gt, long long n, int *meta, cudaStream_t st)
{
    cudaMemsetAsync(meta, 0xff, 2 * sizeof(int), st);       // -1
    cudaMemsetAsync(meta + 2, 0, sizeof(int), st);
    k_ev_range<<<ev_blocks(n), EV_T, 0, st>>>(lab, gt, n, meta);
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
