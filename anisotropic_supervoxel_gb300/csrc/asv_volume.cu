// asv_volume.cu -- per-voxel and per-seed kernels of the supervoxel path.
//
// Compiled with -fmad=false: every float operation is one IEEE operation in
// the order written, so the labels match the CPU restatement bit for bit.
// Reference files (in dongxiao0401/anisotropic_supervoxel): GPU-AS/shaders/*,
// GPU-AS/Image.cpp.
#include "asv_common.cuh"

#include <cuda_fp16.h>

#include <mutex>

#define FULL 0xffffffffu

// ---------------------------------------------------------------------------
// RGB -> LAB (GPU-AS/shaders/RGB2LAB.fs:11-79).  Output bytes are the
// integers the shader writes to its RGB16F target (exact in 8 bits).
// ---------------------------------------------------------------------------
__device__ __forceinline__ float asv_pow_cr(float x, float y)
{
    return (float)pow((double)x, (double)y);
}

__global__ void k_srgb_table(float *__restrict__ tab)
{
    int c = threadIdx.x;
    if (c >= 256) return;
    float v = (float)c / 255.0f;                      // unorm8 texel
    float t;
    if (v <= 0.04045f) t = v / 12.92f;                 // RGB2LAB.fs:27-40
    else t = asv_pow_cr((v + 0.055f) / 1.055f, 2.4f);
    tab[c] = t;
}

// distance of x + 0.5 to the nearest integer (where floor(x + 0.5) can flip)
__device__ __forceinline__ float asv_tie_gap(float x)
{
    float y = x + 0.5f;
    return fabsf(y - rintf(y));
}

// The cube root f = r^(1/3) is first taken in FP32 (exp2/log2, error below
// 1e-6 relative, i.e. below 6e-4 on the scaled L, a, b); only when a scaled
// value lies within 4e-3 of a rounding boundary is the voxel recomputed with
// the correctly rounded FP64 path, so the bytes equal the exact ones.
// asv_lab_of_fp32 is the first part alone: it returns the FP32 bytes and
// whether asv_lab_of would recompute them.
__device__ __forceinline__ bool asv_lab_of_fp32(const float *__restrict__ tab, unsigned r, unsigned g, unsigned b,
                                                uchar4 &out)
{
    float t0 = tab[r], t1 = tab[g], t2 = tab[b];
    float X = (t0 * 0.412453f + t1 * 0.357580f) + t2 * 0.180423f;
    float Y = (t0 * 0.212671f + t1 * 0.715160f) + t2 * 0.072169f;
    float Z = (t0 * 0.019334f + t1 * 0.119193f) + t2 * 0.950227f;
    float rr[3] = { X / 0.950456f, Y / 1.0f, Z / 1.088754f };
    float f[3];
    bool cube[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        cube[k] = rr[k] > 0.008856f;
        if (cube[k]) f[k] = exp2f(log2f(rr[k]) * (1.0f / 3.0f));
        else f[k] = (903.3f * rr[k] + 16.0f) / 116.0f;
    }
    float L = 116.0f * f[1] - 16.0f;
    float A = 500.0f * (f[0] - f[1]);
    float B = 200.0f * (f[1] - f[2]);
    L = L * 2.55f; A = A + 128.0f; B = B + 128.0f;
    const bool fix = (cube[0] || cube[1] || cube[2]) &&
                     fminf(asv_tie_gap(L), fminf(asv_tie_gap(A), asv_tie_gap(B))) < 4e-3f;
    float v0 = floorf(L + 0.5f), v1 = floorf(A + 0.5f), v2 = floorf(B + 0.5f);
    v0 = fminf(fmaxf(v0, 0.0f), 255.0f);
    v1 = fminf(fmaxf(v1, 0.0f), 255.0f);
    v2 = fminf(fmaxf(v2, 0.0f), 255.0f);
    out = make_uchar4((unsigned char)v0, (unsigned char)v1, (unsigned char)v2, 0);
    return fix;
}

__device__ __forceinline__ uchar4 asv_lab_of(const float *__restrict__ tab, unsigned r, unsigned g,
                                             unsigned b)
{
    float t0 = tab[r], t1 = tab[g], t2 = tab[b];
    float X = (t0 * 0.412453f + t1 * 0.357580f) + t2 * 0.180423f;   // fs:19-21, 42-44
    float Y = (t0 * 0.212671f + t1 * 0.715160f) + t2 * 0.072169f;
    float Z = (t0 * 0.019334f + t1 * 0.119193f) + t2 * 0.950227f;
    float rr[3] = { X / 0.950456f, Y / 1.0f, Z / 1.088754f };        // fs:54-55
    float f[3];
    bool cube[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        cube[k] = rr[k] > 0.008856f;                                   // fs:57-70
        if (cube[k]) f[k] = exp2f(log2f(rr[k]) * (1.0f / 3.0f));
        else f[k] = (903.3f * rr[k] + 16.0f) / 116.0f;
    }
    float L = 116.0f * f[1] - 16.0f;                                  // fs:72
    float A = 500.0f * (f[0] - f[1]);
    float B = 200.0f * (f[1] - f[2]);
    L = L * 2.55f; A = A + 128.0f; B = B + 128.0f;                    // fs:74-76
    if ((cube[0] || cube[1] || cube[2]) &&
        fminf(asv_tie_gap(L), fminf(asv_tie_gap(A), asv_tie_gap(B))) < 4e-3f) {
#pragma unroll
        for (int k = 0; k < 3; k++)
            if (cube[k]) f[k] = asv_pow_cr(rr[k], 1.0f / 3.0f);
        L = 116.0f * f[1] - 16.0f;
        A = 500.0f * (f[0] - f[1]);
        B = 200.0f * (f[1] - f[2]);
        L = L * 2.55f; A = A + 128.0f; B = B + 128.0f;
    }
    float v0 = floorf(L + 0.5f), v1 = floorf(A + 0.5f), v2 = floorf(B + 0.5f);
    v0 = fminf(fmaxf(v0, 0.0f), 255.0f);
    v1 = fminf(fmaxf(v1, 0.0f), 255.0f);
    v2 = fminf(fmaxf(v2, 0.0f), 255.0f);
    return make_uchar4((unsigned char)v0, (unsigned char)v1, (unsigned char)v2, 0);
}

__global__ void __launch_bounds__(256) k_rgb2lab(AsvDev d)
{
    __shared__ float tab[256];
    tab[threadIdx.x] = d.srgb[threadIdx.x];
    __syncthreads();
    int si = asv_find_seg(d.chunk_prefix, d.nseg, blockIdx.x);
    const SegDesc &S = d.segs[si];
    long long base = (long long)(blockIdx.x - d.chunk_prefix[si]) * ASV_CHUNK;
    long long n = S.nvox;
    if (base + ASV_CHUNK <= S.lab_from) return;
    for (int i = 0; i < ASV_CHUNK / 256; i++) {
        long long v = base + i * 256 + threadIdx.x;
        if (v >= n) break;
        const uint8_t *p = d.rgb + 3 * (S.vox_off + v);
        d.lab[S.vox_off + v] = asv_lab_of(tab, p[0], p[1], p[2]);
    }
}

// The LAB bytes of all 2^24 RGB values, indexed r << 16 | g << 8 | b, built
// once per device in two passes: every entry in FP32, the entries near a
// rounding tie listed (about 2 %), then those entries again by asv_lab_of
// itself.  So a lookup returns exactly what the computation would (the
// exhaustive RGB2LAB test covers every entry), and the FP64 recomputations
// run in full warps instead of stalling half of all warps on one lane each.
__global__ void __launch_bounds__(256) k_lab_table(const float *__restrict__ srgb, uchar4 *__restrict__ lut,
                                                   unsigned *__restrict__ fix, unsigned *__restrict__ nfix)
{
    __shared__ float tab[256];
    tab[threadIdx.x] = srgb[threadIdx.x];
    __syncthreads();
    const unsigned c = blockIdx.x * 256u + threadIdx.x;              // 65536 blocks x 256
    uchar4 v;
    const bool again = asv_lab_of_fp32(tab, c >> 16, (c >> 8) & 255u, c & 255u, v);
    lut[c] = v;
    const unsigned m = __ballot_sync(0xffffffffu, again);            // one atomic per warp
    if (!m) return;
    const int lane = threadIdx.x & 31;
    unsigned at = 0;
    if (lane == __ffs(m) - 1) at = atomicAdd(nfix, (unsigned)__popc(m));
    at = __shfl_sync(0xffffffffu, at, __ffs(m) - 1);
    if (again) fix[at + __popc(m & ((1u << lane) - 1u))] = c;
}

__global__ void __launch_bounds__(256) k_lab_table_fix(const float *__restrict__ srgb, uchar4 *__restrict__ lut,
                                                       const unsigned *__restrict__ fix,
                                                       const unsigned *__restrict__ nfix)
{
    __shared__ float tab[256];
    tab[threadIdx.x] = srgb[threadIdx.x];
    __syncthreads();
    const unsigned n = *nfix;
    for (unsigned i = blockIdx.x * 256u + threadIdx.x; i < n; i += gridDim.x * 256u) {
        const unsigned c = fix[i];
        lut[c] = asv_lab_of(tab, c >> 16, (c >> 8) & 255u, c & 255u);
    }
}

// RGB -> LAB through the table: one 4-byte gather per voxel
__global__ void __launch_bounds__(256) k_rgb2lab_lut(AsvDev d)
{
    int si = asv_find_seg(d.chunk_prefix, d.nseg, blockIdx.x);
    const SegDesc &S = d.segs[si];
    long long base = (long long)(blockIdx.x - d.chunk_prefix[si]) * ASV_CHUNK;
    long long n = S.nvox;
    if (base + ASV_CHUNK <= S.lab_from) return;
    const uchar4 *__restrict__ lut = d.lablut;
    for (int i = 0; i < ASV_CHUNK / 256; i++) {
        long long v = base + i * 256 + threadIdx.x;
        if (v >= n) break;
        const uint8_t *p = d.rgb + 3 * (S.vox_off + v);
        d.lab[S.vox_off + v] = __ldg(lut + (((unsigned)p[0] << 16) | ((unsigned)p[1] << 8) | p[2]));
    }
}

// ---------------------------------------------------------------------------
// Render::cvMat2TexureInput (GPU-AS/Render.cpp:354-359) for raw frames (BGR8,
// top row first): 3x3 Gaussian blur with sigma 0 (the [1,2,1] x [1,2,1] / 16
// kernel, border reflect-101, rounded half up), BGR -> RGB and the vertical
// flip into texture orientation.  One thread per output pixel and frame;
// the same integer arithmetic as the host asv_preprocess_frame.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int asv_reflect101(int i, int n)
{
    if (n == 1) return 0;
    while (i < 0 || i >= n) i = i < 0 ? -i : 2 * n - 2 - i;
    return i;
}

__global__ void k_preprocess(const uint8_t *__restrict__ bgr, uint8_t *__restrict__ rgb, int W, int H, int D)
{
    const long long fr = (long long)W * H;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= fr * D) return;
    const int z = (int)(t / fr), p = (int)(t - (long long)z * fr);
    const int yo = p / W, x = p - yo * W, y = H - 1 - yo;          // output row yo <- source row y
    const uint8_t *src = bgr + 3 * fr * z;
    int acc[3] = { 0, 0, 0 };
    for (int j = -1; j <= 1; j++) {
        const int yy = asv_reflect101(y + j, H);
        const int wy = j == 0 ? 2 : 1;
        for (int i = -1; i <= 1; i++) {
            const int xx = asv_reflect101(x + i, W);
            const int wgt = wy * (i == 0 ? 2 : 1);
            const uint8_t *q = src + 3 * ((long long)yy * W + xx);
            acc[0] += wgt * q[0];
            acc[1] += wgt * q[1];
            acc[2] += wgt * q[2];
        }
    }
    uint8_t *o = rgb + 3 * t;
    o[0] = (uint8_t)((acc[2] + 8) >> 4);                             // R <- channel 2 of BGR
    o[1] = (uint8_t)((acc[1] + 8) >> 4);
    o[2] = (uint8_t)((acc[0] + 8) >> 4);
}

void asv_launch_preprocess(const uint8_t *bgr, uint8_t *rgb, int W, int H, int D, cudaStream_t st)
{
    const long long n = (long long)W * H * D;
    k_preprocess<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(bgr, rgb, W, H, D);
}

// ---------------------------------------------------------------------------
// Gradient density per grid cell (GPU-AS/Image.cpp:350-620,
// derivative_t.gs:24-49, density_grid.vs:17-43).  Each voxel's gradient is
// rounded to half (RGB16F target) and summed exactly, in units of 2^-24.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float asv_gradient(const uint8_t *__restrict__ rgb, int W, int H, int x,
                                              int y, int z)
{
    long long row = (long long)W;
    long long sl = (long long)W * H;
    long long v = z * sl + y * row + x;
    const uint8_t *c = rgb + 3 * v;
    const uint8_t *nb0 = rgb + 3 * (v - (x > 0 ? 1 : 0));
    const uint8_t *nb1 = rgb + 3 * (v - (y > 0 ? row : 0));
    const uint8_t *nb2 = rgb + 3 * (v - (z > 0 ? sl : 0));
    const uint8_t *nbs[3] = { nb0, nb1, nb2 };
    float g = 0.0f;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const uint8_t *q = nbs[k];
        float s = (float)abs((int)q[0] - (int)c[0]);
        s = s + (float)abs((int)q[1] - (int)c[1]);
        s = s + (float)abs((int)q[2] - (int)c[2]);
        g = g + 0.33f * s;                                            // gs:36, 43, 49
    }
    return g;
}

// value of a non-negative half in units of 2^-24
__device__ __forceinline__ unsigned long long asv_half_units(__half h)
{
    unsigned short b = __half_as_ushort(h);
    unsigned e = (b >> 10) & 0x1fu, m = b & 0x3ffu;
    if (e == 0) return m;
    return (unsigned long long)(1024u + m) << (e - 1);
}

__global__ void __launch_bounds__(256) k_density(AsvDev d)
{
    int si = asv_find_seg(d.chunk_prefix, d.nseg, blockIdx.x);
    const SegDesc &S = d.segs[si];
    const int W = S.W, H = S.H;
    const int *xc = d.cells + S.cell_off, *yc = xc + W, *zc = yc + H;
    const uint8_t *rgb = d.rgb + 3 * S.vox_off;
    unsigned long long *acc = d.dacc + S.seed_off;
    const int cap = d.seed_prefix[si + 1] - S.seed_off;
    long long base = (long long)(blockIdx.x - d.chunk_prefix[si]) * ASV_CHUNK;
    for (int i = 0; i < ASV_CHUNK / 256; i++) {
        long long v = base + i * 256 + threadIdx.x;
        int key = -1;
        unsigned u32 = 0;
        if (v < S.nvox) {
            int x = (int)(v % W);
            long long r = v / W;
            int y = (int)(r % H), z = (int)(r / H);
            int cx = xc[x], cy = yc[y], cz = zc[z];
            if (cx >= 0 && cy >= 0 && cz >= 0) {
                int k = (cz * S.hNum + cy) * S.wNum + cx;
                // cell id stored in an R16F texture (Image.cpp:474)
                int slot = (int)__half2float(__float2half_rn((float)k));
                unsigned long long units = asv_half_units(__float2half_rn(asv_gradient(rgb, W, H, x, y, z)));
                if (slot < cap) {
                    if ((units & 0xfffull) == 0 && (units >> 12) < (1ull << 26)) {
                        key = slot;
                        u32 = (unsigned)(units >> 12);
                    } else {
                        atomicAdd(acc + slot, units);
                    }
                }
            }
        }
        unsigned grp = __match_any_sync(FULL, key);
        unsigned sum = __reduce_add_sync(grp, u32);
        if (key >= 0 && (threadIdx.x & 31) == __ffs(grp) - 1)
            atomicAdd(acc + key, (unsigned long long)sum << 12);
    }
}

// 1-D redistribution of the seeds along the cells (Image.cpp:549-616).  One
// block per segment: the densities are formed in parallel, the prefix sums
// (sequential float sums in the reference) by one thread, the placement in
// parallel; on shared memory when Kp <= ASV_ADJ_SMEM, else on `scratch`
// (Kp floats).
#define ASV_ADJ_SMEM 12256     // floats: with the kernel's static counter the block stays within 48 KB

__global__ void __launch_bounds__(256) k_density_adjust(AsvDev d, float *scratch)
{
    extern __shared__ float sh_len[];
    int si = blockIdx.x;
    if (si >= d.nseg) return;
    const SegDesc &S = d.segs[si];
    const int Kp = S.Kp;
    const unsigned long long *acc = d.dacc + S.seed_off;
    const int *xl = d.cells + S.cell_off + S.W + S.H + S.D, *xr = xl + S.wNum;
    const float4 *grid = d.grid + S.seed_off;
    float *len = Kp <= ASV_ADJ_SMEM ? sh_len : scratch + S.seed_off;
    for (int i = threadIdx.x; i < Kp; i += blockDim.x) {
        unsigned long long tot = acc[i] + (3ull << 24);               // cleared to 3.0 (:506-507)
        float res = __ull2float_rn(tot) * 0x1p-24f;
        len[i] = (float)(0.001 * (double)res);                        // :554
    }
    __shared__ int placed;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 1; i < Kp; i++) len[i] = len[i] + len[i - 1];    // :558-569 (float order kept)
        placed = 0;
    }
    __syncthreads();
    const float interval = len[Kp - 1] / (float)(Kp + 1);             // :570
    // The reference walks seeds and cells together (:586-616): seed i lands
    // in the first cell j1 with seed_in < len[j1], searching on from the
    // previous seed's cell.  seed_in grows with i and len never decreases,
    // so that cell is the first such cell of the whole array: found here by
    // a binary search per seed.  Once no cell qualifies the walk stops, so
    // the placed seeds are a prefix 0..n-1 of the ids.
    int mine = 0;
    for (int i = threadIdx.x; i < Kp; i += blockDim.x) {
        const float seed_in = (float)(i + 1) * interval;
        int lo = 0, hi = Kp;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (seed_in < len[mid]) hi = mid; else lo = mid + 1;
        }
        const int j1 = lo;
        if (j1 == Kp) continue;
        const int c = j1 % S.wNum;
        const int x1 = xl[c], x2 = xr[c];
        const float frac = j1 == 0 ? seed_in / len[j1] : (seed_in - len[j1 - 1]) / (len[j1] - len[j1 - 1]);
        const float ax = floorf((float)x1 + (float)(x2 - x1) * frac);
        const float4 g = grid[j1];
        d.pos0[S.seed_off + i] = make_float4((float)((double)ax + 0.5), g.y, g.z, (float)i);
        mine++;
    }
    atomicAdd(&placed, mine);
    __syncthreads();
    if (threadIdx.x == 0) d.post[si * ASV_POST_WORDS + POST_VALID] = placed;   // checked by the host
}

// ---------------------------------------------------------------------------
// Seeds: first-iteration init (draw_seeds.vs:20-35) and the per-iteration
// draw (draw_next_seeds.vs): seed record at the seed voxel, the later seed
// winning a shared voxel; JFA table packed for the passes.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int asv_seed_seg(const AsvDev &d, int g, int &local)
{
    int si = asv_find_seg(d.seed_prefix, d.nseg, g);
    local = g - d.seed_prefix[si];
    return si;
}

__global__ void k_first_init(AsvDev d)
{
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= d.total_seeds) return;
    int i;
    int si = asv_seed_seg(d, g, i);
    const SegDesc &S = d.segs[si];
    if (i >= S.Kp) return;
    float4 p = d.pos0[g];
    d.pos[g] = p;
    d.mkey[g] = -1;   // a new Lloyd run starts without reseed memo
#pragma unroll
    for (int e = 0; e < 8; e++) d.M[8 * g + e] = d.M0[8 * g + e];
    int x = min(max((int)floorf(p.x), 0), S.W - 1);
    int y = min(max((int)floorf(p.y), 0), S.H - 1);
    int z = min(max((int)floorf(p.z), 0), S.D - 1);
    uchar4 l = d.lab[S.vox_off + ((long long)z * S.H + y) * S.W + x];
    d.slab[g] = make_float4((float)l.x, (float)l.y, (float)l.z, 0.0f);
}

__global__ void k_draw(AsvDev d)
{
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= d.total_seeds) return;
    int i;
    int si = asv_seed_seg(d, g, i);
    const SegDesc &S = d.segs[si];
    if (i >= S.Kp) return;
    float4 p = d.pos[g], c = d.slab[g];
    const float *m = d.M + 8 * g;
    // table: (-x, -y, -z, -L) (M00, M11, 2M01, 2M12) (2M02, M22, -a, -b),
    // laid out for asv_jfa_dist's paired operations.  v - s == v + (-s) in
    // IEEE arithmetic, and doubling is exact, so
    // (dx*dy)*(2*M01) == ((2*dx)*dy)*M01 (flood.gs:85).
    d.jtab[3 * g + 0] = make_float4(-p.x, -p.y, -p.z, -c.x);
    d.jtab[3 * g + 1] = make_float4(m[0], m[3], 2.0f * m[2], 2.0f * m[4]);
    d.jtab[3 * g + 2] = make_float4(2.0f * m[1], m[5], -c.y, -c.z);
    if (!(p.x >= 0.0f && p.y >= 0.0f && p.z >= 0.0f)) return;
    int x = (int)p.x, y = (int)p.y, z = (int)p.z;
    if (x >= S.W || y >= S.H || z >= S.D) return;
    atomicMax(d.labA + S.vox_off + ((long long)z * S.H + y) * S.W + x, i);
}

// ---------------------------------------------------------------------------
// One JFA pass (GPU-AS/shaders/flood.gs:26-182).  27 candidates per voxel in
// the shader's order: slices z, z-step, z+step; in each slice rows
// y-step..y+step, columns x-step..x+step; clamp to edge.  The winner is the
// first candidate of least distance (strict `<` from 1e8), so any list that
// holds every valid candidate id, each first listed in the order of its first
// occurrence, gives the shader's label: a repeated id has the distance of its
// first occurrence and never wins again.
//
// Work layout: a block owns a tile of ASV_TILE_X x ASV_TILE_Y columns and a
// run of `zrun` voxels of each column, taken in chain order for the
// pass's step: z = r, r+step, r+2*step, ... (residue r = 0, 1, ...).  Along a
// chain the slice z+step of one voxel is the centre slice of the next and its
// centre the minus slice after that, so every slice's 9 labels are loaded
// and reduced to a list of ids once and used by up to three voxels (about
// 1.25 slice reductions per voxel instead of 3).  The voxel's list is the
// centre list, then the ids of the minus and plus lists not already listed
// (asv_merge_lists); a warp evaluates it in one loop, paying for its longest
// list.
// ---------------------------------------------------------------------------
#define ASV_JFA_THREADS 256
#define ASV_SLICE_MAX 9
typedef int asv_list_t;      // candidate-list entry in shared memory (ids < 32768)

// chain order of the D slices for `step`: position p -> residue r, index j
// in the chain, chain length len (z = r + j * step)
__device__ __forceinline__ void asv_chain_pos(int p, int D, int step, int &r, int &j, int &len)
{
    if (step >= D) { r = p; j = 0; len = 1; return; }
    const int q = D / step, m = D - q * step;       // m chains of q+1 slices, the rest q
    const int big = m * (q + 1);
    if (p < big) { r = p / (q + 1); j = p - r * (q + 1); len = q + 1; }
    else { const int pp = p - big; r = m + pp / q; j = pp - (r - m) * q; len = q; }
}

// valid ids among the 9 labels of one slice (offset zoff) around the
// column, each once, in first-occurrence order: a label is listed unless it
// equals one of the labels before it (compares against the loaded labels,
// all in registers, so nothing is shifted or stored to dedup).  Writes the
// list (stride ASV_JFA_THREADS), returns its length.
__device__ __forceinline__ int asv_slice_list(const int32_t *__restrict__ in, int zoff, const int xs[3],
                                              const int ys[3], int Kp, asv_list_t *__restrict__ lst)
{
    int32_t c[9];
#pragma unroll
    for (int oy = 0; oy < 3; oy++)
#pragma unroll
        for (int ox = 0; ox < 3; ox++) c[oy * 3 + ox] = __ldg(in + zoff + ys[oy] + xs[ox]);
    int n = 0;
#pragma unroll
    for (int k = 0; k < 9; k++) {
        bool fresh = (unsigned)c[k] < (unsigned)Kp;
#pragma unroll
        for (int e = 0; e < k; e++) fresh = fresh && c[k] != c[e];
        if (fresh) {
            lst[n * ASV_JFA_THREADS] = c[k];
            n++;
        }
    }
    return n;
}

// The voxel's candidate list: the centre list A, then the ids of the minus
// list B and the plus list C that are not among A's first four entries or
// the last two ids appended (appended to X in order).  Returns X's length.
__device__ __forceinline__ int asv_merge_lists(const asv_list_t *__restrict__ A, int na,
                                               const asv_list_t *__restrict__ B, int nb,
                                               const asv_list_t *__restrict__ C, int nc,
                                               asv_list_t *__restrict__ X)
{
    const int h0 = na > 0 ? A[0] : -1, h1 = na > 1 ? A[ASV_JFA_THREADS] : -1;
    const int h2 = na > 2 ? A[2 * ASV_JFA_THREADS] : -1, h3 = na > 3 ? A[3 * ASV_JFA_THREADS] : -1;
    int nx = 0, r1 = -1, r2 = -1;
    const int n = nb + nc;
    for (int i = 0; i < n; i++) {
        const int l = i < nb ? B[i * ASV_JFA_THREADS] : C[(i - nb) * ASV_JFA_THREADS];
        if (l != h0 && l != h1 && l != h2 && l != h3 && l != r1 && l != r2) {
            X[nx * ASV_JFA_THREADS] = l;
            nx++;
            r2 = r1; r1 = l;
        }
    }
    return nx;
}

// flood.gs:72-94: anisotropic distance of the voxel centre to seed l of the
// table, in the shader's operation order: every product and sum of the
// shader on the same operands, each rounded once.  The voxel side comes
// packed as vxy = (x, y), vzl = (z, L), vab = (a, b); the table rows are
// (-x, -y, -z, -L), (M00, M11, 2 M02, 2 M12), (2 M01, M22, -a, -b), so the
// six differences are three two-wide additions (__fadd2_rn: each half
// rounds like the scalar addition, and v + (-s) is v - s) and the products
// pair up two-wide where both operands lie side by side: (dx dx, dy dy),
// (dz dz, eL eL), (ea ea, eb eb), (dx dz, dy dz), then those times
// (M00, M11) and (2 M02, 2 M12).  Every sum stays a scalar addition with
// explicit round-to-nearest (-fmad=false), which the PTX ISA keeps apart
// from the products; a two-wide product feeding a two-wide sum was seen
// fused into a two-wide FMA, so no sum is two-wide.  The bit-exact tests
// against the oracle (millions of distances per run) guard both.
__device__ __forceinline__ float asv_jfa_dist_v(const float4 t0, const float4 t1, const float4 t2, float2 vxy,
                                                float2 vzl, float2 vab, float ratio)
{
    const float2 dxy = __fadd2_rn(vxy, make_float2(t0.x, t0.y));              // (dx, dy)
    const float2 dzl = __fadd2_rn(vzl, make_float2(t0.z, t0.w));              // (dz, eL)
    const float2 eab = __fadd2_rn(vab, make_float2(t2.z, t2.w));              // (ea, eb)
    const float dx = dxy.x, dy = dxy.y, dz = dzl.x;
    const float2 sq = __fmul2_rn(dxy, dxy);
    const float2 zl = __fmul2_rn(dzl, dzl);
    const float2 ab = __fmul2_rn(eab, eab);
    const float2 cz = __fmul2_rn(dxy, make_float2(dz, dz));
    const float2 wa = __fmul2_rn(sq, make_float2(t1.x, t1.y));
    const float2 wc = __fmul2_rn(cz, make_float2(t1.z, t1.w));
    float p1 = wa.x + (dx * dy) * t2.x;
    p1 = p1 + wc.x;
    float p2 = wa.y + wc.y;
    p2 = p2 + zl.x * t2.y;
    float pos = p1 + p2;
    float col = zl.y + ab.x;
    col = col + ab.y;
    pos = (pos < 0.0f) ? 0.0f : pos;                                           // flood.gs:90-93
    return ratio * pos + col;                                                  // flood.gs:94
}

// the same with seed l's row of the table in global memory
__device__ __forceinline__ float asv_jfa_dist(const float4 *__restrict__ tab, int l, float2 vxy, float2 vzl,
                                              float2 vab, float ratio)
{
    return asv_jfa_dist_v(__ldg(tab + 3 * l), __ldg(tab + 3 * l + 1), __ldg(tab + 3 * l + 2), vxy, vzl, vab,
                          ratio);
}

// distance loop over the concatenated lists A (na) and X (nx): the first
// candidate of least distance wins (flood.gs:63, :95-99)
__device__ __forceinline__ int32_t asv_jfa_eval(const asv_list_t *__restrict__ A, int na,
                                                const asv_list_t *__restrict__ X, int nx,
                                                const float4 *__restrict__ tab, uchar4 c, float vx, float vy,
                                                float vz, float ratio)
{
    const float2 vxy = make_float2(vx, vy), vzl = make_float2(vz, (float)c.x);
    const float2 vab = make_float2((float)c.y, (float)c.z);
    float mind = 100000000.0f;
    int32_t best = -1;
    const int n = na + nx;
    int i = 0;
    for (; i + 1 < n; i += 2) {          // two candidates per trip: their loads overlap
        const int32_t la = i < na ? A[i * ASV_JFA_THREADS] : X[(i - na) * ASV_JFA_THREADS];
        const int32_t lb = i + 1 < na ? A[(i + 1) * ASV_JFA_THREADS] : X[(i + 1 - na) * ASV_JFA_THREADS];
        const float da = asv_jfa_dist(tab, la, vxy, vzl, vab, ratio);
        const float db = asv_jfa_dist(tab, lb, vxy, vzl, vab, ratio);
        if (da < mind) { mind = da; best = la; }     // compared in list order
        if (db < mind) { mind = db; best = lb; }
    }
    if (i < n) {
        const int32_t l = i < na ? A[i * ASV_JFA_THREADS] : X[(i - na) * ASV_JFA_THREADS];
        const float dist = asv_jfa_dist(tab, l, vxy, vzl, vab, ratio);
        if (dist < mind) { mind = dist; best = l; }
    }
    return best;
}

// Centroid sums of one voxel in the list form, fused into the last JFA pass
// of a Lloyd iteration (the bit-set form sums runs of equal labels instead,
// asv_run_flush) (centroids.vs:19-54; a label outside [0, Kp) counts in the
// -1 slot, so no slot beyond the segment's is written): the lanes of the warp are grouped by
// destination slot, reduced in the warp, and one u64 atomic per group and
// component is issued.  Every lane of the warp makes this call for every
// voxel of the tile (a lane whose column lies outside the segment passes
// valid = false and joins with key -1, which issues nothing), so the full
// warp mask is exact here whatever path the lanes took through the
// candidate evaluation before it.
__device__ __forceinline__ void asv_accumulate(unsigned long long *__restrict__ sums, int slot0, uchar4 c,
                                               int Kp, int x, int y, int z, int best, bool valid)
{
    const int key = valid ? slot0 + ((unsigned)best < (unsigned)Kp ? best : Kp) : -1;
    const unsigned grp = __match_any_sync(0xffffffffu, key);
    const unsigned q[7] = { 2u * x + 1u, 2u * y + 1u, 2u * z + 1u, 1u, c.x, c.y, c.z };
    unsigned s[7];
#pragma unroll
    for (int k = 0; k < 7; k++) s[k] = __reduce_add_sync(grp, q[k]);
    if (valid && (int)(threadIdx.x & 31) == __ffs(grp) - 1) {
        unsigned long long *dst = sums + 8ull * key;
#pragma unroll
        for (int k = 0; k < 7; k++) atomicAdd(dst + k, (unsigned long long)s[k]);
    }
}

// One column's run of zrun chain positions [p0, p0 + zrun).
// `lists` is this thread's first entry of 3 slice-list rows of ASV_SLICE_MAX
// entries and one merge row of 2 x ASV_SLICE_MAX.  A
// chain continues while z + step < D; the next chain starts at the next
// residue, whose minus slice is slice 0.  A lane whose column lies outside
// the segment runs the same loop on the clamped column (valid = false) and
// stores nothing, so the lanes of a warp stay in the same tile.
template <bool SUMS>
__device__ __forceinline__ void asv_jfa_run(const int32_t *__restrict__ in, int32_t *__restrict__ out,
                                            const uchar4 *__restrict__ lab, const float4 *__restrict__ tab,
                                            unsigned long long *__restrict__ sums, int slot0, int W, int H, int D,
                                            int Kp, int x, int y, int p0, int zrun, int step,
                                            float ratio, asv_list_t *__restrict__ lists, bool valid)
{
    const int sl = W * H;                       // segments hold < 2^31 voxels
    const int xs[3] = { max(x - step, 0), x, min(x + step, W - 1) };
    const int ys[3] = { max(y - step, 0) * W, y * W, min(y + step, H - 1) * W };
    const int col = y * W + x;
    const float vx = (float)x + 0.5f, vy = (float)y + 0.5f;
    const int row = ASV_SLICE_MAX * ASV_JFA_THREADS;
    int r, j, len;
    asv_chain_pos(p0, D, step, r, j, len);
    int z = r + j * step;
    int n = min(zrun, D - p0);
    int sm = 0, sc = 1, sp = 2;                 // list rows of the minus / centre / plus slices
    int nm = asv_slice_list(in, max(z - step, 0) * sl, xs, ys, Kp, lists + sm * row);
    int nc = asv_slice_list(in, z * sl, xs, ys, Kp, lists + sc * row);
    while (true) {
        const bool more = z + step < D;         // the chain goes on
        const int zp = more ? z + step : D - 1;
        const int np = asv_slice_list(in, zp * sl, xs, ys, Kp, lists + sp * row);
        const uchar4 c = __ldg(lab + z * sl + col);
        const int nx = asv_merge_lists(lists + sc * row, nc, lists + sm * row, nm, lists + sp * row, np,
                                       lists + 3 * row);
        const int32_t best = asv_jfa_eval(lists + sc * row, nc, lists + 3 * row, nx, tab, c, vx, vy,
                                          (float)z + 0.5f, ratio);
        if (valid) out[z * sl + col] = best;
        if (SUMS) asv_accumulate(sums, slot0, c, Kp, x, y, z, best, valid);
        if (--n == 0) break;
        if (more) {                             // next voxel of the chain: rotate the rows
            z = zp;
            const int t = sm;
            sm = sc; sc = sp; sp = t;
            nm = nc; nc = np;
        } else {                                // next residue: a new chain
            z = z - (z / step) * step + 1;
            nm = asv_slice_list(in, 0, xs, ys, Kp, lists + sm * row);
            nc = asv_slice_list(in, z * sl, xs, ys, Kp, lists + sc * row);
        }
    }
}

// ---------------------------------------------------------------------------
// Bit-set form of a JFA pass (steps 1..ASV_BITS_MAXS).
//
// The label a voxel takes depends only on the set of distinct valid labels
// among its 27 candidates, except when two of them tie at the least
// distance (then the first in the shader's candidate order wins): the
// distance is a function of the voxel and the label's seed alone.  A
// sub-tile (16 x 16 columns x up to 16 chain positions of the tile) holds
// few distinct labels in its whole footprint (the sub-tile grown by `step`
// on every side; on the benchmarked clips mostly under 32).  So the block
// copies the footprint and the sub-tile's LAB values into shared memory
// with asynchronous copies (one memory latency per sub-tile), numbers the
// footprint's distinct labels 0..T-1 (T <= 32, else the sub-tile takes the
// list form) and turns every footprint entry into its label's bit.  A
// voxel's candidate mask is the OR of the 9 bits of each of its three
// slices (the plus slice's mask becomes the next position's centre mask);
// the voxel evaluates the labels of its mask in any order and keeps the
// least distance below 1e8.  An exact tie at the least distance between two
// labels (about 30 per million voxel-passes on the benchmarked clips) sends
// the voxel through the shader's ordered scan of its 27 candidates instead,
// so every label equals the shader's.
//
// Footprint slices ("slots") of a sub-tile of n chain positions: slot 0 the
// minus slice of position 0, slots 1..n the centre slices, slot n+1 the plus
// slice of position n-1, and where a chain ends inside the sub-tile slot
// n+2 (slice 0, the minus slice of every chain start after the first) and
// slot n+3 (slice D-1, the clamped plus slice of every chain end).  Along a
// chain the minus slice of a position is the centre of the one before it
// and its plus slice the centre of the one after it.
// ---------------------------------------------------------------------------
#define ASV_JFA_LIST_BYTES (5 * ASV_SLICE_MAX * ASV_JFA_THREADS * (int)sizeof(asv_list_t))
#define ASV_BITS_MAXS 6          // largest step taken in bit-set form
#define ASV_BITS_MAXT 32         // labels per sub-tile footprint (one 32-bit mask)
#define ASV_BITS_MAXKP 8192      // segment seed counts up to this use the bit-set form
#define ASV_BITS_TLCAP 256       // claimed labels remembered for the reset
#define ASV_BITS_NONE 255        // table number of no label
#define ASV_ACC_ROW 7            // words per entry of the sub-tile's centroid-sum table (odd: the
                                 // entries' rows start in different shared-memory banks)
#define ASV_BITS_AREA 62464      // shared bytes of the largest sub-tiles (step 4, 16 positions; step 6, 12)
#define ASV_JFA_AREA (ASV_BITS_AREA > ASV_JFA_LIST_BYTES ? ASV_BITS_AREA : ASV_JFA_LIST_BYTES)

struct AsvBitsShared {
    float4 tdat[3 * ASV_BITS_MAXT];             // the table's seed rows (as jtab)
    unsigned acc[(ASV_BITS_MAXT + 1) * ASV_ACC_ROW];   // centroid sums of the sub-tile per table entry (+ label -1)
    unsigned claim[ASV_BITS_MAXKP / 32];        // labels numbered in this sub-tile (all zero between)
    int tlab[ASV_BITS_TLCAP];                   // label of each number
    int slotz[20];                              // slice of each footprint slot
    int tcount;
    unsigned char map8[ASV_BITS_MAXKP];         // number of each claimed label
};
#define ASV_JFA_SMEM (ASV_JFA_AREA + (int)sizeof(AsvBitsShared))

template <int S> struct AsvBitsGeo {
    static constexpr int FW = ASV_TILE_X + 2 * S;                     // footprint width and height
    static constexpr int FP = FW * FW;                                // footprint entries per slot
    // chain positions per sub-tile: deep where the footprint stays small
    static constexpr int SUB = S <= 4 ? 16 : 12;
    static constexpr int NSLOT = SUB + 4;
    static constexpr int NCOL = (FP + ASV_JFA_THREADS - 1) / ASV_JFA_THREADS;
    static constexpr int FLAB_BYTES = NSLOT * FP * 4;
    static_assert(FLAB_BYTES + SUB * ASV_JFA_THREADS * 4 <= ASV_BITS_AREA, "bit-set sub-tile exceeds the shared area");
};

// 4-byte asynchronous copy global -> shared (cp.async, completed by
// asv_cp_async_wait)
__device__ __forceinline__ void asv_cp_async4(void *dst, const void *src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void asv_cp_async_wait()
{
    asm volatile("cp.async.commit_group;\ncp.async.wait_all;\n" ::: "memory");
}

// The shader's ordered scan of the 27 candidates (slices centre, minus,
// plus; rows y-S, y, y+S; columns x-S, x, x+S) over the footprint's label
// bits, strict '<' from 1e8 (flood.gs:63, :95-99): the tie-break path.
template <int S>
__device__ __noinline__ int asv_bits_ordered(const unsigned *__restrict__ fc, const unsigned *__restrict__ fm,
                                             const unsigned *__restrict__ fp, const AsvBitsShared &b,
                                             float2 vxy, float2 vzl, float2 vab, float ratio)
{
    constexpr int FW = AsvBitsGeo<S>::FW;
    float mind = 100000000.0f;
    int best = -1;
    for (int k = 0; k < 3; k++) {
        const unsigned *f = k == 0 ? fc : (k == 1 ? fm : fp);
        for (int a = 0; a < 3; a++)
            for (int c = 0; c < 3; c++) {
                const unsigned bit = f[a * S * FW + c * S];
                if (!bit) continue;
                const int e = __ffs(bit) - 1;
                const float dist = asv_jfa_dist_v(b.tdat[3 * e], b.tdat[3 * e + 1], b.tdat[3 * e + 2], vxy, vzl,
                                                  vab, ratio);
                if (dist < mind) { mind = dist; best = e; }
            }
    }
    return best;                                              // table entry, or -1
}

// A thread's run of voxels with one label, added to its table entry's
// centroid sums in shared memory: count n, sum of 2z+1 and of L, a, b; the
// column's 2x+1 and 2y+1 times n.  Exact u32 sums (a sub-tile holds at most
// 16 x 256 voxels of coordinates below 4096).
__device__ __forceinline__ void asv_run_flush(unsigned *__restrict__ a, unsigned n, unsigned sz, unsigned sl,
                                              unsigned sa, unsigned sb, int x, int y)
{
    atomicAdd(a + 0, n * (2u * (unsigned)x + 1u));
    atomicAdd(a + 1, n * (2u * (unsigned)y + 1u));
    atomicAdd(a + 2, sz);
    atomicAdd(a + 3, n);
    atomicAdd(a + 4, sl);
    atomicAdd(a + 5, sa);
    atomicAdd(a + 6, sb);
}

// One sub-tile of n <= SUB chain positions from p0 in bit-set form; false
// (nothing written) when its footprint holds more than 32 labels.  Called
// by the whole block.
template <int S, bool SUMS>
__device__ bool asv_jfa_bits_sub(const int32_t *__restrict__ in, int32_t *__restrict__ out,
                                 const uchar4 *__restrict__ lab, const float4 *__restrict__ tab,
                                 unsigned long long *__restrict__ sums, int slot0, int W, int H, int D, int Kp,
                                 int tx0, int ty0, int p0, int n, float ratio, unsigned char *smem)
{
    using G = AsvBitsGeo<S>;
    constexpr int FW = G::FW, FP = G::FP;
    int *flab = (int *)smem;                                   // labels, then their bits
    uchar4 *labsh = (uchar4 *)(smem + G::FLAB_BYTES);
    AsvBitsShared &b = *(AsvBitsShared *)(smem + ASV_JFA_AREA);
    const int tid = threadIdx.x, lane = tid & 31;
    const int sl = W * H;
    const int lx = tid % ASV_TILE_X, ly = tid / ASV_TILE_X;
    const int gx = tx0 + lx, gy = ty0 + ly;
    const bool valid = gx < W && gy < H;                       // other lanes run along, store nothing
    const int x = min(gx, W - 1), y = min(gy, H - 1);
    const int col = y * W + x;

    // slices of the footprint slots
    bool brk = false;
    if (tid < n) {
        int r, j, len;
        asv_chain_pos(p0 + tid, D, S, r, j, len);
        const int z = r + j * S;
        b.slotz[1 + tid] = z;
        if (tid == 0) b.slotz[0] = max(z - S, 0);
        if (tid == n - 1) b.slotz[n + 1] = z + S < D ? z + S : D - 1;
        brk = tid < n - 1 && z + S >= D;
    }
    if (tid == 0) { b.slotz[n + 2] = 0; b.slotz[n + 3] = D - 1; }
    const bool any_brk = __syncthreads_or(brk);
    const int nf = any_brk ? n + 4 : n + 2;

    // footprint labels (clamp-to-edge) and the voxels' LAB, copied
    // asynchronously; each thread copies the same footprint columns of every slot
    int coff[G::NCOL];
#pragma unroll
    for (int i = 0; i < G::NCOL; i++) {
        const int e = tid + i * ASV_JFA_THREADS, fy = e / FW, fx = e - fy * FW;
        coff[i] = min(max(ty0 - S + fy, 0), H - 1) * W + min(max(tx0 - S + fx, 0), W - 1);
    }
    for (int k = 0; k < nf; k++) {
        const int32_t *src = in + b.slotz[k] * sl;
#pragma unroll
        for (int i = 0; i < G::NCOL; i++) {
            const int e = tid + i * ASV_JFA_THREADS;
            if (e < FP) asv_cp_async4(flab + k * FP + e, src + coff[i]);
        }
    }
    for (int j = 0; j < n; j++) asv_cp_async4(labsh + j * ASV_JFA_THREADS + tid, lab + b.slotz[j + 1] * sl + col);
    asv_cp_async_wait();
    __syncthreads();

    // number the distinct labels (each thread its own entries)
    for (int k = 0; k < nf; k++) {
#pragma unroll
        for (int i = 0; i < G::NCOL; i++) {
            const int e = tid + i * ASV_JFA_THREADS;
            int v = e < FP ? flab[k * FP + e] : -1;
            if ((unsigned)v >= (unsigned)Kp) v = -1;
            const int vp = __shfl_up_sync(0xffffffffu, v, 1);
            if (v >= 0 && !(lane > 0 && vp == v)) {
                const unsigned w = (unsigned)v >> 5, bit = 1u << (v & 31);
                if (!(*(volatile unsigned *)&b.claim[w] & bit) && !(atomicOr(&b.claim[w], bit) & bit)) {
                    const int idx = atomicAdd(&b.tcount, 1);
                    if (idx < ASV_BITS_TLCAP) b.tlab[idx] = v;
                    b.map8[v] = (unsigned char)(idx < ASV_BITS_MAXT ? idx : ASV_BITS_NONE);
                }
            }
        }
    }
    __syncthreads();
    const int T = b.tcount;
    // the claim bits go back to zero for the next sub-tile
    if (T <= ASV_BITS_TLCAP) {
        for (int i = tid; i < T; i += ASV_JFA_THREADS) b.claim[b.tlab[i] >> 5] = 0u;
    } else {
        for (int i = tid; i < ASV_BITS_MAXKP / 32; i += ASV_JFA_THREADS) b.claim[i] = 0u;
    }
    if (T > ASV_BITS_MAXT) {
        __syncthreads();
        if (tid == 0) b.tcount = 0;
        __syncthreads();
        return false;
    }
    for (int i = tid; i < 3 * T; i += ASV_JFA_THREADS) b.tdat[i] = __ldg(tab + 3 * b.tlab[i / 3] + i % 3);
    if (SUMS)
        for (int i = tid; i < (ASV_BITS_MAXT + 1) * ASV_ACC_ROW; i += ASV_JFA_THREADS) b.acc[i] = 0u;
    // every footprint entry becomes its label's bit (0: no label), in place:
    // each thread converts the entries it copied
    for (int k = 0; k < nf; k++) {
#pragma unroll
        for (int i = 0; i < G::NCOL; i++) {
            const int e = tid + i * ASV_JFA_THREADS;
            if (e < FP) {
                int *q = flab + k * FP + e;
                const int l = *q;
                *q = (int)((unsigned)l < (unsigned)Kp ? 1u << b.map8[l] : 0u);
            }
        }
    }
    __syncthreads();

    // the chain walk of this thread's column
    const unsigned *f0 = (const unsigned *)flab + ly * FW + lx;  // candidate (x - S, y - S) of slot 0
    auto smask = [&](int k) -> unsigned {                         // a slice's 9 candidates
        const unsigned *f = f0 + k * FP;
        unsigned m = 0;
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
            for (int c = 0; c < 3; c++) m |= f[a * S * FW + c * S];
        return m;
    };
    const float2 vxy = make_float2((float)x + 0.5f, (float)y + 0.5f);
    const unsigned m_zero = any_brk ? smask(n + 2) : 0u, m_last = any_brk ? smask(n + 3) : 0u;
    unsigned mm = smask(0), mc = smask(1);
    int im = 0;
    // centroid sums (last pass of an iteration): the thread's current run of
    // equal labels along its column, flushed into the sub-tile's table when
    // the label changes and at the end; the table goes to the global sums
    // once per sub-tile (centroids.vs:19-54; label -1 counts in slot Kp)
    int run_e = -1;
    unsigned run_n = 0u, run_z = 0u, run_l = 0u, run_a = 0u, run_b = 0u;
    for (int j = 0; j < n; j++) {
        const int z = b.slotz[j + 1];
        const bool chain = z + S < D;                         // the plus slice is the next centre
        const int ip = j == n - 1 ? n + 1 : (chain ? j + 2 : n + 3);
        const unsigned mp = (j < n - 1 && !chain) ? m_last : smask(ip);
        const uchar4 c = labsh[j * ASV_JFA_THREADS + tid];
        const float2 vzl = make_float2((float)z + 0.5f, (float)c.x), vab = make_float2((float)c.y, (float)c.z);
        unsigned m = mm | mc | mp;
        float best = 100000000.0f;
        int bt = -1;
        bool tie = false;
        while (m) {
            const int ta = __ffs(m) - 1;
            m &= m - 1;
            const float da = asv_jfa_dist_v(b.tdat[3 * ta], b.tdat[3 * ta + 1], b.tdat[3 * ta + 2], vxy, vzl, vab,
                                            ratio);
            if (da < best) { best = da; bt = ta; tie = false; } else if (da == best) tie = true;
        }
        if (tie) bt = asv_bits_ordered<S>(f0 + (j + 1) * FP, f0 + im * FP, f0 + ip * FP, b, vxy, vzl, vab, ratio);
        const int label = bt >= 0 ? b.tlab[bt] : -1;
        if (valid) out[z * sl + col] = label;
        if (SUMS && valid) {
            const int e = bt >= 0 ? bt : ASV_BITS_MAXT;
            if (e != run_e) {
                if (run_e >= 0) asv_run_flush(b.acc + ASV_ACC_ROW * run_e, run_n, run_z, run_l, run_a, run_b, x, y);
                run_e = e;
                run_n = run_z = run_l = run_a = run_b = 0u;
            }
            run_n++;
            run_z += 2u * (unsigned)z + 1u;
            run_l += c.x; run_a += c.y; run_b += c.z;
        }
        if (j + 1 < n) {
            if (chain) { mm = mc; mc = mp; im = j + 1; }
            else { mm = m_zero; mc = smask(j + 2); im = n + 2; }
        }
    }
    if (SUMS) {
        // the runs left at the end, grouped by entry across the warp (every
        // lane of the block gets here; lanes without a run join with entry
        // -1, which adds nothing), so a warp adds each entry once
        const unsigned grp = __match_any_sync(0xffffffffu, run_e);
        const unsigned q[7] = { run_n * (2u * (unsigned)x + 1u), run_n * (2u * (unsigned)y + 1u), run_z, run_n,
                                run_l, run_a, run_b };
        unsigned t[7];
#pragma unroll
        for (int k = 0; k < 7; k++) t[k] = __reduce_add_sync(grp, q[k]);
        if (run_e >= 0 && lane == __ffs(grp) - 1) {
#pragma unroll
            for (int k = 0; k < 7; k++) atomicAdd(b.acc + ASV_ACC_ROW * run_e + k, t[k]);
        }
        __syncthreads();
        for (int i = tid; i < (T + 1) * 7; i += ASV_JFA_THREADS) {
            const int e = i / 7, k = i - e * 7;
            const int ent = e < T ? e : ASV_BITS_MAXT;           // the -1 entry after the T labels
            const unsigned v = b.acc[ASV_ACC_ROW * ent + k];
            if (v) atomicAdd(sums + 8ull * (slot0 + (ent < ASV_BITS_MAXT ? b.tlab[ent] : Kp)) + k,
                             (unsigned long long)v);
        }
    }
    __syncthreads();                                          // the footprint and table are reused
    if (tid == 0) b.tcount = 0;
    return true;
}

// one tile of a pass: bit-set form by sub-tiles where it applies, else (or
// for a sub-tile whose footprint holds too many labels) the list form
template <bool SUMS>
__device__ __forceinline__ void asv_jfa_tile(const int32_t *__restrict__ in, int32_t *__restrict__ out,
                                             const uchar4 *__restrict__ lab, const float4 *__restrict__ tab,
                                             unsigned long long *__restrict__ sums, int slot0, int W, int H, int D,
                                             int Kp, int tx0, int ty0, int p0, int zrun, int step, float ratio,
                                             unsigned char *smem)
{
    const int n = min(zrun, D - p0);
    const int lx = threadIdx.x % ASV_TILE_X, ly = threadIdx.x / ASV_TILE_X;
    const int gx = tx0 + lx, gy = ty0 + ly;
    const bool valid = gx < W && gy < H;                       // block-uniform loop: every lane runs the tile
    // sub-tiles the bit-set form leaves (a bit per sub-tile of `sub` positions)
    // go through one inlined copy of the list form
    unsigned fail = 1u;
    int sub = n;
    // <= 32 sub-tiles of >= 4; with tiles of 4 positions the footprint slots
    // outnumber the positions from step 3 on, where the list form is faster
    if (step <= ASV_BITS_MAXS && Kp <= ASV_BITS_MAXKP && n <= 32 * 4 && (zrun >= 8 || step <= 2)) {
        fail = 0u;
#define ASV_BITS_CASE(S_)                                                                                    \
    case S_:                                                                                                 \
        sub = AsvBitsGeo<S_>::SUB;                                                                           \
        for (int q0 = 0; q0 < n; q0 += AsvBitsGeo<S_>::SUB)                                                  \
            if (!asv_jfa_bits_sub<S_, SUMS>(in, out, lab, tab, sums, slot0, W, H, D, Kp, tx0, ty0, p0 + q0, \
                                            min(AsvBitsGeo<S_>::SUB, n - q0), ratio, smem))                  \
                fail |= 1u << (q0 / AsvBitsGeo<S_>::SUB);                                                  \
        break;
        switch (step) {
            ASV_BITS_CASE(1) ASV_BITS_CASE(2) ASV_BITS_CASE(3) ASV_BITS_CASE(4) ASV_BITS_CASE(5) ASV_BITS_CASE(6)
        }
#undef ASV_BITS_CASE
    }
    for (int i = 0; fail; i++, fail >>= 1) {
        if (!(fail & 1u)) continue;
        asv_jfa_run<SUMS>(in, out, lab, tab, sums, slot0, W, H, D, Kp, min(gx, W - 1), min(gy, H - 1), p0 + i * sub,
                          min(sub, n - i * sub), step, ratio, (asv_list_t *)smem + threadIdx.x, valid);
        __syncthreads();                                       // the list rows alias the footprint
    }
}

__device__ __forceinline__ void asv_jfa_smem_init(unsigned char *smem)
{
    AsvBitsShared &b = *(AsvBitsShared *)(smem + ASV_JFA_AREA);
    for (int i = threadIdx.x; i < ASV_BITS_MAXKP / 32; i += blockDim.x) b.claim[i] = 0u;
    if (threadIdx.x == 0) b.tcount = 0;
    __syncthreads();
}

// tile = ASV_TILE_X x ASV_TILE_Y columns x S.zrun chain positions
__global__ void __launch_bounds__(ASV_JFA_THREADS, 3) k_jfa(AsvDev d, int pass,
                                                         const int32_t *__restrict__ in,
                                                         int32_t *__restrict__ out)
{
    extern __shared__ __align__(16) unsigned char asv_jfa_smem[];
    asv_jfa_smem_init(asv_jfa_smem);
    for (int t = blockIdx.x; t < d.total_tiles; t += gridDim.x) {
        const int si = asv_find_seg(d.tile_prefix, d.nseg, t);
        const SegDesc &S = d.segs[si];
        if (pass >= S.npass) continue;
        const int lt = t - d.tile_prefix[si];
        const int tx = lt % S.tiles_x, rest = lt / S.tiles_x;
        const int ty = rest % S.tiles_y, p0 = (rest / S.tiles_y) * S.zrun;
        if (pass == S.npass - 1)                   // the iteration's labels: sum them
            asv_jfa_tile<true>(in + S.vox_off, out + S.vox_off, d.lab + S.vox_off, d.jtab + 3 * S.seed_off,
                               d.sums, S.seed_off, S.W, S.H, S.D, S.Kp, tx * ASV_TILE_X, ty * ASV_TILE_Y, p0,
                               S.zrun, S.steps[pass], S.ratio[pass], asv_jfa_smem);
        else
            asv_jfa_tile<false>(in + S.vox_off, out + S.vox_off, d.lab + S.vox_off, d.jtab + 3 * S.seed_off,
                                nullptr, 0, S.W, S.H, S.D, S.Kp, tx * ASV_TILE_X, ty * ASV_TILE_Y, p0,
                                S.zrun, S.steps[pass], S.ratio[pass], asv_jfa_smem);
    }
}

// ---------------------------------------------------------------------------
// The first pass of a Lloyd iteration as a scatter from the seeds.  Its input
// is the drawn seed volume: -1 everywhere but at the seed voxels, each
// holding the seed that won its voxel.  At step 1 a voxel's candidates are
// the seeds within its 3x3x3 neighbourhood (clamped to the edges), so instead
// of every voxel gathering 27 mostly empty labels, each drawn seed visits the
// up to 27 voxels around it.  The winner rule of the gather (least distance,
// the first of equal ones in the shader's candidate order) becomes a 64-bit
// minimum per voxel over keys (distance bits, candidate rank, label):
// distances are >= +0, so their bits order like their values, and the rank is
// the seed's first position in the voxel's candidate order (slices z, z-1,
// z+1; rows y-1..y+1; columns x-1..x+1), which with edge clamping can be an
// earlier offset than the plain one.  A distance that is not below 1e8 (or
// NaN) never wins (flood.gs:63, :95-99).  The output volume is filled with
// -1 first; k_jfa_first_take then hands each touched voxel's key to exactly
// one thread (atomicExch leaves the key empty for the next iteration), which
// writes the label.
// ---------------------------------------------------------------------------
#define ASV_KEY_EMPTY 0xffffffffffffffffull

// first rank, in the order `order` of offsets, of an offset o with
// clamp(v + o) == s along one axis of length n
__device__ __forceinline__ int asv_first_rank(int v, int s, int n, const int order[3])
{
#pragma unroll
    for (int r = 0; r < 3; r++) {
        const int q = min(max(v + order[r], 0), n - 1);
        if (q == s) return r;
    }
    return 3;    // not reached: s lies within one step of v
}

// thread -> (drawn seed, offset); false when the seed lost its voxel or the
// voxel lies outside the segment
__device__ __forceinline__ bool asv_first_target(const AsvDev &d, long long t, int &si, int &i, int &x, int &y,
                                                 int &z, int &sx, int &sy, int &sz)
{
    const int g = (int)(t / 27), o = (int)(t - (long long)g * 27);
    if (g >= d.total_seeds) return false;
    si = asv_seed_seg(d, g, i);
    const SegDesc &S = d.segs[si];
    if (i >= S.Kp) return false;
    const float4 p = d.pos[g];
    if (!(p.x >= 0.0f && p.y >= 0.0f && p.z >= 0.0f)) return false;     // as k_draw
    sx = (int)p.x; sy = (int)p.y; sz = (int)p.z;
    if (sx >= S.W || sy >= S.H || sz >= S.D) return false;
    if (d.labA[S.vox_off + ((long long)sz * S.H + sy) * S.W + sx] != i) return false;   // lost the draw
    x = sx + (o % 3 - 1); y = sy + ((o / 3) % 3 - 1); z = sz + (o / 9 - 1);
    return x >= 0 && x < S.W && y >= 0 && y < S.H && z >= 0 && z < S.D;
}

__global__ void __launch_bounds__(256) k_jfa_first_scatter(AsvDev d)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int si, i, x, y, z, sx, sy, sz;
    if (!asv_first_target(d, t, si, i, x, y, z, sx, sy, sz)) return;
    const SegDesc &S = d.segs[si];
    const int xy_order[3] = { -1, 0, 1 }, z_order[3] = { 0, -1, 1 };
    const int rank = asv_first_rank(z, sz, S.D, z_order) * 9 + asv_first_rank(y, sy, S.H, xy_order) * 3 +
                     asv_first_rank(x, sx, S.W, xy_order);
    const long long v = ((long long)z * S.H + y) * S.W + x;
    const uchar4 c = __ldg(d.lab + S.vox_off + v);
    const float dist = asv_jfa_dist(d.jtab + 3 * S.seed_off, i, make_float2((float)x + 0.5f, (float)y + 0.5f),
                                    make_float2((float)z + 0.5f, (float)c.x), make_float2((float)c.y, (float)c.z),
                                    S.ratio[0]);
    if (!(dist < 100000000.0f)) return;
    const unsigned long long key = ((unsigned long long)__float_as_uint(dist) << 32) |
                                   ((unsigned long long)rank << 16) | (unsigned long long)i;
    atomicMin(d.jkeys + S.vox_off + v, key);
}

__global__ void __launch_bounds__(256) k_jfa_first_take(AsvDev d)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int si, i, x, y, z, sx, sy, sz;
    if (!asv_first_target(d, t, si, i, x, y, z, sx, sy, sz)) return;
    const SegDesc &S = d.segs[si];
    const long long vl = ((long long)z * S.H + y) * S.W + x, v = S.vox_off + vl;
    const unsigned long long key = atomicExch(d.jkeys + v, ASV_KEY_EMPTY);
    if (key != ASV_KEY_EMPTY) {
        d.labB[v] = (int32_t)(key & 0x7fffu);
        d.tlist[atomicAdd(d.tcount, 1)] = ((unsigned long long)si << 32) | (unsigned long long)vl;
    }
}

// ---------------------------------------------------------------------------
// The second pass (step s = steps[1]) as a scatter too: its input, the first
// pass's output, is labelled only at the voxels listed in tlist.  A voxel v
// sees the label at u through offset o when clamp(v + o*s) == u along every
// axis; per axis those v form a range (one voxel inside the volume, up to
// s + 1 next to an edge, where several offsets clamp onto u).  Each (u, o)
// thread visits that box; ranks and keys as in the first pass.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void asv_axis_sources(int u, int o, int s, int n, int &lo, int &hi)
{
    if (o == 0) { lo = hi = u; return; }
    if (o < 0) {                              // clamp(v - s) == u
        if (u > 0) lo = hi = u + s; else { lo = 0; hi = s; }
    } else {                                  // clamp(v + s) == u
        if (u < n - 1) lo = hi = u - s; else { lo = n - 1 - s; hi = n - 1; }
    }
    lo = max(lo, 0);
    hi = min(hi, n - 1);                      // empty when lo > hi
}

// first rank, in the order `order`, of an offset o with clamp(v + o*s) == u
__device__ __forceinline__ int asv_first_rank_step(int v, int u, int s, int n, const int order[3])
{
#pragma unroll
    for (int r = 0; r < 3; r++)
        if (min(max(v + order[r] * s, 0), n - 1) == u) return r;
    return 3;    // not reached: v is one of u's sources
}

template <bool TAKE>
__global__ void __launch_bounds__(256) k_jfa_second(AsvDev d)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long e = t / 27;
    if (e >= *d.tcount) return;
    const int o = (int)(t - e * 27);
    const unsigned long long ent = d.tlist[e];
    const int si = (int)(ent >> 32);
    const long long ul = (long long)(ent & 0xffffffffull);
    const SegDesc &S = d.segs[si];
    const int s = S.steps[1];
    const int ux = (int)(ul % S.W), uy = (int)((ul / S.W) % S.H), uz = (int)(ul / ((long long)S.W * S.H));
    int x0, x1, y0, y1, z0, z1;
    asv_axis_sources(ux, o % 3 - 1, s, S.W, x0, x1);
    asv_axis_sources(uy, (o / 3) % 3 - 1, s, S.H, y0, y1);
    asv_axis_sources(uz, o / 9 - 1, s, S.D, z0, z1);
    if (x0 > x1 || y0 > y1 || z0 > z1) return;
    const int label = d.labB[S.vox_off + ul];
    const int xy_order[3] = { -1, 0, 1 }, z_order[3] = { 0, -1, 1 };
    for (int z = z0; z <= z1; z++)
        for (int y = y0; y <= y1; y++)
            for (int x = x0; x <= x1; x++) {
                const long long v = S.vox_off + ((long long)z * S.H + y) * S.W + x;
                if (TAKE) {
                    const unsigned long long key = atomicExch(d.jkeys + v, ASV_KEY_EMPTY);
                    if (key != ASV_KEY_EMPTY) d.labA[v] = (int32_t)(key & 0x7fffu);
                    continue;
                }
                const int rank = asv_first_rank_step(z, uz, s, S.D, z_order) * 9 +
                                 asv_first_rank_step(y, uy, s, S.H, xy_order) * 3 +
                                 asv_first_rank_step(x, ux, s, S.W, xy_order);
                const uchar4 c = __ldg(d.lab + v);
                const float dist = asv_jfa_dist(d.jtab + 3 * S.seed_off, label,
                                                make_float2((float)x + 0.5f, (float)y + 0.5f),
                                                make_float2((float)z + 0.5f, (float)c.x),
                                                make_float2((float)c.y, (float)c.z), S.ratio[1]);
                if (!(dist < 100000000.0f)) continue;
                const unsigned long long key = ((unsigned long long)__float_as_uint(dist) << 32) |
                                               ((unsigned long long)rank << 16) | (unsigned long long)label;
                atomicMin(d.jkeys + v, key);
            }
}

// single-segment pass with explicit step and ratio (test entry point)
__global__ void __launch_bounds__(ASV_JFA_THREADS) k_jfa_single(AsvDev d, const int32_t *__restrict__ in,
                                                                int32_t *__restrict__ out, int step,
                                                                float ratio)
{
    extern __shared__ __align__(16) unsigned char asv_jfa_smem[];
    asv_jfa_smem_init(asv_jfa_smem);
    const SegDesc &S = d.segs[0];
    const int tiles_z = (S.D + S.zrun - 1) / S.zrun;
    const int ntiles = S.tiles_x * S.tiles_y * tiles_z;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int tx = t % S.tiles_x, rest = t / S.tiles_x;
        const int ty = rest % S.tiles_y, p0 = (rest / S.tiles_y) * S.zrun;
        asv_jfa_tile<false>(in, out, d.lab + S.vox_off, d.jtab + 3 * S.seed_off, nullptr, 0, S.W, S.H, S.D,
                            S.Kp, tx * ASV_TILE_X, ty * ASV_TILE_Y, p0, S.zrun, step, ratio, asv_jfa_smem);
    }
}

// ---------------------------------------------------------------------------
// Centroid sums (centroids.vs:19-54): per label slot (label -1 -> slot Kp)
// sum(2x+1), sum(2y+1), sum(2z+1), count, sum L, a, b -- exact integers.
// Lanes with the same label are reduced in the warp, then one u64 atomic per
// group and component.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_centroids(AsvDev d)
{
    int si = asv_find_seg(d.chunk_prefix, d.nseg, blockIdx.x);
    const SegDesc &S = d.segs[si];
    const int W = S.W, H = S.H;
    const int32_t *lbl = (S.final_buf ? d.labB : d.labA) + S.vox_off;
    const uchar4 *lab = d.lab + S.vox_off;
    unsigned long long *sums = d.sums + 8ull * S.seed_off;
    long long base = (long long)(blockIdx.x - d.chunk_prefix[si]) * ASV_CHUNK;
    const int lane = threadIdx.x & 31;
    for (int i = 0; i < ASV_CHUNK / 256; i++) {
        long long v = base + i * 256 + threadIdx.x;
        int key = -1;
        unsigned q[7] = { 0, 0, 0, 0, 0, 0, 0 };
        if (v < S.nvox) {
            int l = __ldg(lbl + v);
            key = (l < 0 || l >= S.Kp) ? S.Kp : l;   // out-of-range ids (never produced) count as -1
            int x = (int)(v % W);
            long long r = v / W;
            int y = (int)(r % H), z = (int)(r / H);
            uchar4 c = __ldg(lab + v);
            q[0] = 2 * x + 1; q[1] = 2 * y + 1; q[2] = 2 * z + 1; q[3] = 1;
            q[4] = c.x; q[5] = c.y; q[6] = c.z;
        }
        unsigned grp = __match_any_sync(FULL, key);
        unsigned s[7];
#pragma unroll
        for (int k = 0; k < 7; k++) s[k] = __reduce_add_sync(grp, q[k]);
        if (key >= 0 && lane == __ffs(grp) - 1) {
            unsigned long long *dst = sums + 8ull * key;
#pragma unroll
            for (int k = 0; k < 7; k++) atomicAdd(dst + k, (unsigned long long)s[k]);
        }
    }
}

// ---------------------------------------------------------------------------
// Reseed (aver_exception.vs:22-81).  Alive seed: position floor(mean)+0.5,
// colour = mean LAB.  Dead seed: midpoint of the means of slots id-1 and
// id+1 (id 0 reads texel (W-1, 0); slot Kp is the -1 slot), colour sampled
// at the new position.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void asv_slot_mean(const unsigned long long *sums, int Kp, int slot,
                                              float q[3])
{
    if (slot < 0 || slot > Kp) { q[0] = q[1] = q[2] = 0.0f; return; }
    const unsigned long long *s = sums + 8ull * slot;
    float cnt = __ull2float_rn(s[3]);
#pragma unroll
    for (int a = 0; a < 3; a++) {
        float sf = __ull2float_rn(s[a]) * 0.5f;
        q[a] = ((int)cnt != 0) ? sf / cnt : sf;
    }
}

__global__ void k_finalize(AsvDev d)
{
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= d.total_seeds) return;
    int id;
    int si = asv_seed_seg(d, g, id);
    const SegDesc &S = d.segs[si];
    if (id >= S.Kp) return;
    const unsigned long long *sums = d.sums + 8ull * S.seed_off;
    const unsigned long long *s = sums + 8ull * id;
    float p[3], c[3];
    if (s[3] != 0) {
        float cnt = __ull2float_rn(s[3]);
#pragma unroll
        for (int a = 0; a < 3; a++) {
            float sf = __ull2float_rn(s[a]) * 0.5f;
            p[a] = floorf(sf / cnt) + 0.5f;
            c[a] = __ull2float_rn(s[4 + a]) / cnt;
        }
    } else {
        float q1[3], q2[3];
        asv_slot_mean(sums, S.Kp, id == 0 ? S.W - 1 : id - 1, q1);
        asv_slot_mean(sums, S.Kp, id + 1, q2);
#pragma unroll
        for (int a = 0; a < 3; a++) p[a] = floorf(0.5f * (q1[a] + q2[a])) + 0.5f;
        int x = min(max((int)floorf(p[0]), 0), S.W - 1);
        int y = min(max((int)floorf(p[1]), 0), S.H - 1);
        int z = min(max((int)floorf(p[2]), 0), S.D - 1);
        uchar4 l = d.lab[S.vox_off + ((long long)z * S.H + y) * S.W + x];
        c[0] = l.x; c[1] = l.y; c[2] = l.z;
    }
    d.pos[g] = make_float4(p[0], p[1], p[2], (float)id);
    d.slab[g] = make_float4(c[0], c[1], c[2], 0.0f);
}

// ---------------------------------------------------------------------------
// Post-processing (GPU-AS/Image.cpp:1579-1778).
//   k_post_stats: one block per segment -- dead seeds, alive ranks, the
//     relabel LUT of the <= 3 dead case, mode and -1 flags.
//   k_post_chunk_max / k_post_prefix / k_post_apply: forward fills of the
//     reference's raster loops as a max-scan of "source" voxel indices.
// The post-processed labels go to the buffer the last pass did not write.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_post_stats(AsvDev d)
{
    const int si = blockIdx.x;
    const SegDesc &S = d.segs[si];
    const int Kp = S.Kp;
    const unsigned long long *sums = d.sums + 8ull * S.seed_off;
    int *rank = d.rank + S.seed_off;
    int *rec = d.post + si * ASV_POST_WORDS;
    __shared__ int warp_tot[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    // alive rank: exclusive scan of (count >= 1) in seed order (:1603-1618)
    for (int b0 = 0; b0 < Kp; b0 += blockDim.x) {
        int i = b0 + threadIdx.x;
        int alive = (i < Kp && sums[8ull * i + 3] >= 1) ? 1 : 0;
        unsigned bal = __ballot_sync(FULL, alive);
        int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        int pre = __popc(bal & ((1u << lane) - 1u));
        if (lane == 0) warp_tot[w] = __popc(bal);
        __syncthreads();
        if (threadIdx.x < 32) {
            int v = threadIdx.x < (blockDim.x >> 5) ? warp_tot[threadIdx.x] : 0;
            int incl = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int n = __shfl_up_sync(FULL, incl, o);
                if (threadIdx.x >= o) incl += n;
            }
            warp_tot[threadIdx.x] = incl - v;   // exclusive
        }
        __syncthreads();
        if (i < Kp) {
            const int live_before = carry + warp_tot[w] + pre;
            rank[i] = alive ? live_before : -1;
            const int dead_before = i - live_before;        // the first four dead seeds, in order
            if (!alive && dead_before < 4) rec[POST_DEAD0 + dead_before] = i;
        }
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry += warp_tot[w] + pre + alive;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        int valid = carry, dead = Kp - valid;
        long long negc = (long long)sums[8ull * Kp + 3];
        rec[POST_DEAD] = dead;
        rec[POST_NEG] = negc > 0x7fffffffLL ? 0x7fffffff : (int)negc;
        rec[POST_VALID] = valid;
        rec[POST_INVALID] = negc > 0 ? 1 : 0;
        int mode = dead == 0 ? 0 : (dead <= 3 ? 1 : 2);
        rec[POST_MODE] = mode;
        const int32_t *lbl = (S.final_buf ? d.labB : d.labA) + S.vox_off;
        int l0 = lbl[0];
        rec[POST_L0] = l0;
        rec[POST_M0] = (l0 >= 0 && l0 < Kp && rank[l0] >= 0) ? rank[l0] : 0;
    }
}

// relabelled value of a raw label before the fills (the <= 3 dead relabel
// of label_replace.gs:26-29 applied in order, :1652-1673)
__device__ __forceinline__ int asv_relabel(const int *rec, int Kp, int l)
{
    if (rec[POST_MODE] != 1 || l < 0) return l;
    int last = Kp;
    for (int k = 0; k < rec[POST_DEAD]; k++) {
        last -= 1;
        if (l == last) l = rec[POST_DEAD0 + k];
    }
    return l;
}

// source index of voxel v for the forward fill, or -1
__device__ __forceinline__ long long asv_fill_src(const int *rec, int Kp, long long v, int l)
{
    if (rec[POST_MODE] == 2) {                                  // :1738-1746
        if (v == 0) return 0;
        return (l != rec[POST_L0] && l != -1) ? v : -1;
    }
    int r = asv_relabel(rec, Kp, l);                            // :1763-1775
    if (v == 0) return 0;
    return r != -1 ? v : -1;
}

__device__ __forceinline__ bool asv_needs_scan(const int *rec)
{
    return rec[POST_MODE] == 2 || rec[POST_INVALID] != 0;
}

__global__ void __launch_bounds__(256) k_post_chunk_max(AsvDev d)
{
    int si = asv_find_seg(d.chunk_prefix, d.nseg, blockIdx.x);
    const SegDesc &S = d.segs[si];
    const int *rec = d.post + si * ASV_POST_WORDS;
    if (!asv_needs_scan(rec)) return;
    const int32_t *lbl = (S.final_buf ? d.labB : d.labA) + S.vox_off;
    long long base = (long long)(blockIdx.x - d.chunk_prefix[si]) * ASV_CHUNK;
    long long m = -1;
    for (int i = 0; i < ASV_CHUNK / 256; i++) {
        long long v = base + i * 256 + threadIdx.x;
        if (v < S.nvox) { long long s = asv_fill_src(rec, S.Kp, v, lbl[v]); if (s > m) m = s; }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) { long long n = __shfl_xor_sync(FULL, m, o); if (n > m) m = n; }
    __shared__ long long wm[8];
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long r = wm[0];
        for (int k = 1; k < 8; k++) if (wm[k] > r) r = wm[k];
        // store +1 so that a chunk without source is 0
        d.scan[blockIdx.x] = (int)(r + 1);
    }
}

// exclusive max-scan of the chunk maxima within each segment (1 block / segment)
__global__ void __launch_bounds__(1024) k_post_prefix(AsvDev d)
{
    int si = blockIdx.x;
    const int *rec = d.post + si * ASV_POST_WORDS;
    if (!asv_needs_scan(rec)) return;
    int c0 = d.chunk_prefix[si], c1 = d.chunk_prefix[si + 1];
    __shared__ int carry;
    __shared__ int wmax[32];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int b0 = c0; b0 < c1; b0 += blockDim.x) {
        int c = b0 + threadIdx.x;
        int v = c < c1 ? d.scan[c] : 0;
        int incl = v;
        int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) { int n = __shfl_up_sync(FULL, incl, o); if (lane >= o && n > incl) incl = n; }
        if (lane == 31) wmax[w] = incl;
        __syncthreads();
        if (threadIdx.x < 32) {
            int x = wmax[threadIdx.x];
            int ix = x;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) { int n = __shfl_up_sync(FULL, ix, o); if (threadIdx.x >= o && n > ix) ix = n; }
            wmax[threadIdx.x] = ix;
        }
        __syncthreads();
        int before = w > 0 ? wmax[w - 1] : 0;
        int excl_in_warp = __shfl_up_sync(FULL, incl, 1);
        if (lane == 0) excl_in_warp = 0;
        int ex = max(max(carry, before), excl_in_warp);
        int tot = max(carry, wmax[31]);
        __syncthreads();
        if (c < c1) d.scan[c] = ex;      // max source+1 in earlier chunks of the segment
        if (threadIdx.x == 0) carry = tot;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) k_post_apply(AsvDev d)
{
    int si = asv_find_seg(d.chunk_prefix, d.nseg, blockIdx.x);
    const SegDesc &S = d.segs[si];
    const int *rec = d.post + si * ASV_POST_WORDS;
    const int32_t *lbl = (S.final_buf ? d.labB : d.labA) + S.vox_off;
    int32_t *out = (S.final_buf ? d.labA : d.labB) + S.vox_off;
    const int *rank = d.rank + S.seed_off;
    const int Kp = S.Kp;
    long long base = (long long)(blockIdx.x - d.chunk_prefix[si]) * ASV_CHUNK;
    const bool scan = asv_needs_scan(rec);
    const int mode = rec[POST_MODE];
    // carried source index from earlier chunks (stored +1)
    long long carry = scan ? (long long)d.scan[blockIdx.x] - 1 : -1;
    // each thread owns ASV_CHUNK/256 consecutive voxels for the in-block scan
    const int per = ASV_CHUNK / 256;
    long long v0 = base + (long long)threadIdx.x * per;
    long long m = -1;
    if (scan)
        for (int k = 0; k < per; k++) {
            long long v = v0 + k;
            if (v < S.nvox) { long long s = asv_fill_src(rec, Kp, v, lbl[v]); if (s > m) m = s; }
        }
    // exclusive max-scan of the per-thread maxima across the block
    long long excl = -1;
    if (scan) {
        long long incl = m;
        int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) { long long n = __shfl_up_sync(FULL, incl, o); if (lane >= o && n > incl) incl = n; }
        __shared__ long long wmx[8];
        if (lane == 31) wmx[w] = incl;
        __syncthreads();
        long long before = -1;
        for (int k = 0; k < w; k++) if (wmx[k] > before) before = wmx[k];
        long long ew = __shfl_up_sync(FULL, incl, 1);
        if (lane == 0) ew = -1;
        excl = max(max(before, ew), carry);
    }
    long long src = excl;
    for (int k = 0; k < per; k++) {
        long long v = v0 + k;
        if (v >= S.nvox) break;
        int l = lbl[v];
        int r;
        if (!scan) {
            r = asv_relabel(rec, Kp, l);
        } else {
            long long s = asv_fill_src(rec, Kp, v, l);
            if (s > src) src = s;
            if (mode == 2) {
                // out = map(label at src); src 0 -> map(L0)
                if (src <= 0) r = rec[POST_M0];
                else {
                    int ls = lbl[src];
                    r = (ls >= 0 && ls < Kp && rank[ls] >= 0) ? rank[ls] : 0;
                }
            } else {
                int rl = asv_relabel(rec, Kp, l);
                if (v == 0 || rl != -1) r = rl;
                else if (src >= 1) r = asv_relabel(rec, Kp, lbl[src]);
                else {
                    int r0 = asv_relabel(rec, Kp, lbl[0]);
                    r = r0 >= 0 ? r0 : 0;
                }
            }
        }
        out[v] = r;
    }
}

// ---------------------------------------------------------------------------
// launch wrappers
// ---------------------------------------------------------------------------
static inline int seed_blocks(const AsvDev &d) { return (d.total_seeds + 127) / 128; }

void asv_launch_srgb_table(const AsvDev &d, cudaStream_t st) { k_srgb_table<<<1, 256, 0, st>>>(d.srgb); }
void asv_launch_rgb2lab(const AsvDev &d, cudaStream_t st)
{
    if (d.lablut) k_rgb2lab_lut<<<d.total_chunks, 256, 0, st>>>(d);
    else k_rgb2lab<<<d.total_chunks, 256, 0, st>>>(d);
}

// per-device LAB table (64 MiB), built on first use; nullptr when it cannot
// be allocated (k_rgb2lab then computes every voxel)
const uchar4 *asv_lab_table(int device)
{
    static std::mutex mu;
    static uchar4 *tabs[64] = {};
    static bool tried[64] = {};
    if (device < 0 || device >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(mu);
    if (tried[device]) return tabs[device];
    tried[device] = true;
    float *srgb = nullptr;
    uchar4 *lut = nullptr;
    unsigned *fix = nullptr;                       // entries to recompute, then their count
    cudaStream_t st = nullptr;
    if (cudaMalloc(&srgb, 256 * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&lut, sizeof(uchar4) << 24) != cudaSuccess ||
        cudaMalloc(&fix, (sizeof(unsigned) << 24) + sizeof(unsigned)) != cudaSuccess ||
        cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        if (srgb) cudaFree(srgb);
        if (lut) cudaFree(lut);
        if (fix) cudaFree(fix);
        return nullptr;
    }
    unsigned *nfix = fix + (1u << 24);
    cudaMemsetAsync(nfix, 0, sizeof(unsigned), st);
    k_srgb_table<<<1, 256, 0, st>>>(srgb);
    k_lab_table<<<65536, 256, 0, st>>>(srgb, lut, fix, nfix);
    k_lab_table_fix<<<2048, 256, 0, st>>>(srgb, lut, fix, nfix);
    const bool ok = cudaStreamSynchronize(st) == cudaSuccess && cudaGetLastError() == cudaSuccess;
    cudaStreamDestroy(st);
    cudaFree(srgb);
    cudaFree(fix);
    if (!ok) { cudaFree(lut); return nullptr; }
    tabs[device] = lut;
    return lut;
}
void asv_launch_density(const AsvDev &d, cudaStream_t st) { k_density<<<d.total_chunks, 256, 0, st>>>(d); }
void asv_launch_density_adjust(const AsvDev &d, cudaStream_t st)
{
    k_density_adjust<<<d.nseg, 256, ASV_ADJ_SMEM * sizeof(float), st>>>(d, d.Mring);
}
void asv_launch_first_init(const AsvDev &d, cudaStream_t st) { k_first_init<<<seed_blocks(d), 128, 0, st>>>(d); }
void asv_launch_draw(const AsvDev &d, cudaStream_t st) { k_draw<<<seed_blocks(d), 128, 0, st>>>(d); }

// k_jfa's dynamic shared memory (list rows or bit-set footprint, and the
// bit-set table) exceeds the 48 KiB default: raised once per device
static void asv_jfa_attributes()
{
    static std::mutex mu;
    static bool done[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    if (dev >= 0 && dev < 64 && done[dev]) return;
    cudaFuncSetAttribute(k_jfa, cudaFuncAttributeMaxDynamicSharedMemorySize, ASV_JFA_SMEM);
    cudaFuncSetAttribute(k_jfa_single, cudaFuncAttributeMaxDynamicSharedMemorySize, ASV_JFA_SMEM);
    if (dev >= 0 && dev < 64) done[dev] = true;
}

// resident k_jfa blocks on the device (persistent grid size); computed once
// per process (thread-safe static initialisation)
int asv_jfa_resident_blocks()
{
    static const int blocks = [] {
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        asv_jfa_attributes();
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_jfa, ASV_JFA_THREADS, ASV_JFA_SMEM);
        const int b = sms * (per > 0 ? per : 1);
        return b > 0 ? b : 1024;
    }();
    return blocks;
}

int asv_jfa_grid_blocks(int total_tiles)
{
    const int blocks = asv_jfa_resident_blocks();
    return total_tiles < blocks ? total_tiles : blocks;
}

void asv_launch_jfa(const AsvDev &d, int pass, int grid_blocks, cudaStream_t st)
{
    const int32_t *in = (pass & 1) ? d.labB : d.labA;
    int32_t *out = (pass & 1) ? d.labA : d.labB;
    asv_jfa_attributes();
    k_jfa<<<grid_blocks, 256, ASV_JFA_SMEM, st>>>(d, pass, in, out);
}

void asv_launch_jfa_first_scatter(const AsvDev &d, cudaStream_t st)
{
    cudaMemsetAsync(d.labB, 0xff, sizeof(int32_t) * (size_t)d.total_chunks * ASV_CHUNK, st);
    cudaMemsetAsync(d.tcount, 0, sizeof(int), st);
    const long long threads = 27LL * d.total_seeds;
    const int blocks = (int)((threads + 255) / 256);
    k_jfa_first_scatter<<<blocks, 256, 0, st>>>(d);
    k_jfa_first_take<<<blocks, 256, 0, st>>>(d);
}

void asv_launch_jfa_second_scatter(const AsvDev &d, cudaStream_t st)
{
    cudaMemsetAsync(d.labA, 0xff, sizeof(int32_t) * (size_t)d.total_chunks * ASV_CHUNK, st);
    const long long threads = 27LL * 27LL * d.total_seeds;   // tlist holds <= 27 entries per seed
    const int blocks = (int)((threads + 255) / 256);
    k_jfa_second<false><<<blocks, 256, 0, st>>>(d);
    k_jfa_second<true><<<blocks, 256, 0, st>>>(d);
}

void asv_launch_jfa_single(const AsvDev &d, const int32_t *in, int32_t *out, int step, float ratio,
                           cudaStream_t st)
{
    asv_jfa_attributes();
    k_jfa_single<<<asv_jfa_grid_blocks(d.total_tiles), 256, ASV_JFA_SMEM, st>>>(d, in, out, step, ratio);
}

void asv_launch_centroids(const AsvDev &d, cudaStream_t st) { k_centroids<<<d.total_chunks, 256, 0, st>>>(d); }
void asv_launch_finalize(const AsvDev &d, cudaStream_t st) { k_finalize<<<seed_blocks(d), 128, 0, st>>>(d); }

void asv_launch_post(const AsvDev &d, cudaStream_t st)
{
    k_post_stats<<<d.nseg, 1024, 0, st>>>(d);
    k_post_chunk_max<<<d.total_chunks, 256, 0, st>>>(d);
    k_post_prefix<<<d.nseg, 1024, 0, st>>>(d);
    k_post_apply<<<d.total_chunks, 256, 0, st>>>(d);
}
