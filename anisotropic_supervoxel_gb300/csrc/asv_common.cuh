// asv_common.cuh -- device-side layout shared by the kernels and the host
// orchestration of libasv.
//
// A context holds one or more segments (a clip, a streaming window, or the
// clips of a batch).  All volumes of all segments live in single packed
// device arrays; a segment's voxels start at `vox_off` (a multiple of
// ASV_CHUNK) and its seeds at `seed_off`.  Every kernel covers all segments
// in one launch and finds its segment from a prefix table.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define ASV_MAXP 32          // max JFA passes per Lloyd iteration
#define ASV_CHUNK 2048       // voxels per block in the per-voxel kernels
#define ASV_TILE_X 16        // JFA tile: 16 x 16 columns x SegDesc::zrun chain positions
#define ASV_TILE_Y 16        // (a warp covers 16 x 2 columns: fewer distinct candidates)
#define ASV_RING 24          // 8 one-ring + 16 two-ring neighbours of the metric fallback
#define ASV_POST_WORDS 16    // per-segment post-processing record

struct SegDesc {
    int W, H, D, Kp;
    long long vox_off;       // first voxel of the segment in the packed arrays
    long long nvox;          // W*H*D
    int seed_off;            // first seed slot (Kp+1 slots used: slot Kp = label -1)
    int npass;
    int steps[ASV_MAXP];
    float ratio[ASV_MAXP];   // ratio of each pass (base ratio x 1 or x 2)
    int tiles_x, tiles_y;
    int zrun;                // JFA tile depth: chain positions per column and tile
    int angle_filter;        // plain reseed flow-angle filter
    int wNum, hNum, dNum;    // seed grid (density placement)
    int cell_off;            // x cells at cell_off, y at +W, z at +W+H
    int final_buf;           // 0: last pass wrote buffer A, 1: buffer B
    long long lab_from;      // first voxel whose LAB must be computed (streaming windows keep
                             // the LAB of their overlap frames)
};

// post-processing record per segment (ints), written by k_post_stats
enum {
    POST_DEAD = 0, POST_NEG = 1, POST_VALID = 2, POST_MODE = 3, POST_INVALID = 4,
    POST_L0 = 5, POST_M0 = 6, POST_DEAD0 = 7 /* .. +3: first dead ids */
};

#ifdef __CUDACC__
// Binary search: largest i in [0, n) with prefix[i] <= v.
__device__ __forceinline__ int asv_find_seg(const int *__restrict__ prefix, int n, int v)
{
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (__ldg(prefix + mid) <= v) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ long long asv_find_seg64(const long long *__restrict__ prefix, int n,
                                                    long long v)
{
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (__ldg(prefix + mid) <= v) lo = mid; else hi = mid - 1;
    }
    return lo;
}
#endif

// Host-side launch wrappers (defined in the .cu files, called by asv_api.cpp).
struct AsvDev {
    int nseg;
    const SegDesc *segs;         // device copy
    const int *tile_prefix;      // [nseg+1] JFA tiles
    const int *chunk_prefix;     // [nseg+1] ASV_CHUNK-voxel chunks
    const int *seed_prefix;      // [nseg+1] seed slots (seed_off)
    int total_tiles, total_chunks, total_seeds;
    uint8_t *rgb;                // 3 bytes / voxel
    uchar4 *lab;                 // L, a, b, 0
    float2 *fwd, *bwd;
    int32_t *labA, *labB;
    unsigned long long *jkeys;   // first-pass scatter keys, one per voxel, all ~0 between passes
    unsigned long long *tlist;   // voxels labelled by the first pass: (segment << 32) | voxel, 27 per seed
    int *tcount;                 // entries of tlist
    float4 *pos0;                // initial seeds (density placement)
    float *M0;                   // initial metric, 8 floats / seed
    float4 *pos, *slab;          // working seeds
    float *M;                    // working metric, 8 floats / seed
    float4 *jtab;                // JFA seed table, 3 float4 / seed
    unsigned long long *sums;    // 8 u64 / slot
    float *Mself; int *neg;      // metric scratch
    float *Mmemo; int *mkey;     // reseed memo: metric of the voxel key of the last solve
    float *Mring; int *ringok;
    float4 *grid;                // grid seeds
    unsigned long long *dacc;    // density accumulators (2^-24 units)
    int *cells;                  // cell tables
    int *post;                   // ASV_POST_WORDS / segment
    int *rank;                   // per seed: relabel LUT / alive rank
    int *scan;                   // per chunk
    float *srgb;                 // 256-entry sRGB linearisation
    const uchar4 *lablut;        // LAB of every RGB value (per device, shared), or null
    int *err;                    // device error word
};

void asv_launch_srgb_table(const AsvDev &d, cudaStream_t st);
void asv_launch_rgb2lab(const AsvDev &d, cudaStream_t st);
void asv_launch_preprocess(const uint8_t *bgr, uint8_t *rgb, int W, int H, int D, cudaStream_t st);
const uchar4 *asv_lab_table(int device);
void asv_launch_density(const AsvDev &d, cudaStream_t st);
void asv_launch_density_adjust(const AsvDev &d, cudaStream_t st);
void asv_launch_first_init(const AsvDev &d, cudaStream_t st);
void asv_launch_draw(const AsvDev &d, cudaStream_t st);
void asv_launch_jfa(const AsvDev &d, int pass, int grid_blocks, cudaStream_t st);
void asv_launch_jfa_first_scatter(const AsvDev &d, cudaStream_t st);
void asv_launch_jfa_second_scatter(const AsvDev &d, cudaStream_t st);
void asv_launch_jfa_single(const AsvDev &d, const int32_t *in, int32_t *out, int step, float ratio,
                           cudaStream_t st);
void asv_launch_centroids(const AsvDev &d, cudaStream_t st);
void asv_launch_finalize(const AsvDev &d, cudaStream_t st);
void asv_launch_post(const AsvDev &d, cudaStream_t st);
void asv_launch_metric(const AsvDev &d, int reseed, cudaStream_t st);
int asv_jfa_grid_blocks(int total_tiles);
int asv_jfa_resident_blocks();
