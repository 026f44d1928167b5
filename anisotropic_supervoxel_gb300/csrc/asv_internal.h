// asv_internal.h -- host-side helpers of libasv shared by the C ABI files.
#pragma once

#include "asv.h"
#include "asv_common.cuh"

#include <vector>

namespace asv {

struct GridInfo {
    int s = 0, dNum = 0, hNum = 0, wNum = 0, Kp = 0;
};

// Host description of one segment (clip, window or batch member).
struct SegHost {
    int W = 0, H = 0, D = 0, K = 0, Kp = 0;
    GridInfo g;
    std::vector<float> grid;   // grid seeds, 4 floats each (x, y, z, id)
    std::vector<int> cells;    // x/y/z cell tables + x ranges of the columns
    float ratio = 0.f;
    int npass = 0;
    int steps[ASV_MAXP] = {};
    float rmul[ASV_MAXP] = {};
    long long vox_off = 0;
    int seed_off = 0;
    int dead = 0, neg = 0, valid = 0;
};

int grid_seeds(int W, int H, int D, int K, int middlebury, GridInfo *g, std::vector<float> *seeds4);
size_t ctx_bytes(const asv_ctx *ctx);   // device bytes a context holds
void set_stream(asv_ctx *ctx, cudaStream_t st);   // later work of ctx runs on st (caller-owned)
void cell_tables(int W, int H, int D, const GridInfo &g, const std::vector<float> &grid,
                 std::vector<int> *cells);
float ratio_of(int s, float compactness);
int ladder(int s, int full, int maxdim, int *steps, float *rmul, int cap);

} // namespace asv
