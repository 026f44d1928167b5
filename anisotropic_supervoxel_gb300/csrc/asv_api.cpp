// asv_api.cpp -- host side of the C ABI (include/asv.h): context, device
// memory layout, host seed grid, stage sequencing and CUDA-graph replay.
//
// The stage functions follow the reference's Image methods; the reference
// line ranges are in include/asv.h next to each declaration.
#include "asv.h"
#include "asv_common.cuh"
#include "asv_internal.h"
#include "asv_connect.cuh"
#include "asv_flow.cuh"
#include "asv_eval.cuh"
#include "asv_stream.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace asv {

// ---------------------------------------------------------------------------
// Seed grid (GPU-AS/Image.cpp:20-92; streamGPU-AS/Image.cpp:26-103), host.
// ---------------------------------------------------------------------------
int grid_seeds(int W, int H, int D, int K, int middlebury, GridInfo *g, std::vector<float> *seeds4)
{
    if (W < 1 || H < 1 || D < 1 || K < 1) return -1;
    long long N = (long long)W * H * D;
    double voxel_size = (double)(N / K);
    int s = middlebury ? (int)std::floor(std::pow(1.0 * W * H / K, 0.5))
                       : (int)std::floor(std::pow(voxel_size, 1.0 / 3));
    long long kdd = (long long)K * D * D / W / H;
    int dNum = (int)std::pow((double)(float)kdd, 1.0 / 3.0);
    if (dNum == 0) dNum = 1;
    int fsn = K / dNum;
    int wNum = (int)std::sqrt((float)((long long)fsn * W / H));
    if (wNum == 0) return -2;
    int hNum = fsn / wNum;
    if (hNum == 0) return -2;
    g->s = s; g->dNum = dNum; g->hNum = hNum; g->wNum = wNum; g->Kp = dNum * hNum * wNum;
    if (!seeds4) return g->Kp;
    seeds4->clear();
    int stepD = D / dNum, stepH = H / hNum, stepW = W / wNum;
    int d_rem = D - stepD * dNum, h_rem = H - stepH * hNum, w_rem = W - stepW * wNum;
    int td = d_rem < 1 ? 0 : 1;
    int count = 0;
    for (int k = 0; k < dNum; k++) {
        int th = 1;
        for (int i = 0; i < hNum; i++) {
            int tw = 1;
            for (int j = 0; j < wNum; j++) {
                int sx = (int)(j * stepW + 0.5 * stepW + tw);
                int sy = (int)(i * stepH + 0.5 * stepH + th);
                int sz = (int)(k * stepD + 0.5 * stepD + td);
                sx = std::min(sx, W - 1); sy = std::min(sy, H - 1); sz = std::min(sz, D - 1);
                if (tw < w_rem) tw++;
                seeds4->push_back((float)(sx + 0.5));
                seeds4->push_back((float)(sy + 0.5));
                seeds4->push_back((float)(sz + 0.5));
                seeds4->push_back((float)count++);
            }
            if (th < h_rem) th++;
        }
        if (td < d_rem) td++;
    }
    return g->Kp;
}

// cell tables of the density placement (Image.cpp:360-468): per x (y, z)
// the largest grid column (row, layer) whose range holds it, then the x
// ranges of the columns.
void cell_tables(int W, int H, int D, const GridInfo &g, const std::vector<float> &grid,
                 std::vector<int> *cells)
{
    auto mid = [](float a, float b) { return (int)std::floor(0.5 * (double)(a + b)); };
    std::vector<int> xl(g.wNum), xr(g.wNum), yl(g.hNum), yr(g.hNum), zl(g.dNum), zr(g.dNum);
    for (int i = 0; i < g.wNum; i++) {
        float c = grid[4 * i];
        xl[i] = i > 0 ? mid(grid[4 * (i - 1)], c) : 0;
        xr[i] = i < g.wNum - 1 ? mid(grid[4 * (i + 1)], c) : W - 1;
    }
    for (int j = 0; j < g.hNum; j++) {
        float c = grid[4 * (j * g.wNum) + 1];
        yl[j] = j > 0 ? mid(grid[4 * ((j - 1) * g.wNum) + 1], c) : 0;
        yr[j] = j < g.hNum - 1 ? mid(grid[4 * ((j + 1) * g.wNum) + 1], c) : H - 1;
    }
    for (int t = 0; t < g.dNum; t++) {
        float c = grid[4 * (t * g.wNum * g.hNum) + 2];
        zl[t] = t > 0 ? mid(grid[4 * ((t - 1) * g.wNum * g.hNum) + 2], c) : 0;
        zr[t] = t < g.dNum - 1 ? mid(grid[4 * ((t + 1) * g.wNum * g.hNum) + 2], c) : D - 1;
    }
    cells->assign((size_t)W + H + D + 2 * g.wNum, -1);
    for (int x = 0; x < W; x++) for (int i = 0; i < g.wNum; i++) if (xl[i] <= x && x <= xr[i]) (*cells)[x] = i;
    for (int y = 0; y < H; y++) for (int j = 0; j < g.hNum; j++) if (yl[j] <= y && y <= yr[j]) (*cells)[W + y] = j;
    for (int z = 0; z < D; z++) for (int t = 0; t < g.dNum; t++) if (zl[t] <= z && z <= zr[t]) (*cells)[W + H + z] = t;
    for (int i = 0; i < g.wNum; i++) { (*cells)[W + H + D + i] = xl[i]; (*cells)[W + H + D + g.wNum + i] = xr[i]; }
}

float ratio_of(int s, float compactness)
{
    float q = compactness / (float)s;
    return q * q;
}

// JFA ladder (GPU-AS/Image.cpp:1055-1190): [1] + [floor(s/2) halving with
// floor(x/2+0.5) down to 1] + [2, 1] (last two at 2x ratio).
int ladder(int s, int full, int maxdim, int *steps, float *rmul, int cap)
{
    int n = 0;
    auto push = [&](int st, float rm) { if (n < cap) { steps[n] = st; rmul[n] = rm; } n++; };
    push(1, 1.0f);
    if (!full) {
        float st = (float)std::floor(0.5 * s);
        while (st > 0) {
            push((int)st, 1.0f);
            if ((int)st == 1) st = 0;
            st = (float)std::floor(0.5 * st + 0.5);
        }
    } else {
        int p = 1;
        while (p * 2 <= maxdim) p *= 2;
        for (; p >= 1; p /= 2) push(p, 1.0f);
    }
    push(2, 2.0f);
    push(1, 2.0f);
    return n;
}

} // namespace asv

using namespace asv;

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
struct asv_ctx {
    asv_config cfg;
    cudaStream_t st = nullptr;
    bool own_st = false;
    std::string err;
    // layout
    std::vector<SegHost> seg;
    std::vector<SegDesc> sd;
    AsvDev d{};
    std::vector<void *> allocs;
    size_t bytes = 0;
    int jfa_blocks = 0;
    int maxpass = 0;
    // state
    bool have_rgb = false, have_flow = false, have_pos0 = false, have_M0 = false, have_lab = false;
    bool seeded = false, ran = false;
    bool drawn = false;          // labA holds a fresh seed draw: the first pass may scatter
    int post_host[ASV_POST_WORDS];
    // graph
    cudaGraphExec_t gexec = nullptr;
    // instrumentation
    asv_stats stats{};
    std::vector<cudaEvent_t> ev;
    int launches = 0;
    // batched form: which clips have their inputs on the device
    std::vector<uint8_t> up_rgb, up_flow;
    // streaming form (asv_stream_*)
    struct Stream {
        bool on = false;
        int W = 0, H = 0, D_all = 0, bs = 30, seeds100 = 0, nb = 0, next = 0, prev_Db = 0;
        int Kcap = 0, Dcap = 0;
        std::vector<int> iv;   // block intervals [start, end)
        StreamDev s{};
        int placed = 0, kept = 0, last_Kp = 0;
        // blocks fed ahead (asv_stream_feed): two staging slots of new frames
        int fed_next = 0;                          // the block the next feed takes
        int fed_n[2] = { 0, 0 };                   // new frames held by each slot
        bool fed_devflow[2] = { false, false };    // fed without flow: flow on the device
        bool fed_bgr[2] = { false, false };        // fed as decoded BGR: preprocessed on the device
        uint8_t *stg_rgb[2] = { nullptr, nullptr };
        float *stg_fwd[2] = { nullptr, nullptr }, *stg_bwd[2] = { nullptr, nullptr };
        // pinned host staging of a block's small copies (in the context's
        // pinned block hpin), so that none of them is a synchronous copy
        // from pageable memory: prefixes, the segment descriptor, the
        // counters after the seed composition and at the end, cells, grid
        // (one set per block parity: two blocks can be in flight)
        int *h_pref[2] = {}, *h_ctr[2] = {}, *h_ctr2[2] = {}, *h_cells[2] = {};
        SegDesc *h_sdA[2] = {};
        float4 *h_grid[2] = {};
        size_t h_cells_cap = 0;
        // blocks enqueued and not yet finished (asv_stream_push_fed_async /
        // asv_stream_wait), oldest first
        struct Flight { int block = -1, done = 0, launches = 0; };
        Flight flight[2];
        int nflight = 0;
        bool failed = false;                       // a block was refused: the stream is over
    } sm;
    // per block parity: device time start, end, and everything read back
    cudaEvent_t sev[6] = {};
    void *hpin = nullptr;                     // pinned host block of the streaming form
    size_t hpin_bytes = 0;
    // the streaming form's Lloyd loop as a CUDA graph, replayed by every
    // window whose launch configuration (device pointers and totals, JFA grid,
    // pass count) equals the one it was captured with: the per-window data
    // (seed counts, segment descriptor) is read from device memory
    cudaGraphExec_t sgexec = nullptr;
    AsvDev skey{};
    int skey_blocks = -1, skey_passes = -1, skey_iters = -1, sg_launches = 0;
    // copy stream of asv_stream_feed and its events (created on first use):
    // fed_ev[k] = slot k's upload done, used_ev[k] = slot k read by its push
    cudaStream_t cp = nullptr;
    cudaEvent_t fed_ev[2] = { nullptr, nullptr }, used_ev[2] = { nullptr, nullptr }, alloc_ev = nullptr;
    // connectivity enforcement scratch (asv_enforce_connectivity*), grown on demand
    void *cc = nullptr;
    size_t cc_bytes = 0;
    // optical-flow scratch (asv_compute_flow), grown on demand
    void *fl = nullptr;
    size_t fl_bytes = 0;
};

size_t asv::ctx_bytes(const asv_ctx *c) { return c ? c->bytes + c->cc_bytes + c->fl_bytes : 0; }

void asv::set_stream(asv_ctx *c, cudaStream_t st)
{
    if (!c || c->st == st) return;
    cudaStreamSynchronize(c->st);
    if (c->own_st) cudaStreamDestroy(c->st);
    c->st = st;
    c->own_st = false;
}

static asv_status fail(asv_ctx *c, asv_status s, const std::string &m)
{
    if (c) c->err = m;
    return s;
}

static asv_status cuda_fail(asv_ctx *c, cudaError_t e, const char *where)
{
    return fail(c, ASV_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                                     \
    do {                                                             \
        cudaError_t e_ = (call);                                     \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call);     \
    } while (0)

// JFA grid: a persistent grid of the resident blocks, or one block per tile
static int jfa_blocks_for(const asv_ctx *ctx, int tiles)
{
    tiles = std::max(tiles, 1);
    return ctx->cfg.jfa_tile_blocks ? tiles : asv_jfa_grid_blocks(tiles);
}

// Device memory of a context is stream-ordered: cudaMallocAsync and
// cudaFreeAsync on the context's stream, from the device's default memory
// pool.  A free waits for the context's own earlier work only, so a context
// that changes shape or is destroyed never synchronizes the device and the
// other contexts sharing the GPU (the server's slots) keep running.  The
// context's stream changes only after a synchronize (asv::set_stream), so a
// buffer is always allocated, used and freed in stream order.
static cudaError_t ctx_malloc(asv_ctx *ctx, void **p, size_t b) { return cudaMallocAsync(p, b, ctx->st); }

static void ctx_free(asv_ctx *ctx, void *p)
{
    if (p) cudaFreeAsync(p, ctx->st);
}

static void free_layout(asv_ctx *ctx)
{
    if (ctx->cp) cudaStreamSynchronize(ctx->cp);   // uploads into the staging slots end first
    if (ctx->gexec) { cudaGraphExecDestroy(ctx->gexec); ctx->gexec = nullptr; }
    if (ctx->sgexec) { cudaGraphExecDestroy(ctx->sgexec); ctx->sgexec = nullptr; ctx->skey_blocks = -1; }
    for (void *p : ctx->allocs) ctx_free(ctx, p);
    ctx->allocs.clear();
    ctx->bytes = 0;
    ctx->d = AsvDev{};
    ctx->have_rgb = ctx->have_flow = ctx->have_pos0 = ctx->have_M0 = ctx->have_lab = false;
    ctx->seeded = ctx->ran = ctx->drawn = false;
    ctx->sm.on = false;
}

template <typename T>
static asv_status dalloc(asv_ctx *ctx, T **p, size_t n)
{
    size_t b = std::max<size_t>(n, 1) * sizeof(T);
    b = (b + 255) & ~(size_t)255;
    if (ctx->cfg.hbm_budget && ctx->bytes + b > ctx->cfg.hbm_budget)
        return fail(ctx, ASV_ERR_OVER_BUDGET, "allocation exceeds the configured HBM budget");
    void *q = nullptr;
    cudaError_t e = ctx_malloc(ctx, &q, b);
    if (e != cudaSuccess) { cudaGetLastError(); return fail(ctx, ASV_ERR_OOM, std::string("cudaMallocAsync: ") + cudaGetErrorString(e)); }
    ctx->allocs.push_back(q);
    ctx->bytes += b;
    *p = (T *)q;
    return ASV_OK;
}

#define AL(ptr, n)                                              \
    do {                                                        \
        asv_status s_ = dalloc(ctx, &(ptr), (n));               \
        if (s_ != ASV_OK) { free_layout(ctx); return s_; }      \
    } while (0)

// Prepares one segment's host description (grid, ladder, cells).
asv_status asv_prepare_segment(asv_ctx *ctx, int W, int H, int D, int K, SegHost *sh)
{
    if (W < 1 || H < 1 || D < 2 || W > 4096 || H > 4096 || D > 4096 || K < 1)
        return fail(ctx, ASV_ERR_BAD_ARG, "need 1 <= W,H <= 4096, 2 <= D <= 4096, K >= 1");
    if ((long long)W * H * D >= (1LL << 31))
        return fail(ctx, ASV_ERR_BAD_ARG, "a clip holds fewer than 2^31 voxels");
    sh->W = W; sh->H = H; sh->D = D; sh->K = K;
    if (grid_seeds(W, H, D, K, ctx->cfg.middlebury, &sh->g, &sh->grid) <= 0)
        return fail(ctx, ASV_ERR_BAD_ARG, "K too small for the seed grid (no column or row)");
    if (sh->g.Kp >= 32768) return fail(ctx, ASV_ERR_BAD_ARG, "more than 32767 seeds");
    if (sh->g.s < 1) return fail(ctx, ASV_ERR_BAD_ARG, "K larger than the voxel count");
    sh->Kp = sh->g.Kp;
    float compact = ctx->cfg.variant == ASV_VARIANT_STREAM ? 6.0f : 8.0f;
    sh->ratio = ratio_of(sh->g.s, compact);
    int maxdim = std::max(W, std::max(H, D));
    sh->npass = ladder(sh->g.s, ctx->cfg.full_ladder, maxdim, sh->steps, sh->rmul, ASV_MAXP);
    if (sh->npass > ASV_MAXP) return fail(ctx, ASV_ERR_BAD_ARG, "JFA ladder longer than 32 passes");
    cell_tables(W, H, D, sh->g, sh->grid, &sh->cells);
    return ASV_OK;
}

size_t asv_layout_bytes(const std::vector<SegHost> &seg)
{
    size_t vox = 0, seeds = 0, cells = 0, chunks = 0;
    for (auto &s : seg) {
        long long n = (long long)s.W * s.H * s.D;
        vox += (size_t)((n + ASV_CHUNK - 1) / ASV_CHUNK) * ASV_CHUNK;
        chunks += (size_t)((n + ASV_CHUNK - 1) / ASV_CHUNK);
        seeds += (size_t)((s.Kp + 64 + 31) / 32) * 32;
        cells += s.W + s.H + s.D + 2 * s.g.wNum;
    }
    // rgb 3 + lab 4 + fwd/bwd 16 + two label buffers 8 + first-pass keys 8
    size_t per_vox = 3 + 4 + 8 + 8 + 4 + 4 + 8;
    // float4 pos0/pos/slab/grid, 8-float M0/M/Mself/Mmemo, jtab 3 float4, 8 u64
    // sums, int neg/mkey/rank, u64 dacc, the metric ring
    size_t per_seed = 4 * 16 + 4 * 32 + 3 * 16 + 8 * 8 + 3 * 4 + 8 + ASV_RING * (32 + 4) + 27 * 8;
    // each of the ~30 allocations rounds up to 256 bytes
    size_t fixed = 32 * 256 + 256 * 4 + 16;
    size_t per_seg = sizeof(SegDesc) + 3 * 4 + ASV_POST_WORDS * 4;
    return vox * per_vox + seeds * per_seed + cells * 4 + chunks * 4 + fixed + seg.size() * per_seg;
}

// JFA tile depth for a set of segments: the configured one, else the
// deepest of 32/16/8 that still gives every resident block four tiles
// (deeper runs share more slices; shallower ones balance the GPU), else 4.
static int pick_zrun(const asv_ctx *ctx, const std::vector<SegHost> &seg)
{
    if (ctx->cfg.jfa_zrun > 0) return std::min(ctx->cfg.jfa_zrun, 256);
    const long long want = 4LL * asv_jfa_resident_blocks();
    for (int z : { 32, 16, 8 }) {
        long long tiles = 0;
        for (const SegHost &h : seg)
            tiles += (long long)((h.W + ASV_TILE_X - 1) / ASV_TILE_X) * ((h.H + ASV_TILE_Y - 1) / ASV_TILE_Y)
                     * ((h.D + z - 1) / z);
        if (tiles >= want) return z;
    }
    return 4;
}

// Allocates the packed device arrays for the segments in ctx->seg.
asv_status asv_build_layout(asv_ctx *ctx)
{
    free_layout(ctx);
    const int nseg = (int)ctx->seg.size();
    std::vector<int> tile_p(nseg + 1), chunk_p(nseg + 1), seed_p(nseg + 1);
    long long vox = 0;
    int tiles = 0, chunks = 0, seeds = 0, cells = 0;
    ctx->sd.assign(nseg, SegDesc{});
    ctx->maxpass = 0;
    const int zrun = pick_zrun(ctx, ctx->seg);
    for (int i = 0; i < nseg; i++) {
        SegHost &h = ctx->seg[i];
        SegDesc &s = ctx->sd[i];
        long long n = (long long)h.W * h.H * h.D;
        s.W = h.W; s.H = h.H; s.D = h.D; s.Kp = h.Kp;
        s.vox_off = vox; s.nvox = n;
        s.seed_off = seeds;
        s.npass = h.npass;
        for (int p = 0; p < h.npass; p++) { s.steps[p] = h.steps[p]; s.ratio[p] = h.rmul[p] * h.ratio; }
        s.tiles_x = (h.W + ASV_TILE_X - 1) / ASV_TILE_X;
        s.tiles_y = (h.H + ASV_TILE_Y - 1) / ASV_TILE_Y;
        s.zrun = zrun;
        s.angle_filter = ctx->cfg.variant == ASV_VARIANT_PLAIN ? 1 : 0;
        s.wNum = h.g.wNum; s.hNum = h.g.hNum; s.dNum = h.g.dNum;
        s.cell_off = cells;
        s.final_buf = h.npass & 1;
        h.vox_off = vox; h.seed_off = seeds;
        tile_p[i] = tiles; chunk_p[i] = chunks; seed_p[i] = seeds;
        int nchunk = (int)((n + ASV_CHUNK - 1) / ASV_CHUNK);
        vox += (long long)nchunk * ASV_CHUNK;
        chunks += nchunk;
        tiles += s.tiles_x * s.tiles_y * ((h.D + zrun - 1) / zrun);
        seeds += ((h.Kp + 64 + 31) / 32) * 32;
        cells += h.W + h.H + h.D + 2 * h.g.wNum;
        ctx->maxpass = std::max(ctx->maxpass, h.npass);
    }
    tile_p[nseg] = tiles; chunk_p[nseg] = chunks; seed_p[nseg] = seeds;
    AsvDev &d = ctx->d;
    d.nseg = nseg;
    d.total_tiles = tiles; d.total_chunks = chunks; d.total_seeds = seeds;
    SegDesc *segs; int *tp, *cp, *sp;
    AL(segs, nseg); AL(tp, nseg + 1); AL(cp, nseg + 1); AL(sp, nseg + 1);
    d.segs = segs; d.tile_prefix = tp; d.chunk_prefix = cp; d.seed_prefix = sp;
    AL(d.rgb, (size_t)vox * 3);
    AL(d.lab, (size_t)vox);
    AL(d.fwd, (size_t)vox);
    AL(d.bwd, (size_t)vox);
    AL(d.labA, (size_t)vox);
    AL(d.labB, (size_t)vox);
    AL(d.jkeys, (size_t)vox);
    AL(d.tlist, (size_t)seeds * 27);
    AL(d.tcount, 1);
    CK(cudaMemsetAsync(d.jkeys, 0xff, sizeof(unsigned long long) * (size_t)vox, ctx->st));
    AL(d.pos0, seeds); AL(d.M0, (size_t)seeds * 8);
    AL(d.pos, seeds); AL(d.slab, seeds); AL(d.M, (size_t)seeds * 8);
    AL(d.jtab, (size_t)seeds * 3);
    AL(d.sums, (size_t)seeds * 8);
    AL(d.Mself, (size_t)seeds * 8); AL(d.neg, seeds);
    AL(d.Mmemo, (size_t)seeds * 8); AL(d.mkey, seeds);
    AL(d.Mring, (size_t)seeds * ASV_RING * 8); AL(d.ringok, (size_t)seeds * ASV_RING);
    AL(d.grid, seeds);
    AL(d.dacc, seeds);
    AL(d.cells, std::max(cells, 1));
    AL(d.post, (size_t)nseg * ASV_POST_WORDS);
    AL(d.rank, seeds);
    AL(d.scan, std::max(chunks, 1));
    AL(d.srgb, 256);
    AL(d.err, 4);
    CK(cudaMemcpyAsync(segs, ctx->sd.data(), sizeof(SegDesc) * nseg, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(tp, tile_p.data(), sizeof(int) * (nseg + 1), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(cp, chunk_p.data(), sizeof(int) * (nseg + 1), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(sp, seed_p.data(), sizeof(int) * (nseg + 1), cudaMemcpyHostToDevice, ctx->st));
    std::vector<int> allcells((size_t)std::max(cells, 1), -1);
    std::vector<float4> grid((size_t)seeds, make_float4(0, 0, 0, -1));
    for (int i = 0; i < nseg; i++) {
        SegHost &h = ctx->seg[i];
        std::copy(h.cells.begin(), h.cells.end(), allcells.begin() + ctx->sd[i].cell_off);
        for (int k = 0; k < h.Kp; k++)
            grid[h.seed_off + k] = make_float4(h.grid[4 * k], h.grid[4 * k + 1], h.grid[4 * k + 2], h.grid[4 * k + 3]);
    }
    CK(cudaMemcpyAsync(d.cells, allcells.data(), sizeof(int) * allcells.size(), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(d.grid, grid.data(), sizeof(float4) * grid.size(), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemsetAsync(d.post, 0, sizeof(int) * nseg * ASV_POST_WORDS, ctx->st));
    CK(cudaMemsetAsync(d.err, 0, 16, ctx->st));
    CK(cudaMemsetAsync(d.pos0, 0, sizeof(float4) * seeds, ctx->st));
    CK(cudaMemsetAsync(d.pos, 0, sizeof(float4) * seeds, ctx->st));
    CK(cudaMemsetAsync(d.slab, 0, sizeof(float4) * seeds, ctx->st));
    CK(cudaMemsetAsync(d.M0, 0, sizeof(float) * 8 * seeds, ctx->st));
    CK(cudaMemsetAsync(d.M, 0, sizeof(float) * 8 * seeds, ctx->st));
    asv_launch_srgb_table(d, ctx->st);
    CK(cudaGetLastError());
    d.lablut = asv_lab_table(ctx->cfg.device);
    ctx->jfa_blocks = jfa_blocks_for(ctx, tiles);
    return ASV_OK;
}

// ---------------------------------------------------------------------------
// stage sequencing
// ---------------------------------------------------------------------------
static void rec_begin(asv_ctx *ctx, int idx)
{
    if (ctx->cfg.instrument && !ctx->gexec) cudaEventRecord(ctx->ev[idx], ctx->st);
}

static asv_status ensure_events(asv_ctx *ctx, size_t n)
{
    while (ctx->ev.size() < n) {
        cudaEvent_t e;
        CK(cudaEventCreate(&e));
        ctx->ev.push_back(e);
    }
    return ASV_OK;
}

static void do_first_init(asv_ctx *ctx)
{
    asv_launch_first_init(ctx->d, ctx->st);
    cudaMemsetAsync(ctx->d.labA, 0xff, sizeof(int32_t) * (size_t)ctx->d.total_chunks * ASV_CHUNK, ctx->st);
    asv_launch_draw(ctx->d, ctx->st);
    ctx->drawn = true;
    ctx->launches += 2;
}

// the JFA ladder; the last pass of each segment also forms its centroid sums
static void do_flood(asv_ctx *ctx, int evbase)
{
    cudaMemsetAsync(ctx->d.sums, 0, sizeof(unsigned long long) * 8 * (size_t)ctx->d.total_seeds, ctx->st);
    for (int p = 0; p < ctx->maxpass; p++) {
        if (evbase >= 0) rec_begin(ctx, evbase + 2 * p);
        if (p == 0 && ctx->drawn) {
            asv_launch_jfa_first_scatter(ctx->d, ctx->st);   // step 1 from the drawn seeds
            ctx->launches += 2;
        } else if (p == 1 && ctx->drawn) {
            asv_launch_jfa_second_scatter(ctx->d, ctx->st);  // from the first pass's sparse labels
            ctx->launches += 2;
        } else {
            asv_launch_jfa(ctx->d, p, ctx->jfa_blocks, ctx->st);
            ctx->launches++;
        }
        if (evbase >= 0) rec_begin(ctx, evbase + 2 * p + 1);
    }
    ctx->drawn = false;
}

// the reseed of centroids_next_seeds (the sums came with the flood)
static void do_centroids(asv_ctx *ctx, bool reseed)
{
    if (reseed) { asv_launch_finalize(ctx->d, ctx->st); ctx->launches++; }
}

// per-label sums of the labels in the final buffers (caller-supplied labels)
static void do_sums_from_labels(asv_ctx *ctx)
{
    cudaMemsetAsync(ctx->d.sums, 0, sizeof(unsigned long long) * 8 * (size_t)ctx->d.total_seeds, ctx->st);
    asv_launch_centroids(ctx->d, ctx->st);
    ctx->launches++;
}

static void do_next_seeds(asv_ctx *ctx)
{
    asv_launch_metric(ctx->d, 1, ctx->st);
    cudaMemsetAsync(ctx->d.labA, 0xff, sizeof(int32_t) * (size_t)ctx->d.total_chunks * ASV_CHUNK, ctx->st);
    asv_launch_draw(ctx->d, ctx->st);
    ctx->drawn = true;
    ctx->launches += 6;       // five metric kernels + the seed draw
}

static void do_post(asv_ctx *ctx)
{
    asv_launch_post(ctx->d, ctx->st);
    ctx->launches += 4;
}

// the Lloyd loop of Render::run (GPU-AS/Render.cpp:277-303)
static void enqueue_lloyd(asv_ctx *ctx, bool instrument)
{
    const int I = ctx->cfg.lloyd_iters;
    const int per_it = 2 * ctx->maxpass;
    do_first_init(ctx);
    for (int it = 1; it <= I; it++) {
        if (it > 1) do_next_seeds(ctx);
        do_flood(ctx, instrument ? (it - 1) * per_it : -1);
        do_centroids(ctx, it != I);
    }
    do_post(ctx);
}

static asv_status check_ready(asv_ctx *ctx)
{
    if (ctx->seg.empty()) return fail(ctx, ASV_ERR_STATE, "no clip: call asv_init_gpu first");
    if (!ctx->have_flow) return fail(ctx, ASV_ERR_STATE, "no flow: call asv_upload_flow first");
    if (!ctx->have_pos0) return fail(ctx, ASV_ERR_STATE, "no seeds: call asv_initialization first");
    if (!ctx->have_M0) return fail(ctx, ASV_ERR_STATE, "no metric: call asv_seed_matrix first");
    if (!ctx->have_lab) return fail(ctx, ASV_ERR_STATE, "no LAB volume: call asv_rgb2lab first");
    return ASV_OK;
}

static asv_status read_post(asv_ctx *ctx)
{
    std::vector<int> rec(ctx->seg.size() * ASV_POST_WORDS);
    CK(cudaMemcpyAsync(rec.data(), ctx->d.post, sizeof(int) * rec.size(), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    for (size_t i = 0; i < ctx->seg.size(); i++) {
        ctx->seg[i].dead = rec[i * ASV_POST_WORDS + POST_DEAD];
        ctx->seg[i].neg = rec[i * ASV_POST_WORDS + POST_NEG];
        ctx->seg[i].valid = rec[i * ASV_POST_WORDS + POST_VALID];
    }
    return ASV_OK;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
// device buffers of one evaluation, stream-ordered on the context's stream
// and freed on return
struct EvalBuffers {
    asv_ctx *ctx;
    std::vector<void *> p;
    explicit EvalBuffers(asv_ctx *c) : ctx(c) {}
    ~EvalBuffers() { for (void *q : p) ctx_free(ctx, q); }
    template <typename T> cudaError_t get(T **out, size_t n)
    {
        void *q = nullptr;
        cudaError_t e = ctx_malloc(ctx, &q, std::max<size_t>(n, 1) * sizeof(T));
        if (e == cudaSuccess) { p.push_back(q); *out = (T *)q; }
        return e;
    }
};

extern "C" {

void asv_config_default(asv_config *cfg)
{
    if (!cfg) return;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->variant = ASV_VARIANT_PLAIN;
    cfg->lloyd_iters = 20;
    cfg->density_adjust = 1;
    cfg->use_graph = 1;
}

int asv_version(void) { return 100; }

const char *asv_status_string(asv_status st)
{
    switch (st) {
    case ASV_OK: return "ok";
    case ASV_ERR_BAD_ARG: return "bad argument";
    case ASV_ERR_OOM: return "out of device memory";
    case ASV_ERR_OVER_BUDGET: return "over HBM budget";
    case ASV_ERR_TIMEOUT: return "device wait timed out";
    case ASV_ERR_CUDA: return "CUDA error";
    case ASV_ERR_STATE: return "call out of order";
    case ASV_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
    }
}

asv_status asv_create(const asv_config *cfg, asv_ctx **out)
{
    if (!out) return ASV_ERR_BAD_ARG;
    *out = nullptr;
    asv_config c;
    if (cfg) c = *cfg; else asv_config_default(&c);
    if (c.lloyd_iters < 1 || c.lloyd_iters > 1000) return ASV_ERR_BAD_ARG;
    if (c.variant != ASV_VARIANT_PLAIN && c.variant != ASV_VARIANT_STREAM) return ASV_ERR_BAD_ARG;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) { cudaGetLastError(); return ASV_ERR_NO_DEVICE; }
    if (c.device < 0 || c.device >= n) return ASV_ERR_BAD_ARG;
    if (cudaSetDevice(c.device) != cudaSuccess) return ASV_ERR_CUDA;
    asv_ctx *ctx = new asv_ctx();
    ctx->cfg = c;
    if (c.stream) ctx->st = (cudaStream_t)c.stream;
    else {
        if (cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking) != cudaSuccess) { delete ctx; return ASV_ERR_CUDA; }
        ctx->own_st = true;
    }
    *out = ctx;
    return ASV_OK;
}

asv_status asv_destroy(asv_ctx *ctx)
{
    if (!ctx) return ASV_OK;
    cudaSetDevice(ctx->cfg.device);
    cudaStreamSynchronize(ctx->st);
    free_layout(ctx);
    ctx_free(ctx, ctx->cc);
    ctx_free(ctx, ctx->fl);
    cudaStreamSynchronize(ctx->st);
    for (auto e : ctx->ev) cudaEventDestroy(e);
    if (ctx->hpin) cudaFreeHost(ctx->hpin);
    for (auto e : ctx->sev) if (e) cudaEventDestroy(e);
    if (ctx->cp) {
        cudaStreamDestroy(ctx->cp);
        for (int k = 0; k < 2; k++) { cudaEventDestroy(ctx->fed_ev[k]); cudaEventDestroy(ctx->used_ev[k]); }
        cudaEventDestroy(ctx->alloc_ev);
    }
    if (ctx->own_st) cudaStreamDestroy(ctx->st);
    delete ctx;
    return ASV_OK;
}

const char *asv_last_error(const asv_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

size_t asv_clip_bytes(int W, int H, int D, int K)
{
    asv_config c;
    asv_config_default(&c);
    asv_ctx tmp;
    tmp.cfg = c;
    SegHost h;
    if (asv_prepare_segment(&tmp, W, H, D, K, &h) != ASV_OK) return 0;
    std::vector<SegHost> v(1, h);
    return asv_layout_bytes(v);
}

// the clip's RGB volume: copied as is, or (bgr) raw frames copied into the
// second label buffer (unused until the Lloyd loop) and preprocessed into
// the RGB volume on the device
static asv_status upload_clip(asv_ctx *ctx, const uint8_t *px, bool bgr)
{
    const SegDesc &s = ctx->sd[0];
    const size_t n3 = (size_t)s.nvox * 3;
    if (!bgr) {
        CK(cudaMemcpyAsync(ctx->d.rgb, px, n3, cudaMemcpyHostToDevice, ctx->st));
    } else {
        uint8_t *stage = (uint8_t *)ctx->d.labB;                       // 4 bytes / voxel >= 3
        CK(cudaMemcpyAsync(stage, px, n3, cudaMemcpyHostToDevice, ctx->st));
        asv_launch_preprocess(stage, ctx->d.rgb, s.W, s.H, s.D, ctx->st);
        CK(cudaGetLastError());
    }
    ctx->have_rgb = true;
    return ASV_OK;
}

static asv_status init_clip(asv_ctx *ctx, const uint8_t *px, int W, int H, int D, int K, bool bgr)
{
    if (!ctx) return ASV_ERR_BAD_ARG;
    if (!px) return fail(ctx, ASV_ERR_BAD_ARG, "frames pointer is NULL");
    cudaSetDevice(ctx->cfg.device);
    if (ctx->seg.size() == 1 && !ctx->allocs.empty() && !ctx->sm.on) {
        const SegHost &o = ctx->seg[0];
        if (o.W == W && o.H == H && o.D == D && o.K == K) {
            // same clip shape: keep the device layout and the captured graph
            ctx->have_flow = ctx->have_pos0 = ctx->have_M0 = ctx->have_lab = false;
            ctx->seeded = ctx->ran = false;
            return upload_clip(ctx, px, bgr);
        }
    }
    SegHost h;
    asv_status s = asv_prepare_segment(ctx, W, H, D, K, &h);
    if (s != ASV_OK) return s;
    std::vector<SegHost> v(1, h);
    if (ctx->cfg.hbm_budget && asv_layout_bytes(v) > ctx->cfg.hbm_budget)
        return fail(ctx, ASV_ERR_OVER_BUDGET, "clip exceeds the configured HBM budget");
    ctx->seg = v;
    s = asv_build_layout(ctx);
    if (s != ASV_OK) return s;
    return upload_clip(ctx, px, bgr);
}

asv_status asv_init_gpu(asv_ctx *ctx, const uint8_t *rgb, int W, int H, int D, int K)
{
    return init_clip(ctx, rgb, W, H, D, K, false);
}

asv_status asv_init_gpu_bgr(asv_ctx *ctx, const uint8_t *bgr, int W, int H, int D, int K)
{
    return init_clip(ctx, bgr, W, H, D, K, true);
}

asv_status asv_upload_flow(asv_ctx *ctx, const float *fwd, const float *bwd)
{
    if (!ctx) return ASV_ERR_BAD_ARG;
    if (ctx->seg.size() != 1) return fail(ctx, ASV_ERR_STATE, "no clip: call asv_init_gpu first");
    if (!fwd || !bwd) return fail(ctx, ASV_ERR_BAD_ARG, "flow pointer is NULL");
    size_t n = (size_t)ctx->seg[0].W * ctx->seg[0].H * ctx->seg[0].D;
    CK(cudaMemcpyAsync(ctx->d.fwd, fwd, n * 8, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(ctx->d.bwd, bwd, n * 8, cudaMemcpyHostToDevice, ctx->st));
    ctx->have_flow = true;
    return ASV_OK;
}

asv_status asv_compute_flow(asv_ctx *ctx)
{
    if (!ctx) return ASV_ERR_BAD_ARG;
    if (!ctx->have_rgb || ctx->sm.on) return fail(ctx, ASV_ERR_STATE, "no clip: call asv_init_gpu first");
    cudaSetDevice(ctx->cfg.device);
    size_t need = 0;
    for (const SegDesc &s : ctx->sd) need = std::max(need, asv_flow_scratch_bytes(s.W, s.H, s.D));
    if (ctx->fl_bytes < need) {
        if (ctx->cfg.hbm_budget && ctx->bytes + ctx->cc_bytes + need > ctx->cfg.hbm_budget)
            return fail(ctx, ASV_ERR_OVER_BUDGET, "optical-flow scratch exceeds the configured HBM budget");
        if (ctx->fl) { ctx_free(ctx, ctx->fl); ctx->fl = nullptr; ctx->fl_bytes = 0; }
        cudaError_t e = ctx_malloc(ctx, &ctx->fl, need);
        if (e != cudaSuccess) {
            cudaGetLastError();
            ctx->fl = nullptr;
            return fail(ctx, ASV_ERR_OOM, "cudaMallocAsync: optical-flow scratch");
        }
        ctx->fl_bytes = need;
    }
    for (const SegDesc &s : ctx->sd)                    // segments share the scratch, one after another
        if (asv_launch_flow(ctx->d.rgb + 3 * s.vox_off, s.W, s.H, s.D, ctx->d.fwd + s.vox_off,
                            ctx->d.bwd + s.vox_off, ctx->fl, ctx->st) != 0)
            return cuda_fail(ctx, cudaGetLastError(), "optical-flow kernels");
    CK(cudaStreamSynchronize(ctx->st));
    ctx->have_flow = true;
    return ASV_OK;
}

asv_status asv_initialization(asv_ctx *ctx)
{
    if (!ctx) return ASV_ERR_BAD_ARG;
    if (!ctx->have_rgb) return fail(ctx, ASV_ERR_STATE, "no clip: call asv_init_gpu first");
    AsvDev &d = ctx->d;
    if (ctx->cfg.density_adjust) {
        CK(cudaMemsetAsync(d.dacc, 0, sizeof(unsigned long long) * d.total_seeds, ctx->st));
        asv_launch_density(d, ctx->st);
        asv_launch_density_adjust(d, ctx->st);
        CK(cudaGetLastError());
        asv_status s = read_post(ctx);
        if (s != ASV_OK) return s;
        for (auto &h : ctx->seg)
            if (h.valid != h.Kp) return fail(ctx, ASV_ERR_CUDA, "density placement produced fewer seeds than the grid");
    } else {
        CK(cudaMemcpyAsync(d.pos0, d.grid, sizeof(float4) * d.total_seeds, cudaMemcpyDeviceToDevice, ctx->st));
    }
    ctx->have_pos0 = true;
    ctx->have_M0 = false;
    return ASV_OK;
}

asv_status asv_seed_matrix(asv_ctx *ctx)
{
    if (!ctx) return ASV_ERR_BAD_ARG;
    if (!ctx->have_pos0) return fail(ctx, ASV_ERR_STATE, "no seeds: call asv_initialization first");
    if (!ctx->have_flow) return fail(ctx, ASV_ERR_STATE, "no flow: call asv_upload_flow first");
    asv_launch_metric(ctx->d, 0, ctx->st);
    CK(cudaGetLastError());
    ctx->have_M0 = true;
    return ASV_OK;
}

asv_status asv_rgb2lab(asv_ctx *ctx)
{
    if (!ctx) return ASV_ERR_BAD_ARG;
    if (!ctx->have_rgb) return fail(ctx, ASV_ERR_STATE, "no clip: call asv_init_gpu first");
    asv_launch_rgb2lab(ctx->d, ctx->st);
    CK(cudaGetLastError());
    ctx->have_lab = true;
    return ASV_OK;
}

asv_status asv_ld_first_init(asv_ctx *ctx)
{
    if (!ctx) return ASV_ERR_BAD_ARG;
    asv_status s = check_ready(ctx);
    if (s != ASV_OK) return s;
    do_first_init(ctx);
    CK(cudaGetLastError());
    ctx->seeded = true;
    return ASV_OK;
}

asv_status asv_flood(asv_ctx *ctx, int lloyd_iter)
{
    if (!ctx) return ASV_ERR_BAD_ARG;
    (void)lloyd_iter;
    if (!ctx->seeded) return fail(ctx, ASV_ERR_STATE, "no seeds drawn: call asv_ld_first_init first");
    do_flood(ctx, -1);
    CK(cudaGetLastError());
    return ASV_OK;
}

asv_status asv_centroids_next_seeds(asv_ctx *ctx, int lloyd_iter)
{
    if (!ctx) return ASV_ERR_BAD_ARG;
    if (!ctx->seeded) return fail(ctx, ASV_ERR_STATE, "no seeds drawn: call asv_ld_first_init first");
    do_centroids(ctx, lloyd_iter != ctx->cfg.lloyd_iters);
    CK(cudaGetLastError());
    return ASV_OK;
}

asv_status asv_ld_next_seeds_matrix(asv_ctx *ctx, int lloyd_iter)
{
    if (!ctx) return ASV_ERR_BAD_ARG;
    (void)lloyd_iter;
    if (!ctx->seeded) return fail(ctx, ASV_ERR_STATE, "no seeds drawn: call asv_ld_first_init first");
    do_next_seeds(ctx);
    CK(cudaGetLastError());
    return ASV_OK;
}

asv_status asv_check_dead_seeds(asv_ctx *ctx, int32_t *labels_out)
{
    if (!ctx) return ASV_ERR_BAD_ARG;
    if (!ctx->seeded) return fail(ctx, ASV_ERR_STATE, "no labels: run the Lloyd loop first");
    do_post(ctx);
    CK(cudaGetLastError());
    ctx->ran = true;
    asv_status s = read_post(ctx);
    if (s != ASV_OK) return s;
    if (labels_out) return asv_get_labels(ctx, labels_out);
    return ASV_OK;
}

asv_status asv_run_lloyd(asv_ctx *ctx)
{
    if (!ctx) return ASV_ERR_BAD_ARG;
    asv_status s = check_ready(ctx);
    if (s != ASV_OK) return s;
    cudaSetDevice(ctx->cfg.device);
    ctx->launches = 0;
    if (ctx->cfg.instrument) {
        s = ensure_events(ctx, (size_t)2 * ctx->maxpass * ctx->cfg.lloyd_iters + 2);
        if (s != ASV_OK) return s;
        size_t tot = (size_t)2 * ctx->maxpass * ctx->cfg.lloyd_iters;
        CK(cudaEventRecord(ctx->ev[tot], ctx->st));
        enqueue_lloyd(ctx, true);
        CK(cudaEventRecord(ctx->ev[tot + 1], ctx->st));
        CK(cudaGetLastError());
        CK(cudaEventSynchronize(ctx->ev[tot + 1]));
        // every iteration draws its seeds, so its first two passes are the
        // scatters; jfa_ms / jfa_launches cover the k_jfa gather passes
        double jfa = 0.0;
        int gathers = 0;
        for (size_t k = 0; k < tot; k += 2) {
            if ((k / 2) % (size_t)ctx->maxpass < 2) continue;
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, ctx->ev[k], ctx->ev[k + 1]));
            jfa += ms;
            gathers++;
        }
        float all = 0.f;
        CK(cudaEventElapsedTime(&all, ctx->ev[tot], ctx->ev[tot + 1]));
        ctx->stats.jfa_ms = jfa;
        ctx->stats.jfa_launches = gathers;
        ctx->stats.total_ms = all;
        ctx->stats.launches = ctx->launches;
    } else if (ctx->cfg.use_graph) {
        if (!ctx->gexec) {
            cudaGraph_t g;
            CK(cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeThreadLocal));
            enqueue_lloyd(ctx, false);
            cudaError_t e = cudaStreamEndCapture(ctx->st, &g);
            if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaStreamEndCapture");
            e = cudaGraphInstantiate(&ctx->gexec, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) { ctx->gexec = nullptr; return cuda_fail(ctx, e, "cudaGraphInstantiate"); }
            ctx->stats.launches = ctx->launches;
        }
        CK(cudaGraphLaunch(ctx->gexec, ctx->st));
    } else {
        enqueue_lloyd(ctx, false);
        CK(cudaGetLastError());
        ctx->stats.launches = ctx->launches;
    }
    ctx->seeded = true;
    ctx->ran = true;
    return ASV_OK;
}

// re-tiles every segment's JFA passes to depth z (tile prefix, grid size);
// the captured graph holds the old launch shapes and is dropped
static asv_status set_zrun(asv_ctx *ctx, int z)
{
    const int nseg = (int)ctx->sd.size();
    std::vector<int> tp(nseg + 1);
    int tiles = 0;
    for (int i = 0; i < nseg; i++) {
        SegDesc &sd = ctx->sd[i];
        sd.zrun = z;
        tp[i] = tiles;
        tiles += sd.tiles_x * sd.tiles_y * ((sd.D + z - 1) / z);
    }
    tp[nseg] = tiles;
    CK(cudaMemcpyAsync((void *)ctx->d.segs, ctx->sd.data(), sizeof(SegDesc) * nseg, cudaMemcpyHostToDevice,
                       ctx->st));
    CK(cudaMemcpyAsync((void *)ctx->d.tile_prefix, tp.data(), sizeof(int) * (nseg + 1), cudaMemcpyHostToDevice,
                       ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    ctx->d.total_tiles = tiles;
    ctx->jfa_blocks = jfa_blocks_for(ctx, tiles);
    if (ctx->gexec) { cudaGraphExecDestroy(ctx->gexec); ctx->gexec = nullptr; }
    return ASV_OK;
}

asv_status asv_autotune(asv_ctx *ctx, int *zrun_out)
{
    if (!ctx) return ASV_ERR_BAD_ARG;
    if (ctx->sm.on) return fail(ctx, ASV_ERR_STATE, "autotune applies to clip and batch contexts");
    asv_status s = check_ready(ctx);
    if (s != ASV_OK) return s;
    cudaSetDevice(ctx->cfg.device);
    s = ensure_events(ctx, 2);
    if (s != ASV_OK) return s;
    int best = 0;
    float best_ms = 0.f;
    for (int z : { 4, 8, 16, 32 }) {
        if ((s = set_zrun(ctx, z)) != ASV_OK) return s;
        enqueue_lloyd(ctx, false);                        // warm-up at this depth
        CK(cudaEventRecord(ctx->ev[0], ctx->st));
        enqueue_lloyd(ctx, false);
        CK(cudaEventRecord(ctx->ev[1], ctx->st));
        CK(cudaGetLastError());
        CK(cudaEventSynchronize(ctx->ev[1]));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]));
        if (!best || ms < best_ms) { best = z; best_ms = ms; }
    }
    if ((s = set_zrun(ctx, best)) != ASV_OK) return s;
    ctx->cfg.jfa_zrun = best;                             // later layouts keep it
    enqueue_lloyd(ctx, false);                            // labels of the final depth (identical)
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(ctx->st));
    ctx->seeded = ctx->ran = true;
    if (zrun_out) *zrun_out = best;
    return ASV_OK;
}

// Connectivity enforcement: the context's scratch holds the output volume,
// an input volume (caller labels) and the union-find arrays; it is grown on
// demand and kept until the context is destroyed.
static asv_status connect_scratch(asv_ctx *ctx, long long n, int32_t **out, int32_t **in, void **cc)
{
    const size_t vol = ((size_t)n * 4 + 255) & ~(size_t)255;
    const size_t need = 2 * vol + asv_connect_scratch_bytes(n);
    if (ctx->cc_bytes < need) {
        if (ctx->cfg.hbm_budget && ctx->bytes + need > ctx->cfg.hbm_budget)
            return fail(ctx, ASV_ERR_OVER_BUDGET, "connectivity scratch exceeds the configured HBM budget");
        if (ctx->cc) { ctx_free(ctx, ctx->cc); ctx->cc = nullptr; ctx->cc_bytes = 0; }
        cudaError_t e = ctx_malloc(ctx, &ctx->cc, need);
        if (e != cudaSuccess) {
            cudaGetLastError();
            ctx->cc = nullptr;
            return fail(ctx, ASV_ERR_OOM, "cudaMallocAsync: connectivity scratch");
        }
        ctx->cc_bytes = need;
    }
    *out = (int32_t *)ctx->cc;
    *in = (int32_t *)((unsigned char *)ctx->cc + vol);
    *cc = (unsigned char *)ctx->cc + 2 * vol;
    return ASV_OK;
}

static asv_status run_connect(asv_ctx *ctx, const int32_t *lab, int32_t *out, void *cc, int W, int H, int D,
                              int supsz, int32_t *labels_out, int *label_num)
{
    const long long n = (long long)W * H * D;
    int R = 0, num = 0;
    const int rc = asv_launch_connect(lab, W, H, D, supsz, out, cc, ctx->st, &R, &num);
    if (rc == -2) return fail(ctx, ASV_ERR_TIMEOUT, "connectivity: union-find retry bound exceeded");
    if (rc == -3) return fail(ctx, ASV_ERR_BAD_ARG, "connectivity: more than 2^30 segments");
    if (rc != 0) return cuda_fail(ctx, cudaGetLastError(), "connectivity kernels");
    if (labels_out) {
        CK(cudaMemcpyAsync(labels_out, out, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
    }
    if (label_num) *label_num = num;
    return ASV_OK;
}

asv_status asv_enforce_connectivity(asv_ctx *ctx, int supsz, int32_t *labels_out, int *label_num)
{
    if (!ctx) return ASV_ERR_BAD_ARG;
    if (ctx->sm.on || ctx->seg.size() != 1) return fail(ctx, ASV_ERR_STATE, "connectivity needs a context holding one clip");
    if (!ctx->ran) return fail(ctx, ASV_ERR_STATE, "no labels: run the Lloyd loop first");
    cudaSetDevice(ctx->cfg.device);
    const SegDesc &s = ctx->sd[0];
    const SegHost &h = ctx->seg[0];
    if (supsz <= 0) supsz = (int)(s.nvox / std::max(h.K, 1));          // texel_num / seeds_num
    int32_t *out, *in;
    void *cc;
    asv_status st = connect_scratch(ctx, s.nvox, &out, &in, &cc);
    if (st != ASV_OK) return st;
    const int32_t *raw = (s.final_buf == 1 ? ctx->d.labB : ctx->d.labA) + s.vox_off;
    return run_connect(ctx, raw, out, cc, s.W, s.H, s.D, supsz, labels_out, label_num);
}

asv_status asv_enforce_connectivity_labels(asv_ctx *ctx, const int32_t *labels, int W, int H, int D,
                                           int supsz, int32_t *labels_out, int *label_num)
{
    if (!ctx) return ASV_ERR_BAD_ARG;
    if (!labels || W < 1 || H < 1 || D < 1 || supsz < 1 || (long long)W * H * D >= (1LL << 31))
        return fail(ctx, ASV_ERR_BAD_ARG, "need labels, W,H,D >= 1 with W*H*D < 2^31 and supsz >= 1");
    cudaSetDevice(ctx->cfg.device);
    const long long n = (long long)W * H * D;
    int32_t *out, *in;
    void *cc;
    asv_status st = connect_scratch(ctx, n, &out, &in, &cc);
    if (st != ASV_OK) return st;
    CK(cudaMemcpyAsync(in, labels, sizeof(int32_t) * (size_t)n, cudaMemcpyHostToDevice, ctx->st));
    return run_connect(ctx, in, out, cc, W, H, D, supsz, labels_out, label_num);
}

asv_status asv_evaluate(asv_ctx *ctx, const int32_t *labels, const int32_t *truth, int W, int H, int D,
                        asv_eval *out)
{
    if (!ctx) return ASV_ERR_BAD_ARG;
    if (!labels || !truth || !out || W < 1 || H < 1 || D < 1 || (long long)W * H * D >= (1LL << 31))
        return fail(ctx, ASV_ERR_BAD_ARG, "need labels, truth, out and W,H,D >= 1 with W*H*D < 2^31");
    cudaSetDevice(ctx->cfg.device);
    const long long n = (long long)W * H * D;
    cudaStream_t st = ctx->st;
    EvalBuffers b(ctx);
    int32_t *lab, *gt;
    int *meta;
    if (b.get(&lab, n) != cudaSuccess || b.get(&gt, n) != cudaSuccess || b.get(&meta, 4) != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, ASV_ERR_OOM, "cudaMallocAsync: evaluation buffers");
    }
    CK(cudaMemcpyAsync(lab, labels, sizeof(int32_t) * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(gt, truth, sizeof(int32_t) * n, cudaMemcpyHostToDevice, st));
    int hm[3];
    if (asv_launch_eval_range(lab, gt, n, meta, st) != 0) return cuda_fail(ctx, cudaGetLastError(), "eval range");
    CK(cudaMemcpyAsync(hm, meta, sizeof(hm), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (hm[2]) return fail(ctx, ASV_ERR_BAD_ARG, "labels must lie in [-1, 32767) and truth ids in [0, 4096)");
    const int rows = hm[0] + 2, NG = hm[1] + 1;
    unsigned *cnt;
    int *zmin, *zmax;
    uint8_t *sb;
    unsigned long long *tot;
    if (b.get(&cnt, (size_t)rows * NG) != cudaSuccess || b.get(&zmin, rows) != cudaSuccess ||
        b.get(&zmax, rows) != cudaSuccess || b.get(&sb, n) != cudaSuccess || b.get(&tot, 2) != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, ASV_ERR_OOM, "cudaMallocAsync: evaluation counts");
    }
    if (asv_launch_eval(lab, gt, W, H, D, rows, NG, cnt, zmin, zmax, sb, tot, st) != 0)
        return cuda_fail(ctx, cudaGetLastError(), "evaluation kernels");
    std::vector<unsigned> c((size_t)rows * NG);
    std::vector<int> z0(rows), z1(rows);
    unsigned long long t[2];
    CK(cudaMemcpyAsync(c.data(), cnt, sizeof(unsigned) * c.size(), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(z0.data(), zmin, sizeof(int) * rows, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(z1.data(), zmax, sizeof(int) * rows, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(t, tot, sizeof(t), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    // sizes, argmax assignment, then the measures (sums in truth-id order)
    std::vector<long long> ssz(rows, 0), gsz(NG, 0), cover(NG, 0), under(NG, 0);
    std::vector<int> arg(rows, -1);
    for (int s = 0; s < rows; s++)
        for (int g = 0; g < NG; g++) {
            const unsigned v = c[(size_t)s * NG + g];
            ssz[s] += v;
            gsz[g] += v;
            if (v && (arg[s] < 0 || v > c[(size_t)s * NG + arg[s]])) arg[s] = g;
        }
    for (int s = 0; s < rows; s++)
        for (int g = 0; g < NG; g++)
            if (c[(size_t)s * NG + g]) under[g] += ssz[s];
    for (int s = 0; s < rows; s++)
        if (arg[s] >= 0) cover[arg[s]] += c[(size_t)s * NG + arg[s]];
    double ue = 0.0, sa = 0.0;
    int ng = 0;
    for (int g = 0; g < NG; g++)
        if (gsz[g]) {
            ue += (double)(under[g] - gsz[g]) / (double)gsz[g];
            sa += (double)cover[g] / (double)gsz[g];
            ng++;
        }
    int nsv = 0;
    double dur = 0.0;
    for (int s = 0; s < rows; s++)
        if (ssz[s]) {
            nsv++;
            if (s > 0) dur += (double)(z1[s] - z0[s] + 1);   // durations of labels >= 0 only
        }
    out->undersegmentation = ng ? ue / ng : 0.0;
    out->segmentation_accuracy = ng ? sa / ng : 0.0;
    out->boundary_recall = t[0] ? (double)t[1] / (double)t[0] : 1.0;
    const int nlab = nsv - (ssz[0] ? 1 : 0);
    out->mean_duration = nlab ? dur / nlab : 0.0;
    out->supervoxels = nsv;
    out->truth_segments = ng;
    out->truth_boundary = (long long)t[0];
    out->recalled = (long long)t[1];
    return ASV_OK;
}

asv_status asv_segment_clip(asv_ctx *ctx, const uint8_t *rgb, const float *fwd, const float *bwd,
                            int W, int H, int D, int K, int32_t *labels_out)
{
    asv_status s;
    if ((s = asv_init_gpu(ctx, rgb, W, H, D, K)) != ASV_OK) return s;
    if (!fwd && !bwd) s = asv_compute_flow(ctx);             // no flow given: compute it here
    else s = asv_upload_flow(ctx, fwd, bwd);
    if (s != ASV_OK) return s;
    if ((s = asv_initialization(ctx)) != ASV_OK) return s;
    if ((s = asv_seed_matrix(ctx)) != ASV_OK) return s;
    if ((s = asv_rgb2lab(ctx)) != ASV_OK) return s;
    if ((s = asv_run_lloyd(ctx)) != ASV_OK) return s;
    if (labels_out) return asv_get_labels(ctx, labels_out);
    return asv_synchronize(ctx);
}

asv_status asv_get_info(asv_ctx *ctx, asv_info *info)
{
    if (!ctx || !info) return ASV_ERR_BAD_ARG;
    if (ctx->seg.empty()) return fail(ctx, ASV_ERR_STATE, "no clip");
    std::memset(info, 0, sizeof(*info));
    const SegHost &h = ctx->seg[0];
    if (ctx->ran) { asv_status s = read_post(ctx); if (s != ASV_OK) return s; }
    info->W = h.W; info->H = h.H; info->D = h.D; info->K = h.K; info->Kp = h.Kp; info->s = h.g.s;
    info->ratio = h.ratio; info->passes = h.npass;
    for (int p = 0; p < h.npass && p < 32; p++) info->steps[p] = h.steps[p];
    info->dead = h.dead; info->neg_count = h.neg; info->final_label_num = h.valid;
    return ASV_OK;
}

static asv_status copy_labels(asv_ctx *ctx, int32_t *out, bool raw)
{
    if (!ctx || !out) return ASV_ERR_BAD_ARG;
    if (!ctx->ran) return fail(ctx, ASV_ERR_STATE, "no labels: run the Lloyd loop first");
    const SegDesc &s = ctx->sd[0];
    const int32_t *src = ((s.final_buf == 1) == raw ? ctx->d.labB : ctx->d.labA) + s.vox_off;
    CK(cudaMemcpyAsync(out, src, sizeof(int32_t) * (size_t)s.nvox, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return ASV_OK;
}

asv_status asv_get_labels(asv_ctx *ctx, int32_t *out) { return copy_labels(ctx, out, false); }
asv_status asv_get_raw_labels(asv_ctx *ctx, int32_t *out) { return copy_labels(ctx, out, true); }

asv_status asv_get_seeds(asv_ctx *ctx, float *out)
{
    if (!ctx || !out) return ASV_ERR_BAD_ARG;
    if (ctx->seg.empty()) return fail(ctx, ASV_ERR_STATE, "no clip");
    int Kp = ctx->seg[0].Kp, off = ctx->seg[0].seed_off;
    std::vector<float4> p(Kp), c(Kp);
    std::vector<float> m((size_t)Kp * 8);
    bool work = ctx->seeded;
    CK(cudaMemcpyAsync(p.data(), (work ? ctx->d.pos : ctx->d.pos0) + off, sizeof(float4) * Kp, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(c.data(), ctx->d.slab + off, sizeof(float4) * Kp, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(m.data(), (work ? ctx->d.M : ctx->d.M0) + 8 * (size_t)off, sizeof(float) * 8 * Kp, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    for (int i = 0; i < Kp; i++) {
        float *o = out + 12 * (size_t)i;
        o[0] = p[i].x; o[1] = p[i].y; o[2] = p[i].z;
        o[3] = c[i].x; o[4] = c[i].y; o[5] = c[i].z;
        for (int e = 0; e < 6; e++) o[6 + e] = m[8 * (size_t)i + e];
    }
    return ASV_OK;
}

asv_status asv_set_seeds(asv_ctx *ctx, const float *in, int Kp)
{
    if (!ctx || !in) return ASV_ERR_BAD_ARG;
    if (ctx->seg.size() != 1) return fail(ctx, ASV_ERR_STATE, "no clip");
    if (Kp != ctx->seg[0].Kp) return fail(ctx, ASV_ERR_BAD_ARG, "seed count differs from the clip's");
    int off = ctx->seg[0].seed_off;
    std::vector<float4> p(Kp), c(Kp);
    std::vector<float> m((size_t)Kp * 8, 0.f);
    const SegHost &h = ctx->seg[0];
    for (int i = 0; i < Kp; i++) {
        const float *o = in + 12 * (size_t)i;
        if (!(o[0] >= 0.f && o[0] < (float)h.W && o[1] >= 0.f && o[1] < (float)h.H && o[2] >= 0.f &&
              o[2] < (float)h.D))
            return fail(ctx, ASV_ERR_BAD_ARG, "seed position outside the volume");
        p[i] = make_float4(o[0], o[1], o[2], (float)i);
        c[i] = make_float4(o[3], o[4], o[5], 0.f);
        for (int e = 0; e < 6; e++) m[8 * (size_t)i + e] = o[6 + e];
    }
    CK(cudaMemcpyAsync(ctx->d.pos + off, p.data(), sizeof(float4) * Kp, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(ctx->d.slab + off, c.data(), sizeof(float4) * Kp, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(ctx->d.M + 8 * (size_t)off, m.data(), sizeof(float) * 8 * Kp, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemsetAsync(ctx->d.mkey + off, 0xff, sizeof(int) * Kp, ctx->st));   // drop the reseed memo
    asv_launch_draw(ctx->d, ctx->st);   // packs the JFA table (the label write is ignored here)
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(ctx->st));
    ctx->seeded = true;
    return ASV_OK;
}

asv_status asv_get_lab(asv_ctx *ctx, uint8_t *out)
{
    if (!ctx || !out) return ASV_ERR_BAD_ARG;
    if (!ctx->have_lab) return fail(ctx, ASV_ERR_STATE, "no LAB volume: call asv_rgb2lab first");
    const SegDesc &s = ctx->sd[0];
    CK(cudaMemcpyAsync(out, ctx->d.lab + s.vox_off, 4 * (size_t)s.nvox, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return ASV_OK;
}

asv_status asv_get_flow(asv_ctx *ctx, float *fwd, float *bwd)
{
    if (!ctx || !fwd || !bwd) return ASV_ERR_BAD_ARG;
    if (!ctx->have_flow || ctx->sd.empty()) return fail(ctx, ASV_ERR_STATE, "no flow on the device");
    const SegDesc &s = ctx->sd[0];
    CK(cudaMemcpyAsync(fwd, ctx->d.fwd + s.vox_off, 8 * (size_t)s.nvox, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(bwd, ctx->d.bwd + s.vox_off, 8 * (size_t)s.nvox, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return ASV_OK;
}

asv_status asv_get_sums(asv_ctx *ctx, int64_t *out)
{
    if (!ctx || !out) return ASV_ERR_BAD_ARG;
    if (ctx->seg.empty()) return fail(ctx, ASV_ERR_STATE, "no clip");
    int Kp = ctx->seg[0].Kp, off = ctx->seg[0].seed_off;
    std::vector<unsigned long long> s((size_t)(Kp + 1) * 8);
    CK(cudaMemcpyAsync(s.data(), ctx->d.sums + 8 * (size_t)off, sizeof(unsigned long long) * s.size(), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    for (int i = 0; i <= Kp; i++)
        for (int k = 0; k < 7; k++) out[7 * (size_t)i + k] = (int64_t)s[8 * (size_t)i + k];
    return ASV_OK;
}

asv_status asv_check_dead_seeds_host(asv_ctx *ctx, const int32_t *raw_in, int32_t *out)
{
    if (!ctx || !raw_in || !out) return ASV_ERR_BAD_ARG;
    if (ctx->seg.size() != 1 || !ctx->have_lab)
        return fail(ctx, ASV_ERR_STATE, "need a clip and its LAB volume");
    const SegDesc &s = ctx->sd[0];
    for (long long v = 0; v < s.nvox; v++)
        if (raw_in[v] < -1 || raw_in[v] >= s.Kp) return fail(ctx, ASV_ERR_BAD_ARG, "label outside [-1, Kp)");
    int32_t *fin = (s.final_buf ? ctx->d.labB : ctx->d.labA) + s.vox_off;
    CK(cudaMemcpyAsync(fin, raw_in, 4 * (size_t)s.nvox, cudaMemcpyHostToDevice, ctx->st));
    do_sums_from_labels(ctx);
    do_post(ctx);
    CK(cudaGetLastError());
    ctx->ran = true;
    asv_status st = read_post(ctx);
    if (st != ASV_OK) return st;
    return asv_get_labels(ctx, out);
}

asv_status asv_jfa_pass_host(asv_ctx *ctx, int step, float ratio, const int32_t *in, int32_t *out)
{
    if (!ctx || !in || !out || step < 1) return ASV_ERR_BAD_ARG;
    if (ctx->seg.size() != 1 || !ctx->have_lab || !ctx->seeded)
        return fail(ctx, ASV_ERR_STATE, "need a clip, its LAB volume and a seed table");
    const SegDesc &s = ctx->sd[0];
    size_t n = (size_t)s.nvox;
    int32_t *din = ctx->d.labA + s.vox_off, *dout = ctx->d.labB + s.vox_off;
    CK(cudaMemcpyAsync(din, in, 4 * n, cudaMemcpyHostToDevice, ctx->st));
    asv_launch_jfa_single(ctx->d, din, dout, step, ratio, ctx->st);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, dout, 4 * n, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return ASV_OK;
}

asv_status asv_get_stats(asv_ctx *ctx, asv_stats *st)
{
    if (!ctx || !st) return ASV_ERR_BAD_ARG;
    *st = ctx->stats;
    return ASV_OK;
}

asv_status asv_get_stream(asv_ctx *ctx, void **stream)
{
    if (!ctx || !stream) return ASV_ERR_BAD_ARG;
    *stream = (void *)ctx->st;
    return ASV_OK;
}

asv_status asv_synchronize(asv_ctx *ctx)
{
    if (!ctx) return ASV_ERR_BAD_ARG;
    CK(cudaStreamSynchronize(ctx->st));
    CK(cudaGetLastError());
    return ASV_OK;
}

// ---------------------------------------------------------------------------
// Batched form: many clips, one launch per stage
// ---------------------------------------------------------------------------
static asv_status batch_segments(asv_ctx *ctx, int n, const int *W, const int *H, const int *D,
                                 const int *K, std::vector<SegHost> *v)
{
    if (n < 1 || n > 4096 || !W || !H || !D || !K) return fail(ctx, ASV_ERR_BAD_ARG, "bad batch description");
    v->clear();
    for (int i = 0; i < n; i++) {
        SegHost h;
        asv_status s = asv_prepare_segment(ctx, W[i], H[i], D[i], K[i], &h);
        if (s != ASV_OK) return s;
        v->push_back(h);
    }
    return ASV_OK;
}

size_t asv_batch_bytes(int n, const int *W, const int *H, const int *D, const int *K)
{
    asv_ctx tmp;
    asv_config_default(&tmp.cfg);
    std::vector<SegHost> v;
    if (batch_segments(&tmp, n, W, H, D, K, &v) != ASV_OK) return 0;
    return asv_layout_bytes(v);
}

asv_status asv_batch_init(asv_ctx *ctx, int n, const int *W, const int *H, const int *D, const int *K)
{
    if (!ctx) return ASV_ERR_BAD_ARG;
    cudaSetDevice(ctx->cfg.device);
    std::vector<SegHost> v;
    asv_status s = batch_segments(ctx, n, W, H, D, K, &v);
    if (s != ASV_OK) return s;
    if (ctx->cfg.hbm_budget && asv_layout_bytes(v) > ctx->cfg.hbm_budget)
        return fail(ctx, ASV_ERR_OVER_BUDGET, "batch exceeds the configured HBM budget");
    ctx->seg = v;
    s = asv_build_layout(ctx);
    if (s != ASV_OK) return s;
    ctx->up_rgb.assign(n, 0);
    ctx->up_flow.assign(n, 0);
    return ASV_OK;
}

asv_status asv_batch_upload(asv_ctx *ctx, int clip, const uint8_t *rgb, const float *fwd, const float *bwd)
{
    if (!ctx) return ASV_ERR_BAD_ARG;
    if (clip < 0 || clip >= (int)ctx->seg.size() || ctx->up_rgb.size() != ctx->seg.size())
        return fail(ctx, ASV_ERR_BAD_ARG, "no such clip in the batch");
    if (!rgb || !fwd || !bwd) return fail(ctx, ASV_ERR_BAD_ARG, "NULL buffer");
    const SegDesc &s = ctx->sd[clip];
    size_t n = (size_t)s.nvox;
    CK(cudaMemcpyAsync(ctx->d.rgb + 3 * s.vox_off, rgb, 3 * n, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(ctx->d.fwd + s.vox_off, fwd, 8 * n, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(ctx->d.bwd + s.vox_off, bwd, 8 * n, cudaMemcpyHostToDevice, ctx->st));
    ctx->up_rgb[clip] = ctx->up_flow[clip] = 1;
    bool all = true;
    for (auto u : ctx->up_rgb) all = all && u;
    ctx->have_rgb = ctx->have_flow = all;
    return ASV_OK;
}

asv_status asv_batch_get_labels(asv_ctx *ctx, int clip, int32_t *out)
{
    if (!ctx || !out) return ASV_ERR_BAD_ARG;
    if (clip < 0 || clip >= (int)ctx->seg.size()) return fail(ctx, ASV_ERR_BAD_ARG, "no such clip");
    if (!ctx->ran) return fail(ctx, ASV_ERR_STATE, "no labels: run the Lloyd loop first");
    const SegDesc &s = ctx->sd[clip];
    const int32_t *src = (s.final_buf ? ctx->d.labA : ctx->d.labB) + s.vox_off;
    CK(cudaMemcpyAsync(out, src, sizeof(int32_t) * (size_t)s.nvox, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return ASV_OK;
}

asv_status asv_batch_get_info(asv_ctx *ctx, int clip, asv_info *info)
{
    if (!ctx || !info) return ASV_ERR_BAD_ARG;
    if (clip < 0 || clip >= (int)ctx->seg.size()) return fail(ctx, ASV_ERR_BAD_ARG, "no such clip");
    if (ctx->ran) { asv_status s = read_post(ctx); if (s != ASV_OK) return s; }
    std::memset(info, 0, sizeof(*info));
    const SegHost &h = ctx->seg[clip];
    info->W = h.W; info->H = h.H; info->D = h.D; info->K = h.K; info->Kp = h.Kp; info->s = h.g.s;
    info->ratio = h.ratio; info->passes = h.npass;
    for (int p = 0; p < h.npass && p < 32; p++) info->steps[p] = h.steps[p];
    info->dead = h.dead; info->neg_count = h.neg; info->final_label_num = h.valid;
    return ASV_OK;
}

// ---------------------------------------------------------------------------
// Streaming form (streamGPU-AS/Render.cpp:100-569)
// ---------------------------------------------------------------------------

// block intervals (Render.cpp:199-241)
static int stream_blocks(int D_all, int bs, std::vector<int> *iv)
{
    int one_third = bs / 3, two_third = 2 * bs / 3;
    int last_end = bs;
    bool done = false;
    iv->clear();
    if (D_all < bs + one_third) {
        iv->push_back(0); iv->push_back(D_all);
    } else {
        iv->push_back(0); iv->push_back(last_end);
        while (last_end + two_third < D_all) {
            if (D_all - last_end - two_third < one_third) {
                iv->push_back(last_end - one_third); iv->push_back(D_all);
                done = true;
            } else {
                iv->push_back(last_end - one_third); iv->push_back(last_end + two_third);
            }
            last_end += two_third;
        }
        if (!done) { iv->push_back(last_end - one_third); iv->push_back(D_all); }
    }
    return (int)iv->size() / 2;
}

// new seeds requested for block b (Render.cpp:351-356, :394)
static int stream_seeds_num(const asv_ctx *ctx, int b)
{
    const auto &m = ctx->sm;
    int Db = m.iv[2 * b + 1] - m.iv[2 * b];
    if (b == 0) return m.nb > 1 ? m.seeds100 * (Db - 10) / 100 : m.seeds100 * Db / 100;
    return m.seeds100 * (Db - 10) / 100;
}

// frames block b takes from the caller: all of the first block's, then the
// block's frames after the overlap kept on the device
static int stream_new_frames(const asv_ctx::Stream &m, int b)
{
    return m.iv[2 * b + 1] - m.iv[2 * b] - (b == 0 ? 0 : 10);
}

asv_status asv_stream_begin(asv_ctx *ctx, int W, int H, int D_all, int K_video, int seeds_num_100,
                            int block_size)
{
    if (!ctx) return ASV_ERR_BAD_ARG;
    if (block_size <= 0) block_size = 30;
    if (W < 1 || H < 1 || D_all < 2 || block_size < 6 || (K_video < 1 && seeds_num_100 < 1))
        return fail(ctx, ASV_ERR_BAD_ARG, "need W,H >= 1, D_all >= 2, block_size >= 6 and seeds");
    cudaSetDevice(ctx->cfg.device);
    if (ctx->sm.nflight) cudaStreamSynchronize(ctx->st);   // blocks in flight finish their copies first
    free_layout(ctx);
    ctx->cfg.variant = ASV_VARIANT_STREAM;          // compactness 6, no angle filter
    auto &m = ctx->sm;
    m = asv_ctx::Stream{};
    m.W = W; m.H = H; m.D_all = D_all; m.bs = block_size;
    m.seeds100 = seeds_num_100 > 0 ? seeds_num_100 : K_video * 100 / D_all;   // Render.cpp:157
    m.nb = stream_blocks(D_all, block_size, &m.iv);
    int kn_max = 0, wmax = 1, hmax = 1, dmax = 1;
    for (int b = 0; b < m.nb; b++) {
        int Db = m.iv[2 * b + 1] - m.iv[2 * b];
        if (Db < 2) return fail(ctx, ASV_ERR_BAD_ARG, "a block shorter than 2 frames");
        SegHost h;
        asv_status s = asv_prepare_segment(ctx, W, H, Db, stream_seeds_num(ctx, b), &h);
        if (s != ASV_OK) return s;
        kn_max = std::max(kn_max, h.Kp);
        wmax = std::max(wmax, h.g.wNum); hmax = std::max(hmax, h.g.hNum); dmax = std::max(dmax, h.g.dNum);
        m.Dcap = std::max(m.Dcap, Db);
    }
    m.Kcap = std::min(3 * kn_max + 256, 32767);
    SegHost cap;
    cap.W = W; cap.H = H; cap.D = m.Dcap; cap.Kp = m.Kcap; cap.npass = 1;
    cap.g.wNum = wmax; cap.g.hNum = hmax; cap.g.dNum = dmax; cap.g.Kp = m.Kcap;
    cap.cells.assign((size_t)W + H + m.Dcap + 2 * wmax, -1);
    {                                              // the pinned host staging of every block's small copies
        size_t off = 0;
        auto take = [&](size_t b) { const size_t o = off; off += (b + 255) & ~(size_t)255; return o; };
        size_t o_pref[2], o_sda[2], o_ctr[2], o_ctr2[2], o_cells[2], o_grid[2];
        for (int q = 0; q < 2; q++) {
            o_pref[q] = take(6 * sizeof(int));
            o_sda[q] = take(sizeof(SegDesc));
            o_ctr[q] = take(sizeof(int) * STREAM_CTR_WORDS);
            o_ctr2[q] = take(sizeof(int) * STREAM_CTR_WORDS);
            o_cells[q] = take(sizeof(int) * cap.cells.size());
            o_grid[q] = take(sizeof(float4) * (size_t)m.Kcap);
        }
        if (ctx->hpin_bytes < off) {
            if (ctx->hpin) {
                cudaStreamSynchronize(ctx->st);
                cudaFreeHost(ctx->hpin);
                ctx->hpin = nullptr;
                ctx->hpin_bytes = 0;
            }
            if (cudaHostAlloc(&ctx->hpin, off, cudaHostAllocDefault) != cudaSuccess) {
                cudaGetLastError();
                ctx->hpin = nullptr;
                return fail(ctx, ASV_ERR_OOM, "cudaHostAlloc: stream staging");
            }
            ctx->hpin_bytes = off;
        }
        char *hb = (char *)ctx->hpin;
        for (int q = 0; q < 2; q++) {
            m.h_pref[q] = (int *)(hb + o_pref[q]);
            m.h_sdA[q] = (SegDesc *)(hb + o_sda[q]);
            m.h_ctr[q] = (int *)(hb + o_ctr[q]);
            m.h_ctr2[q] = (int *)(hb + o_ctr2[q]);
            m.h_cells[q] = (int *)(hb + o_cells[q]);
            m.h_grid[q] = (float4 *)(hb + o_grid[q]);
        }
        m.h_cells_cap = cap.cells.size();
        for (auto &e : ctx->sev)
            if (!e && cudaEventCreate(&e) != cudaSuccess) {
                cudaGetLastError();
                e = nullptr;
                return fail(ctx, ASV_ERR_CUDA, "cudaEventCreate: stream events");
            }
    }
    cap.grid.assign((size_t)4 * m.Kcap, 0.f);
    ctx->seg.assign(1, cap);
    asv_status s = asv_build_layout(ctx);
    if (s != ASV_OK) return s;
    StreamDev &sd = m.s;
    AL(sd.kept_pos, m.Kcap); AL(sd.kept_next, m.Kcap);
    AL(sd.gmap_prev, m.Kcap); AL(sd.gmap_cur, m.Kcap);
    AL(sd.ctr, STREAM_CTR_WORDS);
    AL(sd.lab_out, (size_t)W * H * m.Dcap);
    CK(cudaMemsetAsync(sd.ctr, 0, sizeof(int) * STREAM_CTR_WORDS, ctx->st));
    m.on = true;
    return ASV_OK;
}

asv_status asv_stream_info_get(asv_ctx *ctx, asv_stream_info *info)
{
    if (!ctx || !info) return ASV_ERR_BAD_ARG;
    const auto &m = ctx->sm;
    if (!m.on) return fail(ctx, ASV_ERR_STATE, "no stream: call asv_stream_begin first");
    std::memset(info, 0, sizeof(*info));
    info->blocks = m.nb;
    info->next_block = m.next;
    info->seeds_placed = m.placed;
    info->block_Kp = m.last_Kp;
    if (m.next < m.nb) {
        info->block_start = m.iv[2 * m.next];
        info->block_end = m.iv[2 * m.next + 1];
        info->frames_needed = stream_new_frames(m, m.next);
    }
    return ASV_OK;
}

asv_status asv_stream_block(asv_ctx *ctx, int b, int *block_start, int *block_end, int *frames_needed)
{
    if (!ctx) return ASV_ERR_BAD_ARG;
    const auto &m = ctx->sm;
    if (!m.on) return fail(ctx, ASV_ERR_STATE, "no stream: call asv_stream_begin first");
    if (b < 0 || b >= m.nb) return fail(ctx, ASV_ERR_BAD_ARG, "no such block");
    if (block_start) *block_start = m.iv[2 * b];
    if (block_end) *block_end = m.iv[2 * b + 1];
    if (frames_needed) *frames_needed = stream_new_frames(m, b);
    return ASV_OK;
}

static asv_status stream_feed(asv_ctx *ctx, bool bgr, const uint8_t *rgb, const float *fwd, const float *bwd)
{
    if (!ctx) return ASV_ERR_BAD_ARG;
    auto &m = ctx->sm;
    if (!m.on) return fail(ctx, ASV_ERR_STATE, "no stream: call asv_stream_begin first");
    m.fed_next = std::max(m.fed_next, m.next);
    if (m.fed_next >= m.nb) return fail(ctx, ASV_ERR_STATE, "every block of the video is fed");
    if (m.fed_next > m.next + 1) return fail(ctx, ASV_ERR_STATE, "two blocks are fed ahead: push one first");
    if (!rgb || (!fwd) != (!bwd)) return fail(ctx, ASV_ERR_BAD_ARG, "NULL buffer");
    cudaSetDevice(ctx->cfg.device);
    if (!ctx->cp) {
        CK(cudaStreamCreateWithFlags(&ctx->cp, cudaStreamNonBlocking));
        for (int k = 0; k < 2; k++) {
            CK(cudaEventCreateWithFlags(&ctx->fed_ev[k], cudaEventDisableTiming));
            CK(cudaEventCreateWithFlags(&ctx->used_ev[k], cudaEventDisableTiming));
        }
        CK(cudaEventCreateWithFlags(&ctx->alloc_ev, cudaEventDisableTiming));
    }
    const int b = m.fed_next, slot = b & 1;
    const size_t WH = (size_t)m.W * m.H, n = (size_t)stream_new_frames(m, b) * WH;
    {                                               // both slots' staging, stream-ordered on the context
        const size_t cap = (size_t)m.Dcap * WH;     // (each buffer set only once allocated, so a failed
        bool fresh = false;                         //  allocation leaves nothing half made for a retry)
        for (int k = 0; k < 2; k++) {
            asv_status s;
            if (!m.stg_rgb[k]) { if ((s = dalloc(ctx, &m.stg_rgb[k], 3 * cap)) != ASV_OK) return s; fresh = true; }
            if (!m.stg_fwd[k]) { if ((s = dalloc(ctx, &m.stg_fwd[k], 2 * cap)) != ASV_OK) return s; fresh = true; }
            if (!m.stg_bwd[k]) { if ((s = dalloc(ctx, &m.stg_bwd[k], 2 * cap)) != ASV_OK) return s; fresh = true; }
        }
        if (fresh) {
            CK(cudaEventRecord(ctx->alloc_ev, ctx->st));
            CK(cudaStreamWaitEvent(ctx->cp, ctx->alloc_ev, 0));
        }
    }
    CK(cudaStreamWaitEvent(ctx->cp, ctx->used_ev[slot], 0));   // block b-2's push has read the slot
    CK(cudaMemcpyAsync(m.stg_rgb[slot], rgb, 3 * n, cudaMemcpyHostToDevice, ctx->cp));
    if (fwd) {
        CK(cudaMemcpyAsync(m.stg_fwd[slot], fwd, 8 * n, cudaMemcpyHostToDevice, ctx->cp));
        CK(cudaMemcpyAsync(m.stg_bwd[slot], bwd, 8 * n, cudaMemcpyHostToDevice, ctx->cp));
    }
    CK(cudaEventRecord(ctx->fed_ev[slot], ctx->cp));
    m.fed_n[slot] = stream_new_frames(m, b);
    m.fed_devflow[slot] = !fwd;
    m.fed_bgr[slot] = bgr;
    m.fed_next = b + 1;
    return ASV_OK;
}

asv_status asv_stream_feed(asv_ctx *ctx, const uint8_t *rgb, const float *fwd, const float *bwd)
{
    return stream_feed(ctx, false, rgb, fwd, bwd);
}

asv_status asv_stream_feed_bgr(asv_ctx *ctx, const uint8_t *bgr, const float *fwd, const float *bwd)
{
    return stream_feed(ctx, true, bgr, fwd, bwd);
}

// Enqueues the next block on the context's stream: new frames from the
// caller (asv_stream_push) or fed ahead into a staging slot
// (asv_stream_push_fed); stream_finish waits for it.  Everything the block
// reads back goes to the pinned set of its parity, so two blocks can be in
// flight.
static asv_status stream_enqueue(asv_ctx *ctx, bool fed, const uint8_t *rgb, const float *fwd, const float *bwd,
                                 int32_t *labels_out)
{
    if (!ctx) return ASV_ERR_BAD_ARG;
    auto &m = ctx->sm;
    if (!m.on) return fail(ctx, ASV_ERR_STATE, "no stream: call asv_stream_begin first");
    if (m.failed) return fail(ctx, ASV_ERR_STATE, "a block of the stream was refused");
    if (m.next >= m.nb) return fail(ctx, ASV_ERR_STATE, "the stream is finished");
    if (m.nflight >= 2) return fail(ctx, ASV_ERR_STATE, "two blocks in flight: asv_stream_wait first");
    if (fed && m.fed_next <= m.next) return fail(ctx, ASV_ERR_STATE, "the block was not fed: asv_stream_feed first");
    if (!fed && m.fed_next > m.next) return fail(ctx, ASV_ERR_STATE, "the block was fed: use asv_stream_push_fed");
    if (!labels_out || (!fed && (!rgb || (!fwd) != (!bwd)))) return fail(ctx, ASV_ERR_BAD_ARG, "NULL buffer");
    const int slot = m.next & 1, par = slot;                        // staging slot and pinned set
    const bool device_flow = fed ? m.fed_devflow[slot] : !fwd;     // no flow given: computed here
    cudaSetDevice(ctx->cfg.device);
    const int b = m.next;
    const int Db = m.iv[2 * b + 1] - m.iv[2 * b];
    const int one_third = m.bs / 3, two_third = m.bs - one_third;   // Render.cpp:515-516
    const int z0 = b == 0 ? 0 : 10;                                 // overlap frames kept on the device
    const size_t WH = (size_t)m.W * m.H;
    AsvDev &d = ctx->d;
    cudaStream_t st = ctx->st;
    if (b > 0) {                                                    // Render.cpp:405-412, :545-556
        size_t src = (size_t)(m.prev_Db - 10) * WH, n = 10 * WH;
        CK(asv_copy_d2d(d.rgb, d.rgb + 3 * src, 3 * n, st));
        CK(asv_copy_d2d(d.lab, d.lab + src, 4 * n, st));
        CK(asv_copy_d2d(d.fwd, d.fwd + src, 8 * n, st));
        CK(asv_copy_d2d(d.bwd, d.bwd + src, 8 * n, st));
    }
    const size_t nnew = (size_t)(Db - z0) * WH;
    if (fed) {                                                      // uploaded during the previous block
        if (m.fed_n[slot] != Db - z0) return fail(ctx, ASV_ERR_STATE, "the fed frames do not match the block");
        CK(cudaStreamWaitEvent(st, ctx->fed_ev[slot], 0));
        if (m.fed_bgr[slot]) {                                      // cvMat2TexureInput per frame
            asv_launch_preprocess(m.stg_rgb[slot], d.rgb + 3 * z0 * WH, m.W, m.H, Db - z0, st);
            CK(cudaGetLastError());
        } else {
            CK(asv_copy_d2d(d.rgb + 3 * z0 * WH, m.stg_rgb[slot], 3 * nnew, st));
        }
        if (!device_flow) {
            CK(asv_copy_d2d(d.fwd + z0 * WH, m.stg_fwd[slot], 8 * nnew, st));
            CK(asv_copy_d2d(d.bwd + z0 * WH, m.stg_bwd[slot], 8 * nnew, st));
        }
        CK(cudaEventRecord(ctx->used_ev[slot], st));
    } else {
        CK(cudaMemcpyAsync(d.rgb + 3 * z0 * WH, rgb, 3 * nnew, cudaMemcpyHostToDevice, st));
        if (!device_flow) {
            CK(cudaMemcpyAsync(d.fwd + z0 * WH, fwd, 8 * nnew, cudaMemcpyHostToDevice, st));
            CK(cudaMemcpyAsync(d.bwd + z0 * WH, bwd, 8 * nnew, cudaMemcpyHostToDevice, st));
        }
    }
    cudaEvent_t ev_start = ctx->sev[3 * par], ev_end = ctx->sev[3 * par + 1], ev_read = ctx->sev[3 * par + 2];
    if (device_flow) {
        CK(cudaEventRecord(ev_start, st));
        // the block's flow from its own frames, as the streaming program does
        // per block.  Pairs within the overlap frames were computed by the
        // previous block (same two frames, same flow) and came along with the
        // shift; the pairs touching a new frame are computed here: frames
        // z0-1 .. Db-1, keeping the backward flow of frame z0-1.  The last
        // frame's forward flow is not read by the metric.
        const int zf = z0 > 0 ? z0 - 1 : 0;
        const size_t need = asv_flow_scratch_bytes(m.W, m.H, Db - zf);
        if (ctx->fl_bytes < need) {
            if (ctx->fl) { ctx_free(ctx, ctx->fl); ctx->fl = nullptr; ctx->fl_bytes = 0; }
            cudaError_t e = ctx_malloc(ctx, &ctx->fl, need);
            if (e != cudaSuccess) {
                cudaGetLastError();
                ctx->fl = nullptr;
                return fail(ctx, ASV_ERR_OOM, "cudaMallocAsync: optical-flow scratch");
            }
            ctx->fl_bytes = need;
        }
        if (asv_launch_flow(d.rgb + 3 * zf * WH, m.W, m.H, Db - zf, d.fwd + zf * WH, d.bwd + zf * WH, ctx->fl,
                            st, zf > 0) != 0)
            return cuda_fail(ctx, cudaGetLastError(), "optical-flow kernels");
    }

    // new seeds of the block: grid + density placement (Render.cpp:376-379, :429-432)
    SegHost h;
    asv_status s = asv_prepare_segment(ctx, m.W, m.H, Db, stream_seeds_num(ctx, b), &h);
    if (s != ASV_OK) return s;
    const int Kn = h.Kp;
    SegDesc &sd = ctx->sd[0];
    const int seed_cap = d.total_seeds;
    sd.W = m.W; sd.H = m.H; sd.D = Db; sd.Kp = Kn;
    sd.vox_off = 0; sd.nvox = (long long)WH * Db; sd.seed_off = 0;
    sd.npass = h.npass;
    for (int p = 0; p < h.npass; p++) { sd.steps[p] = h.steps[p]; sd.ratio[p] = h.rmul[p] * h.ratio; }
    sd.tiles_x = (m.W + ASV_TILE_X - 1) / ASV_TILE_X;
    sd.tiles_y = (m.H + ASV_TILE_Y - 1) / ASV_TILE_Y;
    sd.zrun = pick_zrun(ctx, std::vector<SegHost>(1, h));
    sd.angle_filter = 0;
    sd.wNum = h.g.wNum; sd.hNum = h.g.hNum; sd.dNum = h.g.dNum;
    sd.cell_off = 0;
    sd.final_buf = h.npass & 1;
    sd.lab_from = (long long)z0 * WH;
    const int tiles = sd.tiles_x * sd.tiles_y * ((Db + sd.zrun - 1) / sd.zrun);
    const int chunks = (int)((sd.nvox + ASV_CHUNK - 1) / ASV_CHUNK);
    d.total_tiles = tiles;
    d.total_chunks = chunks;
    // (the pinned set of this parity is free again: its previous block was finished)
    if (h.cells.size() > m.h_cells_cap || Kn > m.Kcap) return fail(ctx, ASV_ERR_STATE, "block larger than its layout");
    int *pref = m.h_pref[par];
    pref[0] = 0; pref[1] = tiles; pref[2] = 0; pref[3] = chunks; pref[4] = 0; pref[5] = seed_cap;
    CK(cudaMemcpyAsync((void *)d.tile_prefix, pref, 2 * sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync((void *)d.chunk_prefix, pref + 2, 2 * sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync((void *)d.seed_prefix, pref + 4, 2 * sizeof(int), cudaMemcpyHostToDevice, st));
    *m.h_sdA[par] = sd;
    CK(cudaMemcpyAsync((void *)d.segs, m.h_sdA[par], sizeof(SegDesc), cudaMemcpyHostToDevice, st));
    std::memcpy(m.h_cells[par], h.cells.data(), sizeof(int) * h.cells.size());
    CK(cudaMemcpyAsync(d.cells, m.h_cells[par], sizeof(int) * h.cells.size(), cudaMemcpyHostToDevice, st));
    float4 *grid4 = m.h_grid[par];
    for (int k = 0; k < Kn; k++)
        grid4[k] = make_float4(h.grid[4 * k], h.grid[4 * k + 1], h.grid[4 * k + 2], h.grid[4 * k + 3]);
    CK(cudaMemcpyAsync(d.grid, grid4, sizeof(float4) * Kn, cudaMemcpyHostToDevice, st));
    ctx->maxpass = h.npass;
    ctx->jfa_blocks = jfa_blocks_for(ctx, tiles);

    // device time of the window's compute: from here (its frames are on the
    // device; before the flow kernels when the flow is computed here) to the
    // labels mapped, before they are read back
    if (!device_flow) CK(cudaEventRecord(ev_start, st));
    asv_launch_rgb2lab(d, st);                                   // new frames only (lab_from)
    CK(cudaMemsetAsync(d.dacc, 0, sizeof(unsigned long long) * d.total_seeds, st));
    asv_launch_density(d, st);
    asv_launch_density_adjust(d, st);
    asv_launch_stream_compose(d, m.s, Kn, m.Kcap, st);          // kept seeds first, then the new ones
    CK(cudaGetLastError());
    // the composed seed count went to the segment descriptor on the device
    // (k_stream_compose), so the rest of the block is enqueued without a
    // host round trip; the counters of this point are read at the end
    CK(cudaMemcpyAsync(m.h_ctr[par], m.s.ctr, sizeof(int) * STREAM_CTR_WORDS, cudaMemcpyDeviceToHost, st));
    ctx->seg[0] = h;
    ctx->seg[0].vox_off = 0;
    ctx->seg[0].seed_off = 0;

    // seed_matrix, RGB2LAB (above), Lloyd loop, check_dead_seeds (Render.cpp:470-512)
    ctx->launches = 4;                                           // LAB, density (2), seed composition
    asv_launch_metric(d, 0, st);
    ctx->launches += 5;
    if (ctx->cfg.use_graph && !ctx->cfg.instrument) {
        const bool same = ctx->sgexec && std::memcmp(&ctx->skey, &d, sizeof(AsvDev)) == 0 &&
                          ctx->skey_blocks == ctx->jfa_blocks && ctx->skey_passes == ctx->maxpass &&
                          ctx->skey_iters == ctx->cfg.lloyd_iters;
        if (!same) {
            if (ctx->sgexec) { cudaGraphExecDestroy(ctx->sgexec); ctx->sgexec = nullptr; }
            const int before = ctx->launches;
            cudaGraph_t g;
            CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            enqueue_lloyd(ctx, false);
            cudaError_t e = cudaStreamEndCapture(st, &g);
            if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaStreamEndCapture");
            e = cudaGraphInstantiate(&ctx->sgexec, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) { ctx->sgexec = nullptr; return cuda_fail(ctx, e, "cudaGraphInstantiate"); }
            std::memcpy(&ctx->skey, &d, sizeof(AsvDev));
            ctx->skey_blocks = ctx->jfa_blocks;
            ctx->skey_passes = ctx->maxpass;
            ctx->skey_iters = ctx->cfg.lloyd_iters;
            ctx->sg_launches = ctx->launches - before;
        } else {
            ctx->launches += ctx->sg_launches;
        }
        CK(cudaGraphLaunch(ctx->sgexec, st));
    } else {
        enqueue_lloyd(ctx, false);
    }
    const int keep = b < m.nb - 1;
    asv_launch_stream_next(d, m.s, (float)(m.bs - one_third), (float)two_third, keep, st);
    const int done = keep ? Db - one_third : Db;
    asv_launch_stream_map(d, m.s, (long long)WH * done, st);
    ctx->launches += 2;
    CK(cudaGetLastError());
    CK(cudaEventRecord(ev_end, st));
    CK(cudaMemcpyAsync(labels_out, m.s.lab_out, sizeof(int32_t) * WH * done, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(m.h_ctr2[par], m.s.ctr, sizeof(int) * STREAM_CTR_WORDS, cudaMemcpyDeviceToHost, st));
    CK(cudaEventRecord(ev_read, st));
    // the next block's device buffers and frame positions (its kernels run
    // after these in stream order)
    std::swap(m.s.kept_pos, m.s.kept_next);
    std::swap(m.s.gmap_prev, m.s.gmap_cur);
    m.prev_Db = Db;
    m.next++;
    m.fed_next = std::max(m.fed_next, m.next);
    ctx->have_rgb = ctx->have_flow = ctx->have_pos0 = ctx->have_M0 = ctx->have_lab = true;
    ctx->seeded = ctx->ran = true;
    auto &f = m.flight[m.nflight++];
    f.block = b;
    f.done = done;
    f.launches = ctx->launches;
    return ASV_OK;
}

// Waits for the oldest block in flight and takes in what it read back.
static asv_status stream_finish(asv_ctx *ctx, int *block, int *done_frames)
{
    if (!ctx) return ASV_ERR_BAD_ARG;
    auto &m = ctx->sm;
    if (!m.on || m.nflight == 0) return fail(ctx, ASV_ERR_STATE, "no block in flight");
    const asv_ctx::Stream::Flight f = m.flight[0];
    m.flight[0] = m.flight[1];
    m.nflight--;
    const int par = f.block & 1;
    cudaSetDevice(ctx->cfg.device);
    CK(cudaEventSynchronize(ctx->sev[3 * par + 2]));
    const int kp = m.h_ctr[par][STREAM_KP];
    if (kp < 0) {
        m.failed = true;
        return fail(ctx, kp == -2 ? ASV_ERR_CUDA : ASV_ERR_OVER_BUDGET,
                    kp == -2 ? "density placement produced fewer seeds than the grid"
                             : "kept + new seeds exceed the stream's seed capacity");
    }
    float wms = 0.f;
    CK(cudaEventElapsedTime(&wms, ctx->sev[3 * par], ctx->sev[3 * par + 1]));
    ctx->stats.window_ms = wms;
    ctx->stats.launches = f.launches;
    if (m.nflight == 0) ctx->seg[0].Kp = kp;                   // the host record is the last block's
    m.placed = m.h_ctr2[par][STREAM_PLACED];
    m.kept = m.h_ctr2[par][STREAM_KEPT];
    m.last_Kp = kp;
    if (block) *block = f.block;
    if (done_frames) *done_frames = f.done;
    return ASV_OK;
}

static asv_status stream_push(asv_ctx *ctx, bool fed, const uint8_t *rgb, const float *fwd, const float *bwd,
                              int32_t *labels_out, int *done_frames)
{
    if (ctx && ctx->sm.nflight > 0)
        return fail(ctx, ASV_ERR_STATE, "blocks in flight: asv_stream_wait for them first");
    const asv_status s = stream_enqueue(ctx, fed, rgb, fwd, bwd, labels_out);
    if (s != ASV_OK) return s;
    return stream_finish(ctx, nullptr, done_frames);
}

asv_status asv_stream_push(asv_ctx *ctx, const uint8_t *rgb, const float *fwd, const float *bwd,
                           int32_t *labels_out, int *done_frames)
{
    return stream_push(ctx, false, rgb, fwd, bwd, labels_out, done_frames);
}

asv_status asv_stream_push_fed(asv_ctx *ctx, int32_t *labels_out, int *done_frames)
{
    return stream_push(ctx, true, nullptr, nullptr, nullptr, labels_out, done_frames);
}

asv_status asv_stream_push_fed_async(asv_ctx *ctx, int32_t *labels_out)
{
    return stream_enqueue(ctx, true, nullptr, nullptr, nullptr, labels_out);
}

asv_status asv_stream_wait(asv_ctx *ctx, int *block, int *done_frames)
{
    return stream_finish(ctx, block, done_frames);
}

} // extern "C"
