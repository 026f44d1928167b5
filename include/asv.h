/*
 * asv.h -- C ABI of the GB300 supervoxel engine (libasv.so).
 *
 * The reference (dongxiao0401/anisotropic_supervoxel) has no plugin API; its
 * operator surface is the `Image` class that `Render::run` drives in a fixed
 * order (GPU-AS/Image.h:73-88, call order GPU-AS/Render.cpp:254-319).  Each
 * entry point below replaces one of those methods; the comment on each names
 * the method and the lines it replaces.
 *
 * Conventions
 *  - Every call returns asv_status (0 = ASV_OK).  asv_last_error() gives the
 *    message of the last failing call on a context.  No exception crosses
 *    the ABI.
 *  - The context owns all device memory.  Host buffers passed in or out stay
 *    owned by the caller and are not retained after the call returns.  The
 *    one exception is a 64 MiB RGB->LAB table per device, built by the first
 *    context that lays out a clip on that device, shared by all contexts,
 *    kept until the process exits and not counted against hbm_budget.
 *  - A context runs on one CUDA stream (its own, or the one in the config)
 *    and is not thread-safe; distinct contexts are independent.
 *  - Volumes are x-fastest [D][H][W] in texture orientation (row y = 0 is
 *    the bottom image row, as after the reference's vertical flip,
 *    GPU-AS/Render.cpp:354-359).  RGB is 3 bytes per voxel, flow is 2
 *    floats (dx, dy) per voxel, labels are int32 (-1 = no seed reached).
 *  - Sizes: 2 <= D, W,H,D <= 4096, requested seeds K >= 1, actual seed count
 *    K' < 32768 (the reference stores labels as R16I, GPU-AS/Image.cpp:263).
 */
#ifndef ASV_H
#define ASV_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int asv_status;
enum {
    ASV_OK = 0,
    ASV_ERR_BAD_ARG = 1,     /* invalid size / pointer / order of calls */
    ASV_ERR_OOM = 2,         /* device allocation failed */
    ASV_ERR_OVER_BUDGET = 3, /* request exceeds the configured HBM budget */
    ASV_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up */
    ASV_ERR_CUDA = 5,        /* a CUDA runtime call failed */
    ASV_ERR_STATE = 6,       /* call out of order (e.g. flood before init) */
    ASV_ERR_NO_DEVICE = 7    /* no CUDA device visible */
};

enum { ASV_VARIANT_PLAIN = 0, ASV_VARIANT_STREAM = 1 };

typedef struct asv_config {
    int variant;        /* ASV_VARIANT_PLAIN: compactness 8 + flow-angle filter on reseed
                           (GPU-AS/Image.cpp:1050, :1407-1410); ASV_VARIANT_STREAM:
                           compactness 6, no filter (streamGPU-AS/Image.cpp:968). */
    int lloyd_iters;    /* Lloyd iterations; reference default 20 (GPU-AS/Render.cpp:11) */
    int full_ladder;    /* 0: reference JFA ladder; 1: powers of two from log2(max dim) */
    int middlebury;     /* 1: s = floor(sqrt(W*H/K)) (GPU-AS/Image.cpp:25-29) */
    int density_adjust; /* 1: gradient-density seed placement (reference); 0: grid only */
    int device;         /* CUDA device ordinal */
    void *stream;       /* cudaStream_t to run on; NULL: the context creates its own */
    size_t hbm_budget;  /* bytes the context may allocate; 0 = unlimited */
    int use_graph;      /* 1: asv_run_lloyd replays a captured CUDA graph */
    int instrument;     /* 1: record per-stage CUDA-event times (asv_get_stats) */
    int jfa_zrun;       /* JFA tile depth (voxels of a column per tile, walked along the
                           step's chains); 0: chosen from the clip sizes; asv_autotune
                           measures it */
    int jfa_tile_blocks; /* 1: a JFA pass launches one block per tile, so its blocks retire
                           after each tile and kernels on higher-priority streams get SMs
                           between them (the server's contexts); 0: a persistent grid of
                           the resident blocks loops over the tiles (fastest alone) */
} asv_config;

typedef struct asv_info {
    int W, H, D;
    int K;              /* requested seeds */
    int Kp;             /* ac_seeds_num: seeds actually placed */
    int s;              /* JFA base step (GPU-AS/Image.cpp:24-33) */
    float ratio;        /* (compactness/s)^2 */
    int passes;         /* JFA passes per Lloyd iteration */
    int steps[32];      /* step of each pass */
    int dead;           /* dead seeds after the last iteration (GPU-AS/Image.cpp:1603-1618) */
    int neg_count;      /* voxels left at label -1 by the last JFA pass */
    int final_label_num;
} asv_info;

typedef struct asv_stats {
    double jfa_ms;      /* summed device time of the k_jfa gather passes of the last run
                           (every pass but each iteration's first two, seed scatters) */
    int jfa_launches;
    double centroid_ms;
    double metric_ms;
    double total_ms;    /* device time of the last asv_run_lloyd */
    int launches;       /* kernels launched by the last asv_run_lloyd or asv_stream_push */
    double window_ms;   /* device time of the last asv_stream_push's compute: from its
                           first kernel (the window's new frames already uploaded; the
                           optical flow included when it is computed on the device) to
                           the window's labels mapped, before they are read back */
} asv_stats;

typedef struct asv_ctx asv_ctx;

/* ---- lifetime ---------------------------------------------------------- */
void asv_config_default(asv_config *cfg);
asv_status asv_create(const asv_config *cfg, asv_ctx **out);
asv_status asv_destroy(asv_ctx *ctx);
const char *asv_last_error(const asv_ctx *ctx);
const char *asv_status_string(asv_status st);
int asv_version(void);

/* ---- the reference's Image methods, one entry point each -------------- */

/* Image::init_gpu + init_image_texture + init_seeds + init_variables
 * (GPU-AS/Image.cpp:320-345, :198-272, :20-158, :1047-1053): uploads the
 * RGB8 clip (D*H*W*3 bytes) and places the regular grid of seeds for K. */
asv_status asv_init_gpu(asv_ctx *ctx, const uint8_t *rgb, int W, int H, int D, int K);

/* asv_init_gpu for raw frames: D frames of BGR8, each top row first (as
 * read from a video), preprocessed on the device as Render::cvMat2TexureInput
 * does (GPU-AS/Render.cpp:354-359: 3x3 Gaussian blur, BGR -> RGB, vertical
 * flip) before they become the clip's RGB volume.  Same bytes as running
 * asv_preprocess_frame (asv_host.h) on each frame and calling asv_init_gpu. */
asv_status asv_init_gpu_bgr(asv_ctx *ctx, const uint8_t *bgr, int W, int H, int D, int K);

/* Output of Image::forward_backward_flow (GPU-AS/Image.cpp:643-686), which
 * the reference computes with OpenCV; here it is an input: fwd[z] is the
 * flow z -> z+1, bwd[z] the flow z -> z-1, each D*H*W*2 floats.  fwd[D-1]
 * and bwd[0] are not read by the metric solve. */
asv_status asv_upload_flow(asv_ctx *ctx, const float *fwd, const float *bwd);

/* Image::forward_backward_flow (GPU-AS/Image.cpp:643-686) on the device:
 * the forward (z -> z+1) and backward (z -> z-1) dense flow of every frame
 * of the clip(s) already uploaded, from their grey frames, in place of
 * asv_upload_flow.  The reference calls OpenCV's CUDA Farneback with its
 * default configuration; OpenCV is not available to this library, so this is
 * its own implementation of Farneback's polynomial-expansion method with that
 * configuration (5 levels, scale 0.5, neighbourhood 5, sigma 1.1, 13x13
 * window, 10 iterations): not bit-identical to OpenCV's.  Device scratch of
 * about 50 bytes per voxel and frame pair is held by the context. */
asv_status asv_compute_flow(asv_ctx *ctx);

/* Image::initialization (GPU-AS/Image.cpp:350-620): gradient-density seed
 * placement (derivative_t.gs, density_grid.vs, 1-D redistribution). */
asv_status asv_initialization(asv_ctx *ctx);

/* Image::seed_matrix (GPU-AS/Image.cpp:689-872) with matrix_slover
 * (:874-1009): per-seed metric tensor from flow, with the 1-ring / 2-ring /
 * nearest-PSD fallbacks, on the device. */
asv_status asv_seed_matrix(asv_ctx *ctx);

/* Image::RGB2LAB (GPU-AS/Image.cpp:296-315, shaders/RGB2LAB.fs). */
asv_status asv_rgb2lab(asv_ctx *ctx);

/* Image::Ld_first_init (GPU-AS/Image.cpp:1017-1045, shaders/draw_seeds). */
asv_status asv_ld_first_init(asv_ctx *ctx);

/* Image::flood (GPU-AS/Image.cpp:1061-1190, shaders/flood.gs): the JFA
 * ladder of one Lloyd iteration. */
asv_status asv_flood(asv_ctx *ctx, int lloyd_iter);

/* Image::centroids_next_seeds (GPU-AS/Image.cpp:1238-1297, shaders/
 * centroids.vs, aver_exception.vs): per-label sums and, unless lloyd_iter is
 * the last iteration, the reseed. */
asv_status asv_centroids_next_seeds(asv_ctx *ctx, int lloyd_iter);

/* Image::Ld_next_seeds_matrix (GPU-AS/Image.cpp:1300-1575): metric at the
 * new seed positions and the seed redraw, without the host round trip. */
asv_status asv_ld_next_seeds_matrix(asv_ctx *ctx, int lloyd_iter);

/* Image::check_dead_seeds + sequence_label (GPU-AS/Image.cpp:1579-1778):
 * dead-seed relabel and -1 fill on the device; copies the final labels to
 * labels_out (D*H*W int32) when it is not NULL. */
asv_status asv_check_dead_seeds(asv_ctx *ctx, int32_t *labels_out);

/* The whole Lloyd loop of Render::run (GPU-AS/Render.cpp:277-303): first
 * init, `lloyd_iters` x (reseed, flood, centroids), check_dead_seeds.  The
 * final labels stay on the device (read them with asv_get_labels). */
asv_status asv_run_lloyd(asv_ctx *ctx);

/* No counterpart in the reference.  Times the whole Lloyd loop at JFA tile
 * depths 4, 8, 16 and 32 (the voxels of a column one block walks along a
 * step's chains: deeper shares more slice work, shallower fills the GPU
 * better), keeps the fastest for this context (also for its later layouts)
 * and returns it in *zrun (may be NULL).  Needs a context ready for
 * asv_run_lloyd (clip or batch, not streaming); leaves the labels of a
 * complete run, which do not depend on the depth. */
asv_status asv_autotune(asv_ctx *ctx, int *zrun);

/* Convenience: init_gpu + upload_flow + initialization + seed_matrix +
 * RGB2LAB + run_lloyd + labels, the plain per-clip form of Render::run.
 * fwd and bwd both NULL: asv_compute_flow instead of upload_flow. */
asv_status asv_segment_clip(asv_ctx *ctx, const uint8_t *rgb, const float *fwd,
                            const float *bwd, int W, int H, int D, int K,
                            int32_t *labels_out);

/* Image::enforce_connectivity_3d (GPU-AS/Image.cpp:1808-1837) with
 * EnforceLabelConnectivity3D (:1938-2063), the reference's alternative to
 * check_dead_seeds (Render.cpp "6.2"): the raw labels of the last JFA pass
 * are split into connected segments (24-neighbourhood: the 8 in-plane
 * offsets in slices z-1, z, z+1) numbered in raster order, and segments of
 * fewer than supsz/4 voxels take the label of a neighbouring earlier
 * segment.  supsz <= 0 means W*H*D / K (texel_num / seeds_num, :1833).
 * Writes labels_out (D*H*W int32, may be NULL) and *label_num (may be NULL).
 * One clip per context (not a batch or a stream).  Device scratch of about
 * 32 bytes per voxel is held by the context after the first call. */
asv_status asv_enforce_connectivity(asv_ctx *ctx, int supsz, int32_t *labels_out, int *label_num);

/* The same on caller-provided labels: Render::label_connected3D of the
 * streaming form over a whole video (streamGPU-AS/Render.cpp:572-695), or any
 * label volume.  labels: D*H*W int32 host array; supsz > 0. */
asv_status asv_enforce_connectivity_labels(asv_ctx *ctx, const int32_t *labels, int W, int H, int D,
                                           int supsz, int32_t *labels_out, int *label_num);

/* ---- evaluation --------------------------------------------------------- */

/* Supervoxel quality against a ground-truth segmentation, as the LIBSVX
 * benchmark the reference is evaluated with (README.md:26-28; Xu & Corso,
 * CVPR 2012).  LIBSVX's code is not available to this library; these are
 * the definitions computed (n_sg = voxels of supervoxel s in truth segment
 * g, |s| and |g| the sizes, means over the truth segments present):
 *   undersegmentation    mean_g (sum_{s: n_sg > 0} |s| - |g|) / |g|
 *   segmentation_accuracy mean_g sum_{s: argmax_g' n_sg' = g} n_sg / |g|
 *                        (ties to the smaller truth id)
 *   boundary_recall      truth boundary voxels (a 6-neighbour in another
 *                        truth segment) with a supervoxel boundary voxel in
 *                        their 3x3x3 neighbourhood, over all of them
 *   mean_duration        mean over labels >= 0 of last - first frame + 1
 * Label -1 counts as one more supervoxel in the other measures.  labels: D*H*W int32 in
 * [-1, 32767); truth: D*H*W int32 in [0, 4096); both host arrays. */
typedef struct asv_eval {
    double undersegmentation;
    double segmentation_accuracy;
    double boundary_recall;
    double mean_duration;
    int supervoxels;            /* distinct labels present (with -1 if present) */
    int truth_segments;         /* distinct truth ids present */
    long long truth_boundary;   /* truth boundary voxels */
    long long recalled;         /* ... with a supervoxel boundary within one voxel */
} asv_eval;

asv_status asv_evaluate(asv_ctx *ctx, const int32_t *labels, const int32_t *truth, int W, int H, int D,
                        asv_eval *out);

/* ---- state access ------------------------------------------------------ */
asv_status asv_get_info(asv_ctx *ctx, asv_info *info);
asv_status asv_get_labels(asv_ctx *ctx, int32_t *out);     /* post-processed */
asv_status asv_get_raw_labels(asv_ctx *ctx, int32_t *out); /* last JFA pass */
/* the flow volumes on the device (uploaded or computed), D*H*W*2 floats each */
asv_status asv_get_flow(asv_ctx *ctx, float *fwd, float *bwd);
/* seed table, Kp x 12 floats: x, y, z, L, a, b, M00, M01, M02, M11, M12, M22 */
asv_status asv_get_seeds(asv_ctx *ctx, float *out);
asv_status asv_set_seeds(asv_ctx *ctx, const float *in, int Kp);
asv_status asv_get_lab(asv_ctx *ctx, uint8_t *out);        /* D*H*W*4 (L, a, b, 0) */
/* per-label sums of the last centroid pass, (Kp+1) x 7 int64: sum(2x+1),
 * sum(2y+1), sum(2z+1), count, sum L, sum a, sum b; row Kp = label -1 */
asv_status asv_get_sums(asv_ctx *ctx, int64_t *out);
/* check_dead_seeds over caller-given raw labels (D*H*W int32, -1 allowed):
 * recomputes the per-label sums from them, then relabels and fills as
 * asv_check_dead_seeds does; post-processed labels to out. */
asv_status asv_check_dead_seeds_host(asv_ctx *ctx, const int32_t *raw_in, int32_t *out);
/* one JFA pass over host label volumes with the current seed table */
asv_status asv_jfa_pass_host(asv_ctx *ctx, int step, float ratio, const int32_t *in, int32_t *out);
asv_status asv_get_stats(asv_ctx *ctx, asv_stats *st);
asv_status asv_get_stream(asv_ctx *ctx, void **stream);
asv_status asv_synchronize(asv_ctx *ctx);
/* bytes of device memory a clip of this size needs (admission control) */
size_t asv_clip_bytes(int W, int H, int D, int K);

/* ---- batched form -------------------------------------------------------- */

/* No single counterpart in the reference, which runs clips one after the
 * other (GPU-AS/main.cpp:74-83, one Render::run each).  Many clips of uneven
 * size share one context: every stage is one launch over all of them (each
 * JFA pass one persistent launch over the tiles of all clips; a clip with a
 * shorter ladder sits out the extra passes), and asv_run_lloyd replays the
 * whole loop as one CUDA graph.  Each clip's results equal its single-clip
 * run.  After asv_batch_init and one asv_batch_upload per clip, call
 * asv_initialization, asv_seed_matrix, asv_rgb2lab and asv_run_lloyd as for
 * one clip. */
asv_status asv_batch_init(asv_ctx *ctx, int n, const int *W, const int *H, const int *D, const int *K);
asv_status asv_batch_upload(asv_ctx *ctx, int clip, const uint8_t *rgb, const float *fwd, const float *bwd);
asv_status asv_batch_get_labels(asv_ctx *ctx, int clip, int32_t *out);
asv_status asv_batch_get_info(asv_ctx *ctx, int clip, asv_info *info);
/* bytes of device memory a batch needs (admission control) */
size_t asv_batch_bytes(int n, const int *W, const int *H, const int *D, const int *K);

/* ---- streaming form ---------------------------------------------------- */

/* The reference's streamGPU-AS form (streamGPU-AS/Render.cpp:100-569): a
 * long video segmented in blocks of `block_size` frames (30) that overlap by
 * block_size/3 (10); each block places its new seeds (grid + gradient
 * density) after the seeds carried from the previous block (final centroids
 * with z > block_size - block_size/3, shifted back), runs the Lloyd loop
 * with compactness 6 and no flow-angle filter, and maps its labels to
 * video-wide ids (block2all).  Here the overlap frames (RGB, LAB, flow), the
 * carried seeds and the id maps stay on the device between blocks; each push
 * uploads only the frames the block does not have yet. */
typedef struct asv_stream_info {
    int blocks;          /* blocks of the video */
    int next_block;      /* the block the next asv_stream_push processes */
    int block_start;     /* its frame range [block_start, block_end) */
    int block_end;
    int frames_needed;   /* new frames the next push must carry */
    int seeds_placed;    /* seeds_num_placed after the last processed block */
    int block_Kp;        /* seeds (carried + new) of the last processed block */
} asv_stream_info;

/* Replaces the block scheduling of Render::run (streamGPU-AS/Render.cpp:
 * 149-241).  seeds_num_100 (new seeds per 100 frames) is K_video*100/D_all
 * when given as 0 (:156-158); block_size 0 means 30.  Sets the context's
 * variant to ASV_VARIANT_STREAM. */
asv_status asv_stream_begin(asv_ctx *ctx, int W, int H, int D_all, int K_video, int seeds_num_100,
                            int block_size);
asv_status asv_stream_info_get(asv_ctx *ctx, asv_stream_info *info);

/* prepare_data_seeds + block_segment + post_and_next for the next block
 * (streamGPU-AS/Render.cpp:348-569).  rgb / fwd / bwd: the block's new
 * frames (frames_needed of them, same layouts as asv_init_gpu and
 * asv_upload_flow; fwd of a frame is its flow to the next frame of the
 * video).  fwd and bwd both NULL: the block's flow is computed on the
 * device from its frames (asv_compute_flow's method), as the streaming
 * program computes it per block.  labels_out: the video-wide labels of the
 * block's finished frames [block_start, block_start + *done_frames),
 * W*H*done_frames int32. */
asv_status asv_stream_push(asv_ctx *ctx, const uint8_t *rgb, const float *fwd, const float *bwd,
                           int32_t *labels_out, int *done_frames);

/* Frame range and new-frame count of block b (0 <= b < blocks). */
asv_status asv_stream_block(asv_ctx *ctx, int b, int *block_start, int *block_end, int *frames_needed);

/* Uploading ahead.  No counterpart in the reference, which reads a block's
 * frames when the block starts.  asv_stream_feed queues the host->device
 * copy of the new frames of the next block not yet fed (same buffers and
 * NULL-flow rule as asv_stream_push; frames_needed from asv_stream_block)
 * on the context's copy stream and returns at once, so the copy runs while
 * the block before it computes.  At most two blocks are fed ahead of the
 * next push (ASV_ERR_STATE beyond).  The host buffers must stay valid and
 * unchanged until the push of that block returns; pinned buffers make the
 * copy asynchronous.  A fed block is processed by asv_stream_push_fed (its
 * frames move from the staging slot into the window on the device); an
 * asv_stream_push of a fed block, or an asv_stream_push_fed of a block not
 * fed, fails with ASV_ERR_STATE.  The two staging slots (2 x block frames x
 * W*H*19 bytes) are allocated at the first feed. */
asv_status asv_stream_feed(asv_ctx *ctx, const uint8_t *rgb, const float *fwd, const float *bwd);
/* As asv_stream_feed with the frames as cv::imread gives them (8-bit BGR,
 * top row first): the push runs Render::cvMat2TexureInput on the device
 * (streamGPU-AS/Render.cpp:696-702: 3x3 Gaussian blur, BGR -> RGB, vertical
 * flip; the same arithmetic as asv_preprocess_frame). */
asv_status asv_stream_feed_bgr(asv_ctx *ctx, const uint8_t *bgr, const float *fwd, const float *bwd);
asv_status asv_stream_push_fed(asv_ctx *ctx, int32_t *labels_out, int *done_frames);

/* Pipelined form of asv_stream_push_fed: enqueues the next (fed) block and
 * returns at once, so the host can feed and enqueue the block after it while
 * this one runs; asv_stream_wait waits for the oldest block in flight and
 * gives its index and finished frame count (its labels are then in the
 * labels_out given at its enqueue, which must stay untouched until then).
 * At most two blocks are in flight (ASV_ERR_STATE beyond); the synchronous
 * asv_stream_push / asv_stream_push_fed need none in flight.  A block that
 * is refused (seed capacity) is reported by its wait, and the stream then
 * takes no further block.  No counterpart in the reference. */
asv_status asv_stream_push_fed_async(asv_ctx *ctx, int32_t *labels_out);
asv_status asv_stream_wait(asv_ctx *ctx, int *block, int *done_frames);

/* ---- serving ------------------------------------------------------------- */

/* No counterpart in the reference (a desktop program that segments one clip
 * at a time).  A request pool on one GPU: clip requests of any size are
 * admitted as soon as a slot and enough of the HBM budget are free (first
 * fit, so a small request can pass a large one that does not fit yet), each
 * admitted request runs on its slot's own CUDA stream so that the work of
 * several requests overlaps on the device (clips of up to 4 Mi voxels on a
 * higher-priority stream than larger ones, streaming windows on the highest
 * priority), and a slot keeps its device layout and captured graph for the
 * next request of the same shape.  Streaming
 * sessions hold a resident streaming context (asv_stream_*) whose windows
 * are processed in order.  Results are those of the single-clip / streaming
 * calls, whatever else is running. */
typedef struct asv_server asv_server;

enum { ASV_REQ_CLIP = 0, ASV_REQ_WINDOW = 1 };

typedef struct asv_request {
    int kind;             /* ASV_REQ_CLIP or ASV_REQ_WINDOW */
    int session;          /* window requests: the session id */
    int W, H, D, K;       /* clip requests: sizes and requested seeds */
    const uint8_t *rgb;   /* host inputs, valid until the request completes; for a window,
                             the block's new frames (asv_stream_push) */
    const float *fwd, *bwd;  /* both NULL: flow computed on the device */
    int32_t *labels_out;  /* host output: clip labels (D*H*W) or the window's finished frames
                             (room for W*H*(block_size + block_size/3) int32: the last
                             block of a video can be that long) */
} asv_request;

typedef struct asv_server_stats {
    long long submitted, completed, failed, queued, running;
    size_t bytes_in_use, budget;
    int slots, sessions;
} asv_server_stats;

/* max_slots: concurrent clip requests; hbm_budget: bytes all slots and
 * sessions together may hold (0 = no limit).  cfg applies to every slot.
 * With two or more slots, slot 0 serves clips of up to 4 Mi voxels only. */
asv_status asv_server_create(const asv_config *cfg, int max_slots, size_t hbm_budget, asv_server **out);
/* runs what is queued, then frees everything; no asv_server_wait may be in
 * progress on another thread.  A clip request that cannot fit beside the
 * open sessions even with every idle slot emptied fails with
 * ASV_ERR_OVER_BUDGET. */
asv_status asv_server_destroy(asv_server *srv);
/* a streaming session (asv_stream_begin semantics); fails with
 * ASV_ERR_OVER_BUDGET when its memory does not fit the budget */
asv_status asv_server_open_session(asv_server *srv, int W, int H, int D_all, int K_video,
                                   int seeds_num_100, int block_size, int *session);
asv_status asv_server_submit(asv_server *srv, const asv_request *req, long long *id);
/* blocks until request `id` completes; latency = submit -> completion (ms),
 * queue_ms = submit -> start; done_frames for windows */
asv_status asv_server_wait(asv_server *srv, long long id, double *latency_ms, double *queue_ms,
                           int *done_frames);
asv_status asv_server_poll(asv_server *srv, long long id, int *done);
asv_status asv_server_get_stats(asv_server *srv, asv_server_stats *st);

/* ---- post-processing without device allocation ------------------------- */

/* No counterpart in the reference.  The same dead-seed relabel and -1 fill
 * as asv_check_dead_seeds, for callers that cannot let a library allocate
 * device memory: hosts that give out every device byte from their own pool,
 * or latency-bound stages where cudaMalloc/cudaFree would synchronize the
 * device mid-pipeline.  The caller passes device buffers (d_raw: W*H*D
 * int32 raw labels in [-1, Kp); d_out: W*H*D int32) and an optional stream;
 * no context is needed.  d_raw and d_out must not overlap (an in-place call
 * returns ASV_ERR_BAD_ARG).  A label outside [-1, Kp) is read as -1.
 * Scratch is a fixed array of about 320 KiB inside
 * the library's device image, held by every device the library is loaded on
 * until the process exits.  Limits: W*H*D <= 2^25 voxels, Kp <= 32767
 * (ASV_ERR_BAD_ARG beyond).  The first call on a device resolves the
 * scratch address (make it before any stream capture).  All calls on a
 * device share the scratch and leave it holding their data; calls whose
 * work overlaps on the GPU race, so serialize them.  Run with the buffers'
 * device current.  A CUDA error already pending on the calling thread is
 * returned as ASV_ERR_CUDA before any work and left pending. */
#define ASV_NOALLOC_MAX_VOXELS (1LL << 25)
#define ASV_NOALLOC_MAX_SEEDS 32767
asv_status asv_check_dead_seeds_noalloc(const int32_t *d_raw, int32_t *d_out, int W, int H, int D,
                                        int Kp, void *stream);

#ifdef __cplusplus
}
#endif
#endif
