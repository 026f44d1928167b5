/*
 * asv_oracle.h -- CPU restatement of the reference supervoxel path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle the CUDA path is tested against:
 * only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg (and
 * the `--impl reference` arm) may load it.  The product (libasv) never links
 * or calls it.
 *
 * It restates, stage by stage, the reference's shader maths (GPU-AS/shaders)
 * and its Image.cpp host logic, with the float evaluation order written out
 * (compiled with -ffp-contract=off, so no FMA contraction).  Each function
 * names the reference file:line it follows.  Two points where the reference
 * itself is not deterministic are fixed here, identically in the CUDA path:
 *   - additive-blend FP32 sums (density per grid cell, centroid sums) are the
 *     exact sums (integer fixed point), rounded once to float where the
 *     reference reads them back as float;
 *   - GLSL pow() is taken as correctly rounded float pow.
 */
#ifndef ASV_ORACLE_H
#define ASV_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Smallest float cosine the plain-form flow-angle filter accepts
 * (GPU-AS/Image.cpp:1407-1409): theta = float(double(acosf(c))*(180/PI))
 * with PI = 3.141592653 is < 90 exactly for T <= c <= 1 when acosf is
 * correctly rounded.  Bits 0x328885a3. */
#define ORC_FLOW_COS_MIN 1.5893254712295857e-08f

typedef struct orc_grid_info {
    int s;       /* JFA base step, GPU-AS/Image.cpp:24-33 */
    int dNum, hNum, wNum;
    int Kp;      /* ac_seeds_num */
} orc_grid_info;

typedef struct orc_params {
    int W, H, D;
    int K;              /* requested seeds */
    int iters;          /* Lloyd iterations (reference default 20) */
    int variant;        /* 0 = plain GPU-AS (compactness 8, flow-angle filter), 1 = stream (6, none) */
    int full_ladder;    /* 0 = reference ladder, 1 = powers of two from log2(max dim) */
    int middlebury;     /* s from the 2-frame rule, GPU-AS/Image.cpp:25-29 */
    int density_adjust; /* 1 = reference gradient-density seed placement, 0 = grid only */
    int nthreads;       /* 1 = parity build order; >1 = OpenMP timing */
} orc_params;

/* ---- stages ---------------------------------------------------------- */
int  orc_grid_seeds(int W, int H, int D, int K, int middlebury,
                    float *seeds4, int cap, orc_grid_info *info);
float orc_ratio(int s, float compactness);
void orc_rgb2lab(const uint8_t *rgb, long n, uint8_t *lab4);
uint16_t orc_float_to_half(float f);
void orc_gradient_half(const uint8_t *rgb, int W, int H, int D, uint16_t *half_out);
void orc_grid_cell_tables(int W, int H, int D, const float *grid4, const orc_grid_info *g,
                          int *xcell, int *ycell, int *zcell);
int  orc_density_adjust(const uint8_t *rgb, int W, int H, int D, const float *grid4,
                        const orc_grid_info *g, float *seeds4_out, float *density_out);
/* 0: the primary solver (the CUDA path's twin); 1: the FP32 restatement of
 * the algorithms of the reference's Eigen calls (QR-preconditioned two-sided
 * Jacobi SVD, Hessenberg + Francis QR eigenvalues), for measuring how much
 * the labels depend on the solver.  Process-wide. */
void orc_set_solver(int mode);
void orc_eig3_real(const float M9[9], float wr[3]);                       /* test hooks of mode 1 */
void orc_lsq_qrsvd(int m, const float *A6, const float *b, float x[6]);
int  orc_m6_negative(const float M[6]);   /* exact "an eigenvalue < 0" of (M00,M01,M02,M11,M12,M22) */
int  orc_metric_solve(const float *fwd, const float *bwd, int W, int H, int D,
                      float sx, float sy, int frame, float M[6]);
void orc_seed_metrics(const float *fwd, const float *bwd, int W, int H, int D, int Kp,
                      const float *pos3, int reseed, int angle_filter, float *M6, int *kind);
int  orc_ladder(int s, int full, int maxdim, int *steps, float *rmul, int cap);
void orc_draw_seeds(int W, int H, int D, int Kp, const float *pos3, int32_t *labels);
void orc_seed_lab(int W, int H, int D, int Kp, const float *pos3, const uint8_t *lab4, float *slab3);
void orc_jfa_pass(int W, int H, int D, const int32_t *in, int32_t *out, const uint8_t *lab4,
                  const float *pos3, const float *slab3, const float *M6, int step, float ratio,
                  int nthreads);
void orc_centroid_sums(int W, int H, int D, int Kp, const int32_t *labels, const uint8_t *lab4,
                       int64_t *sums, int nthreads);
void orc_finalize(int W, int H, int D, int Kp, const int64_t *sums, const uint8_t *lab4,
                  float *pos3, float *slab3);
int  orc_postprocess(int W, int H, int D, int Kp, const int64_t *sums, int32_t *labels, int *stats);
int  orc_enforce_connectivity(const int32_t *labels, int W, int H, int D, int supsz, int32_t *out);
void orc_final_centroids(int Kp, const int64_t *sums, float *seeds4_out, int *nalive);

/* ---- whole plain per-clip run (GPU-AS/Render.cpp:254-303) ----------- */
int orc_run_clip(const orc_params *p, const uint8_t *rgb, const float *fwd, const float *bwd,
                 int32_t *labels_out, int32_t *raw_labels_out, float *seeds_out, int *info_out);

/* ---- streaming run (streamGPU-AS/Render.cpp:156-569) ----------------- */
typedef struct orc_stream_params {
    int W, H, D_all;
    int K_video;       /* seeds for the whole video (seeds_num_100 = K*100/D_all) */
    int seeds_num_100; /* if > 0, overrides the value derived from K_video */
    int iters;
    int block_size;    /* 30 */
    int nthreads;
} orc_stream_params;
int orc_run_stream(const orc_stream_params *p, const uint8_t *rgb, const float *fwd,
                   const float *bwd, int32_t *labels_all, int *info_out);

#ifdef __cplusplus
}
#endif
#endif
