/*
 * asv_oracle.c -- CPU restatement of the reference supervoxel path.
 *
 * TEST INFRASTRUCTURE ONLY (see asv_oracle.h).  Compiled with
 * -ffp-contract=off: every float/double operation below is one IEEE
 * operation in the order written, which is the evaluation order the CUDA
 * kernels reproduce.
 *
 * Reference files (paths inside dongxiao0401/anisotropic_supervoxel):
 *   GPU-AS/Image.cpp, GPU-AS/Render.cpp, GPU-AS/shaders,
 *   streamGPU-AS/Image.cpp, streamGPU-AS/Render.cpp.
 */
#include "asv_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define IDX(x, y, z) (((long)(z) * H + (y)) * (long)W + (x))

static int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* ======================================================================
 * Grid seeds: GPU-AS/Image.cpp:20-92 (init_seeds),
 *             streamGPU-AS/Image.cpp:26-103 (initialization_grid).
 * ==================================================================== */
int orc_grid_seeds(int W, int H, int D, int K, int middlebury, float *seeds4, int cap,
                   orc_grid_info *info)
{
    if (W < 1 || H < 1 || D < 1 || K < 1) return -1;
    long N = (long)W * H * D;
    double voxel_size = (double)(N / K);                       /* Image.cpp:24 (int division) */
    int s;
    if (middlebury) s = (int)floor(pow(1.0 * W * H / K, 0.5)); /* Image.cpp:28 */
    else s = (int)floor(pow(voxel_size, 1.0 / 3));             /* Image.cpp:32 */
    long kdd = (long)K * D * D / W / H;                         /* Image.cpp:37 */
    int dNum = (int)pow((double)(float)kdd, 1.0 / 3.0);
    if (dNum == 0) dNum = 1;
    int fsn = K / dNum;                                         /* :42 */
    int wNum = (int)sqrtf((float)((long)fsn * W / H));          /* :43 float sqrt */
    if (wNum == 0) return -2;
    int hNum = fsn / wNum;                                      /* :44 */
    if (hNum == 0) return -2;
    int Kp = dNum * hNum * wNum;                                /* :45 */
    if (info) {
        info->s = s; info->dNum = dNum; info->hNum = hNum; info->wNum = wNum; info->Kp = Kp;
    }
    if (!seeds4) return Kp;
    if (cap < Kp) return -3;
    int stepD = D / dNum, stepH = H / hNum, stepW = W / wNum;   /* :46-48 */
    int d_rem = D - stepD * dNum, h_rem = H - stepH * hNum, w_rem = W - stepW * wNum;
    int td = (d_rem < 1) ? 0 : 1, th, tw;                       /* :57-60 */
    int count = 0;
    for (int k = 0; k < dNum; k++) {
        th = 1;
        for (int i = 0; i < hNum; i++) {
            tw = 1;
            for (int j = 0; j < wNum; j++) {
                int sx = (int)(j * stepW + 0.5 * stepW + tw);   /* :71-73 double -> int */
                int sy = (int)(i * stepH + 0.5 * stepH + th);
                int sz = (int)(k * stepD + 0.5 * stepD + td);
                if (sx > W - 1) sx = W - 1;
                if (sy > H - 1) sy = H - 1;
                if (sz > D - 1) sz = D - 1;
                if (tw < w_rem) tw++;
                seeds4[4 * count + 0] = (float)(sx + 0.5);
                seeds4[4 * count + 1] = (float)(sy + 0.5);
                seeds4[4 * count + 2] = (float)(sz + 0.5);
                seeds4[4 * count + 3] = (float)count;
                count++;
            }
            if (th < h_rem) th++;
        }
        if (td < d_rem) td++;
    }
    return Kp;
}

/* ratio = (compactness/s)^2 in float: GPU-AS/Image.cpp:1050-1051,
 * streamGPU-AS/Image.cpp:968-969. */
float orc_ratio(int s, float compactness)
{
    float q = compactness / (float)s;
    return q * q;
}

/* ======================================================================
 * RGB -> LAB: GPU-AS/shaders/RGB2LAB.fs:11-79.  Input texel = unorm8/255.
 * ==================================================================== */
static float pow_cr(float x, float y) { return (float)pow((double)x, (double)y); }

static void lab_of(const uint8_t *c, uint8_t *out)
{
    float rgb[3], t[3];
    for (int k = 0; k < 3; k++) rgb[k] = (float)c[k] / 255.0f;
    for (int k = 0; k < 3; k++) {
        if (rgb[k] <= 0.04045f) t[k] = rgb[k] / 12.92f;                      /* fs:27-40 */
        else t[k] = pow_cr((rgb[k] + 0.055f) / 1.055f, 2.4f);
    }
    float X = (t[0] * 0.412453f + t[1] * 0.357580f) + t[2] * 0.180423f;    /* fs:19-21,42-44 */
    float Y = (t[0] * 0.212671f + t[1] * 0.715160f) + t[2] * 0.072169f;
    float Z = (t[0] * 0.019334f + t[1] * 0.119193f) + t[2] * 0.950227f;
    float r[3] = { X / 0.950456f, Y / 1.0f, Z / 1.088754f };                 /* fs:54-55 */
    float f[3];
    for (int k = 0; k < 3; k++) {
        if (r[k] > 0.008856f) f[k] = pow_cr(r[k], 1.0f / 3.0f);               /* fs:57-70 */
        else f[k] = (903.3f * r[k] + 16.0f) / 116.0f;
    }
    float L = 116.0f * f[1] - 16.0f;                                          /* fs:72 */
    float A = 500.0f * (f[0] - f[1]);
    float B = 200.0f * (f[1] - f[2]);
    L = L * 2.55f; A = A + 128.0f; B = B + 128.0f;                            /* fs:74-76 */
    float v[3] = { floorf(L + 0.5f), floorf(A + 0.5f), floorf(B + 0.5f) };   /* fs:77 */
    for (int k = 0; k < 3; k++) {
        float q = v[k] < 0.0f ? 0.0f : (v[k] > 255.0f ? 255.0f : v[k]);
        out[k] = (uint8_t)q;
    }
}

void orc_rgb2lab(const uint8_t *rgb, long n, uint8_t *lab4)
{
    for (long i = 0; i < n; i++) {
        lab_of(rgb + 3 * i, lab4 + 4 * i);
        lab4[4 * i + 3] = 0;
    }
}

/* ======================================================================
 * Gradient: GPU-AS/shaders/derivative_t.gs:24-49 (left, "up" = y-1 and
 * previous frame, clamp-to-edge), stored as RGB16F (Image.cpp:236-238).
 * ==================================================================== */
uint16_t orc_float_to_half(float f)
{
    uint32_t u; memcpy(&u, &f, 4);
    uint32_t sign = (u >> 16) & 0x8000u;
    uint32_t exp = (u >> 23) & 0xffu;
    uint32_t man = u & 0x7fffffu;
    if (exp == 0xffu) return (uint16_t)(sign | 0x7c00u | (man ? 0x200u : 0u));
    int e = (int)exp - 127 + 15;
    if (e >= 31) return (uint16_t)(sign | 0x7c00u);
    if (e <= 0) {
        if (e < -10) return (uint16_t)sign;
        man |= 0x800000u;
        int shift = 14 - e;
        uint32_t h = man >> shift;
        uint32_t rem = man & ((1u << shift) - 1u), half = 1u << (shift - 1);
        if (rem > half || (rem == half && (h & 1u))) h++;
        return (uint16_t)(sign | h);
    }
    uint32_t h = ((uint32_t)e << 10) | (man >> 13);
    uint32_t rem = man & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h++;
    return (uint16_t)(sign | h);
}

/* value of a non-negative half in units of 2^-24 */
static uint64_t half_units(uint16_t h)
{
    uint32_t e = (h >> 10) & 0x1fu, m = h & 0x3ffu;
    if (e == 0) return m;
    return (uint64_t)(1024u + m) << (e - 1);
}

static float gradient_of(const uint8_t *rgb, int W, int H, int D, int x, int y, int z)
{
    (void)D;
    const uint8_t *c = rgb + 3 * IDX(x, y, z);
    const uint8_t *nb[3] = { rgb + 3 * IDX(x > 0 ? x - 1 : 0, y, z),
                             rgb + 3 * IDX(x, y > 0 ? y - 1 : 0, z),
                             rgb + 3 * IDX(x, y, z > 0 ? z - 1 : 0) };
    float g = 0.0f;
    for (int k = 0; k < 3; k++) {
        float s = (float)abs((int)nb[k][0] - (int)c[0]);
        s = s + (float)abs((int)nb[k][1] - (int)c[1]);
        s = s + (float)abs((int)nb[k][2] - (int)c[2]);
        g = g + 0.33f * s;                                  /* derivative_t.gs:36,43,49 */
    }
    return g;
}

void orc_gradient_half(const uint8_t *rgb, int W, int H, int D, uint16_t *half_out)
{
    for (int z = 0; z < D; z++)
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++)
                half_out[IDX(x, y, z)] = orc_float_to_half(gradient_of(rgb, W, H, D, x, y, z));
}

/* ======================================================================
 * Gradient-density seed placement: GPU-AS/Image.cpp:350-620.
 * ==================================================================== */
static int mid_floor(float a, float b) { return (int)floor(0.5 * (double)(a + b)); } /* :375 */

/* Per-axis cell ranges of the grid seeds (Image.cpp:360-443).  The ranges
 * of a row/column depend on one index only, so the grid-cell id the
 * reference writes voxel by voxel (last k wins, :449-468) is the largest
 * (t, j, i) whose ranges contain the voxel. */
static void axis_ranges(const float *grid4, const orc_grid_info *g, int W, int H, int D,
                        int *xl, int *xr, int *yl, int *yr, int *zl, int *zr)
{
    int wN = g->wNum, hN = g->hNum, dN = g->dNum;
    for (int i = 0; i < wN; i++) {
        float c = grid4[4 * i];
        xl[i] = i > 0 ? mid_floor(grid4[4 * (i - 1)], c) : 0;
        xr[i] = i < wN - 1 ? mid_floor(grid4[4 * (i + 1)], c) : W - 1;
    }
    for (int j = 0; j < hN; j++) {
        float c = grid4[4 * (j * wN) + 1];
        yl[j] = j > 0 ? mid_floor(grid4[4 * ((j - 1) * wN) + 1], c) : 0;
        yr[j] = j < hN - 1 ? mid_floor(grid4[4 * ((j + 1) * wN) + 1], c) : H - 1;
    }
    for (int t = 0; t < dN; t++) {
        float c = grid4[4 * (t * wN * hN) + 2];
        zl[t] = t > 0 ? mid_floor(grid4[4 * ((t - 1) * wN * hN) + 2], c) : 0;
        zr[t] = t < dN - 1 ? mid_floor(grid4[4 * ((t + 1) * wN * hN) + 2], c) : D - 1;
    }
}

void orc_grid_cell_tables(int W, int H, int D, const float *grid4, const orc_grid_info *g,
                          int *xcell, int *ycell, int *zcell)
{
    int *xl = malloc(sizeof(int) * g->wNum), *xr = malloc(sizeof(int) * g->wNum);
    int *yl = malloc(sizeof(int) * g->hNum), *yr = malloc(sizeof(int) * g->hNum);
    int *zl = malloc(sizeof(int) * g->dNum), *zr = malloc(sizeof(int) * g->dNum);
    axis_ranges(grid4, g, W, H, D, xl, xr, yl, yr, zl, zr);
    for (int x = 0; x < W; x++) { xcell[x] = -1; for (int i = 0; i < g->wNum; i++) if (xl[i] <= x && x <= xr[i]) xcell[x] = i; }
    for (int y = 0; y < H; y++) { ycell[y] = -1; for (int j = 0; j < g->hNum; j++) if (yl[j] <= y && y <= yr[j]) ycell[y] = j; }
    for (int z = 0; z < D; z++) { zcell[z] = -1; for (int t = 0; t < g->dNum; t++) if (zl[t] <= z && z <= zr[t]) zcell[z] = t; }
    free(xl); free(xr); free(yl); free(yr); free(zl); free(zr);
}

int orc_density_adjust(const uint8_t *rgb, int W, int H, int D, const float *grid4,
                       const orc_grid_info *g, float *seeds4_out, float *density_out)
{
    int Kp = g->Kp;
    int *xc = malloc(sizeof(int) * W), *yc = malloc(sizeof(int) * H), *zc = malloc(sizeof(int) * D);
    orc_grid_cell_tables(W, H, D, grid4, g, xc, yc, zc);
    int nslot = Kp + 64;
    uint64_t *acc = calloc((size_t)nslot, sizeof(uint64_t));
    /* density_grid.vs:23-30: cell id read from an R16F texture (:474), slot
     * = id; the sum texture is cleared to 3.0 (Image.cpp:506-507). */
    for (int z = 0; z < D; z++)
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++) {
                if (xc[x] < 0 || yc[y] < 0 || zc[z] < 0) continue;
                int k = (zc[z] * g->hNum + yc[y]) * g->wNum + xc[x];
                uint16_t kh = orc_float_to_half((float)k);
                int slot = (int)(half_units(kh) >> 24);
                if (slot >= nslot) continue;
                uint16_t gh = orc_float_to_half(gradient_of(rgb, W, H, D, x, y, z));
                acc[slot] += half_units(gh);
            }
    float *dens = malloc(sizeof(float) * Kp), *len = malloc(sizeof(float) * Kp);
    for (int i = 0; i < Kp; i++) {
        uint64_t tot = acc[i] + ((uint64_t)3 << 24);
        float res = (float)tot * 0x1p-24f;                 /* read back as float */
        if (density_out) density_out[i] = res;
        dens[i] = (float)(0.001 * (double)res);            /* :554 */
    }
    for (int i = 0; i < Kp; i++) len[i] = i == 0 ? dens[0] : dens[i] + len[i - 1]; /* :558-569 */
    float interval = len[Kp - 1] / (float)(Kp + 1);        /* :570 */
    int *xl = malloc(sizeof(int) * g->wNum), *xr = malloc(sizeof(int) * g->wNum);
    int *yl = malloc(sizeof(int) * g->hNum), *yr = malloc(sizeof(int) * g->hNum);
    int *zl = malloc(sizeof(int) * g->dNum), *zr = malloc(sizeof(int) * g->dNum);
    axis_ranges(grid4, g, W, H, D, xl, xr, yl, yr, zl, zr);
    int i = 0, j1 = 0, n = 0;
    while (i < Kp) {                                       /* :586-616 */
        float seed_in = (float)(i + 1) * interval;
        if (seed_in < len[j1]) {
            int c = j1 % g->wNum;                          /* seed_range1d of cell j1 */
            int x1 = xl[c], x2 = xr[c];
            float frac = j1 == 0 ? seed_in / len[j1]
                                 : (seed_in - len[j1 - 1]) / (len[j1] - len[j1 - 1]);
            float ax = floorf((float)x1 + (float)(x2 - x1) * frac);
            seeds4_out[4 * n + 0] = (float)(ax + 0.5);
            seeds4_out[4 * n + 1] = grid4[4 * j1 + 1];
            seeds4_out[4 * n + 2] = grid4[4 * j1 + 2];
            seeds4_out[4 * n + 3] = (float)i;
            n++; i++;
        } else {
            j1++;
            if (j1 == Kp) break;
        }
    }
    free(xl); free(xr); free(yl); free(yr); free(zl); free(zr);
    free(xc); free(yc); free(zc); free(acc); free(dens); free(len);
    return n;
}

/* ======================================================================
 * Metric tensor from flow: GPU-AS/Image.cpp:874-1009 (matrix_slover).
 * Min-norm least squares in FP32, the reference's precision (it calls
 * Eigen's float BDCSVD::solve, :946-961), computed here with a one-sided
 * Jacobi SVD and Eigen's rank rule: keep singular values
 * >= max(sigma_max * min(m,6) * FLT_EPSILON, FLT_MIN).  Column dot products
 * are summed in a fixed pairwise order (lane_sum).
 * ==================================================================== */
#define SVD_SWEEPS 30

/* Sum of v[0..m-1] in the CUDA solver's warp butterfly order: 32 slots
 * (the values, then +0); for off = 16, 8, 4, 2, 1 slot i < off takes
 * t[i] + t[i + off]; the sum is slot 0. */
static int g_solver;
static float lane_sum(const float *v, int m)
{
    if (g_solver & 8) {                      /* the control: the same sums in sequential order */
        float acc = 0.0f;
        for (int i = 0; i < m; i++) acc = acc + v[i];
        return acc;
    }
    float t[32];
    for (int i = 0; i < 32; i++) t[i] = i < m ? v[i] : 0.0f;
    for (int off = 16; off > 0; off >>= 1)
        for (int i = 0; i < off; i++) t[i] = t[i] + t[i + off];
    return t[0];
}

static void lsq_minnorm(int m, float U[18][6], const float *b, float x[6])
{
    float tmp[18];
    float V[6][6];
    for (int r = 0; r < 6; r++) for (int c = 0; c < 6; c++) V[r][c] = r == c ? 1.0f : 0.0f;
    for (int sw = 0; sw < SVD_SWEEPS; sw++) {
        int rot = 0;
        for (int p = 0; p < 5; p++)
            for (int q = p + 1; q < 6; q++) {
                for (int i = 0; i < m; i++) tmp[i] = U[i][p] * U[i][p];
                const float al = lane_sum(tmp, m);
                for (int i = 0; i < m; i++) tmp[i] = U[i][q] * U[i][q];
                const float be = lane_sum(tmp, m);
                for (int i = 0; i < m; i++) tmp[i] = U[i][p] * U[i][q];
                const float ga = lane_sum(tmp, m);
                if (ga == 0.0f) continue;
                if (fabsf(ga) <= FLT_EPSILON * sqrtf(al * be)) continue;
                float zeta = (be - al) / (2.0f * ga);
                float t = 1.0f / (fabsf(zeta) + sqrtf(1.0f + zeta * zeta));
                if (zeta < 0.0f) t = -t;
                float c = 1.0f / sqrtf(1.0f + t * t);
                float s = c * t;
                for (int i = 0; i < m; i++) {
                    float up = U[i][p], uq = U[i][q];
                    U[i][p] = c * up - s * uq;
                    U[i][q] = s * up + c * uq;
                }
                for (int i = 0; i < 6; i++) {
                    float vp = V[i][p], vq = V[i][q];
                    V[i][p] = c * vp - s * vq;
                    V[i][q] = s * vp + c * vq;
                }
                rot++;
            }
        if (!rot) break;
    }
    float sig[6], smax = 0.0f;
    for (int j = 0; j < 6; j++) {
        for (int i = 0; i < m; i++) tmp[i] = U[i][j] * U[i][j];
        sig[j] = sqrtf(lane_sum(tmp, m));
        if (sig[j] > smax) smax = sig[j];
    }
    float thr = smax * ((float)(m < 6 ? m : 6) * FLT_EPSILON);
    if (thr < FLT_MIN) thr = FLT_MIN;
    for (int r = 0; r < 6; r++) x[r] = 0.0f;
    for (int j = 0; j < 6; j++) {
        if (!(sig[j] >= thr)) continue;
        for (int i = 0; i < m; i++) tmp[i] = U[i][j] * b[i];
        const float ub = lane_sum(tmp, m);
        float coef = (ub / sig[j]) / sig[j];
        for (int r = 0; r < 6; r++) x[r] = x[r] + V[r][j] * coef;
    }
}

/* Symmetric 3x3 eigen-decomposition, cyclic Jacobi in FP64. */
static void sym3_eig(const double Ain[3][3], double w[3], double V[3][3])
{
    double a[3][3];
    memcpy(a, Ain, sizeof(a));
    for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) V[r][c] = r == c ? 1.0 : 0.0;
    static const int P[3] = { 0, 0, 1 }, Q[3] = { 1, 2, 2 };
    for (int sw = 0; sw < 50; sw++) {
        int rot = 0;
        for (int k = 0; k < 3; k++) {
            int p = P[k], q = Q[k];
            double apq = a[p][q];
            if (apq == 0.0) continue;
            if (fabs(apq) <= 1e-18 * (fabs(a[p][p]) + fabs(a[q][q]))) continue;
            double th = (a[q][q] - a[p][p]) / (2.0 * apq);
            double t = 1.0 / (fabs(th) + sqrt(th * th + 1.0));
            if (th < 0.0) t = -t;
            double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
            for (int r = 0; r < 3; r++) {
                double ap = a[r][p], aq = a[r][q];
                a[r][p] = c * ap - s * aq;
                a[r][q] = s * ap + c * aq;
            }
            for (int r = 0; r < 3; r++) {
                double ap = a[p][r], aq = a[q][r];
                a[p][r] = c * ap - s * aq;
                a[q][r] = s * ap + c * aq;
            }
            for (int r = 0; r < 3; r++) {
                double vp = V[r][p], vq = V[r][q];
                V[r][p] = c * vp - s * vq;
                V[r][q] = s * vp + c * vq;
            }
            rot++;
        }
        if (!rot) break;
    }
    for (int k = 0; k < 3; k++) w[k] = a[k][k];
}

static void m6_to_3(const float M[6], double A[3][3])
{
    A[0][0] = M[0]; A[0][1] = M[1]; A[0][2] = M[2];
    A[1][0] = M[1]; A[1][1] = M[3]; A[1][2] = M[4];
    A[2][0] = M[2]; A[2][1] = M[4]; A[2][2] = M[5];
}

/* Knuth's TwoSum and the FMA TwoProduct: exact error terms */
static void two_sum(double a, double b, double *s, double *e)
{
    *s = a + b;
    double bb = *s - a;
    *e = (a - (*s - bb)) + (b - bb);
}

static void two_prod(double a, double b, double *p, double *e)
{
    *p = a * b;
    *e = fma(a, b, -*p);
}

/* Any eigenvalue < 0 (Image.cpp:997-1006), decided exactly: a symmetric
 * matrix is PSD iff every principal minor is >= 0.  Float products of two
 * are exact in double; the determinant is the exact sum of five triple
 * products, each split into an exact (hi, lo) pair, accumulated as a
 * nonoverlapping expansion (Shewchuk, "Adaptive precision floating-point
 * arithmetic", Grow-Expansion); its most significant non-zero component has
 * the sign of the sum.  Non-finite entries count as no negative eigenvalue. */
static int m6_negative(const float M[6])
{
    const double a = M[0], b = M[1], c = M[2], d = M[3], e = M[4], f = M[5];
    if (!(isfinite(a) && isfinite(b) && isfinite(c) && isfinite(d) && isfinite(e) && isfinite(f)))
        return 0;
    if (a < 0.0 || d < 0.0 || f < 0.0) return 1;
    if (a * d < b * b || a * f < c * c || d * f < e * e) return 1;
    double t[10], x[10];
    two_prod(a * d, f, &t[0], &t[1]);
    two_prod(2.0 * (b * c), e, &t[2], &t[3]);
    two_prod(-(a * e), e, &t[4], &t[5]);
    two_prod(-(d * c), c, &t[6], &t[7]);
    two_prod(-(f * b), b, &t[8], &t[9]);
    int n = 0;
    for (int k = 0; k < 10; k++) {
        double q = t[k];
        for (int i = 0; i < n; i++) {
            double h;
            two_sum(q, x[i], &q, &h);
            x[i] = h;
        }
        x[n++] = q;
    }
    for (int i = n - 1; i >= 0; i--)
        if (x[i] != 0.0) return x[i] < 0.0 ? 1 : 0;
    return 0;
}

int orc_m6_negative(const float M[6]) { return m6_negative(M); }

/* nearest PSD by clipping negative eigenvalues: Image.cpp:786-835 */
static void m6_nearest_psd(const float M[6], float out[6])
{
    double A[3][3], w[3], V[3][3];
    m6_to_3(M, A);
    sym3_eig(A, w, V);
    for (int k = 0; k < 3; k++) if (w[k] < 0.0) w[k] = 0.0;
    static const int R[6] = { 0, 0, 0, 1, 1, 2 }, C[6] = { 0, 1, 2, 1, 2, 2 };
    for (int e = 0; e < 6; e++) {
        int i = R[e], j = C[e];
        double acc = (V[i][0] * w[0]) * V[j][0];
        acc = acc + (V[i][1] * w[1]) * V[j][1];
        acc = acc + (V[i][2] * w[2]) * V[j][2];
        out[e] = (float)acc;
    }
}

/* ======================================================================
 * Second restatement of the metric solve, for measuring how much the
 * labels depend on the solver (orc_set_solver(1)): the algorithms of the
 * reference's Eigen calls, all in FP32 as the reference's MatrixXf is.
 *   - BDCSVD(A).solve(b) (Image.cpp:961): for a matrix of 6 columns BDCSVD
 *     hands the work to a two-sided Jacobi SVD; a non-square matrix is first
 *     reduced by a Householder QR with column pivoting (of A when it has
 *     more rows than columns, of A^T otherwise), the square factor is
 *     diagonalised by 2x2 rotation pairs (the left rotation makes the 2x2
 *     block symmetric, a symmetric Jacobi rotation then diagonalises it)
 *     until every off-diagonal entry is within 2 eps of its diagonal pair;
 *     singular values below sigma_max * min(m, 6) * eps count as zero and
 *     the solve is the minimum-norm one.
 *   - eigenvalues() (Image.cpp:997-1006): the matrix as a general 3x3 one,
 *     Householder reduction to Hessenberg form, then Francis double-shift QR
 *     steps with deflation on negligible subdiagonal entries; "negative"
 *     when an eigenvalue's real part is below 0.
 *   - the nearest PSD matrix (Image.cpp:786-835, :1460-1534): eigenvectors
 *     of the symmetric matrix (cyclic Jacobi in FP32), negative eigenvalues
 *     set to 0, V diag V^T.
 * These are this project's implementations of the published methods, not
 * Eigen itself (which is not vendored); they differ from the primary solver
 * (and from Eigen) in rounding only.
 * ==================================================================== */
/* g_solver bit 0: least squares, bit 1: PSD test, bit 2: nearest PSD by
 * the second restatement; bit 3: the primary solver's column sums in
 * sequential order (a control: the same algorithm, other rounding) */
void orc_set_solver(int mode) { g_solver = mode == 1 ? 7 : mode; }

/* two-sided Jacobi SVD of the square n x n matrix a (row-major, n <= 6):
 * a = U diag(s) V^T, s >= 0 sorted descending */
static void jacobi2_svd(int n, float a[6][6], float U[6][6], float V[6][6], float s[6])
{
    for (int r = 0; r < n; r++)
        for (int c = 0; c < n; c++) { U[r][c] = r == c ? 1.0f : 0.0f; V[r][c] = U[r][c]; }
    for (int sweep = 0; sweep < 64; sweep++) {
        int done = 1;
        for (int p = 1; p < n; p++)
            for (int q = 0; q < p; q++) {
                float thr = 2.0f * FLT_EPSILON * fmaxf(fabsf(a[p][p]), fabsf(a[q][q]));
                if (thr < FLT_MIN) thr = FLT_MIN;
                if (!(fabsf(a[p][q]) > thr || fabsf(a[q][p]) > thr)) continue;
                done = 0;
                /* block [[w, x], [y, z]] on rows/cols (q, p) */
                float w = a[q][q], x = a[q][p], y = a[p][q], z = a[p][p];
                /* left rotation making it symmetric: tan(t) = (y - x) / (w + z) */
                float c1 = 1.0f, s1 = 0.0f;
                float num = y - x, den = w + z;
                if (fabsf(num) > FLT_MIN) {
                    if (fabsf(den) < FLT_MIN) { c1 = 0.0f; s1 = num > 0.0f ? 1.0f : -1.0f; }
                    else {
                        float u = num / den, r = sqrtf(1.0f + u * u);
                        c1 = 1.0f / r; s1 = u / r;
                        if (den < 0.0f) { c1 = -c1; s1 = -s1; }
                    }
                }
                /* the symmetric block [[sa, sb], [sb, sd]] = R1 B */
                float sa = c1 * w + s1 * y, sb = c1 * x + s1 * z, sd = -s1 * x + c1 * z;
                float c2 = 1.0f, s2 = 0.0f;
                if (fabsf(sb) > FLT_MIN) {
                    float zeta = (sd - sa) / (2.0f * sb);
                    float t = 1.0f / (fabsf(zeta) + sqrtf(1.0f + zeta * zeta));
                    if (zeta < 0.0f) t = -t;
                    c2 = 1.0f / sqrtf(1.0f + t * t);
                    s2 = t * c2;
                }
                /* left: L = J^T R1, right: J = [[c2, s2], [-s2, c2]] */
                float lc = c2 * c1 + s2 * s1, ls = c2 * s1 - s2 * c1;
                for (int k = 0; k < n; k++) {           /* rows q, p of a <- L */
                    float aq = a[q][k], ap = a[p][k];
                    a[q][k] = lc * aq + ls * ap;
                    a[p][k] = -ls * aq + lc * ap;
                }
                for (int k = 0; k < n; k++) {           /* U <- U L^T */
                    float uq = U[k][q], up = U[k][p];
                    U[k][q] = lc * uq + ls * up;
                    U[k][p] = -ls * uq + lc * up;
                }
                for (int k = 0; k < n; k++) {           /* cols q, p of a <- a J; V <- V J */
                    float aq = a[k][q], ap = a[k][p];
                    a[k][q] = c2 * aq - s2 * ap;
                    a[k][p] = s2 * aq + c2 * ap;
                    float vq = V[k][q], vp = V[k][p];
                    V[k][q] = c2 * vq - s2 * vp;
                    V[k][p] = s2 * vq + c2 * vp;
                }
            }
        if (done) break;
    }
    for (int i = 0; i < n; i++) {
        s[i] = fabsf(a[i][i]);
        if (a[i][i] < 0.0f) for (int k = 0; k < n; k++) U[k][i] = -U[k][i];
    }
    for (int i = 0; i < n; i++) {                      /* sort descending */
        int best = i;
        for (int j = i + 1; j < n; j++) if (s[j] > s[best]) best = j;
        if (best != i) {
            float t = s[i]; s[i] = s[best]; s[best] = t;
            for (int k = 0; k < n; k++) {
                t = U[k][i]; U[k][i] = U[k][best]; U[k][best] = t;
                t = V[k][i]; V[k][i] = V[k][best]; V[k][best] = t;
            }
        }
    }
}

/* Householder QR with column pivoting of the r x c matrix M (r >= c, c <= 18
 * rows of at most 18): M P = Q R.  Q is r x c (thin), R c x c, perm[j] the
 * column of M in position j. */
static void qr_colpiv(int r, int c, float M[18][18], float Q[18][18], float R[6][6], int perm[18])
{
    float A[18][18];
    float vs[18][18];
    float beta[18];
    for (int i = 0; i < r; i++) for (int j = 0; j < c; j++) A[i][j] = M[i][j];
    for (int j = 0; j < c; j++) perm[j] = j;
    for (int k = 0; k < c; k++) {
        int best = k;
        float bn = -1.0f;
        for (int j = k; j < c; j++) {
            float s = 0.0f;
            for (int i = k; i < r; i++) s = s + A[i][j] * A[i][j];
            if (s > bn) { bn = s; best = j; }
        }
        if (best != k) {
            for (int i = 0; i < r; i++) { float t = A[i][k]; A[i][k] = A[i][best]; A[i][best] = t; }
            int t = perm[k]; perm[k] = perm[best]; perm[best] = t;
        }
        float norm = 0.0f;
        for (int i = k; i < r; i++) norm = norm + A[i][k] * A[i][k];
        norm = sqrtf(norm);
        for (int i = 0; i < r; i++) vs[k][i] = 0.0f;
        beta[k] = 0.0f;
        if (norm > 0.0f) {
            float alpha = A[k][k] > 0.0f ? -norm : norm;
            float v0 = A[k][k] - alpha;
            vs[k][k] = 1.0f;
            for (int i = k + 1; i < r; i++) vs[k][i] = A[i][k] / v0;
            float vv = 0.0f;
            for (int i = k; i < r; i++) vv = vv + vs[k][i] * vs[k][i];
            beta[k] = 2.0f / vv;
            for (int j = k; j < c; j++) {
                float d = 0.0f;
                for (int i = k; i < r; i++) d = d + vs[k][i] * A[i][j];
                d = d * beta[k];
                for (int i = k; i < r; i++) A[i][j] = A[i][j] - d * vs[k][i];
            }
        }
    }
    for (int i = 0; i < c; i++) for (int j = 0; j < c; j++) R[i][j] = j >= i ? A[i][j] : 0.0f;
    /* Q = H_0 ... H_{c-1} applied to the first c columns of the identity */
    for (int i = 0; i < r; i++) for (int j = 0; j < c; j++) Q[i][j] = i == j ? 1.0f : 0.0f;
    for (int k = c - 1; k >= 0; k--) {
        if (beta[k] == 0.0f) continue;
        for (int j = 0; j < c; j++) {
            float d = 0.0f;
            for (int i = k; i < r; i++) d = d + vs[k][i] * Q[i][j];
            d = d * beta[k];
            for (int i = k; i < r; i++) Q[i][j] = Q[i][j] - d * vs[k][i];
        }
    }
}

/* min-norm solution of the m x 6 system A x = b in the Eigen-style solver */
static void lsq_minnorm_qrsvd(int m, float A[18][6], const float *b, float x[6])
{
    float Ua[18][6], Va[6][6], s[6];
    int n = m < 6 ? m : 6;                             /* the diagonal size */
    float sq[6][6], Us[6][6], Vs[6][6];
    if (m == 6) {
        for (int i = 0; i < 6; i++) for (int j = 0; j < 6; j++) sq[i][j] = A[i][j];
        jacobi2_svd(6, sq, Us, Vs, s);
        for (int i = 0; i < 6; i++) for (int j = 0; j < 6; j++) { Ua[i][j] = Us[i][j]; Va[i][j] = Vs[i][j]; }
    } else if (m > 6) {                                /* A P = Q R, R = Us S Vs^T */
        float M[18][18], Q[18][18], R[6][6];
        int perm[18];
        for (int i = 0; i < m; i++) for (int j = 0; j < 6; j++) M[i][j] = A[i][j];
        qr_colpiv(m, 6, M, Q, R, perm);
        jacobi2_svd(6, R, Us, Vs, s);
        for (int i = 0; i < m; i++)
            for (int j = 0; j < 6; j++) {
                float acc = 0.0f;
                for (int k = 0; k < 6; k++) acc = acc + Q[i][k] * Us[k][j];
                Ua[i][j] = acc;
            }
        for (int j = 0; j < 6; j++) for (int k = 0; k < 6; k++) Va[perm[j]][k] = Vs[j][k];
    } else {                                           /* A^T P = Q R: A = P R^T Q^T */
        float M[18][18], Q[18][18], R[6][6], Rt[6][6];
        int perm[18];
        for (int i = 0; i < 6; i++) for (int j = 0; j < m; j++) M[i][j] = A[j][i];
        qr_colpiv(6, m, M, Q, R, perm);
        for (int i = 0; i < m; i++) for (int j = 0; j < m; j++) Rt[i][j] = R[j][i];
        jacobi2_svd(m, Rt, Us, Vs, s);                 /* R^T = Us S Vs^T */
        for (int i = 0; i < m; i++) for (int k = 0; k < m; k++) Ua[perm[i]][k] = Us[i][k];
        for (int i = 0; i < 6; i++)
            for (int j = 0; j < m; j++) {
                float acc = 0.0f;
                for (int k = 0; k < m; k++) acc = acc + Q[i][k] * Vs[k][j];
                Va[i][j] = acc;
            }
    }
    float thr = s[0] * ((float)n * FLT_EPSILON);
    if (thr < FLT_MIN) thr = FLT_MIN;
    for (int r = 0; r < 6; r++) x[r] = 0.0f;
    for (int j = 0; j < n; j++) {
        if (s[j] < thr) break;
        float ub = 0.0f;
        for (int i = 0; i < m; i++) ub = ub + Ua[i][j] * b[i];
        float coef = ub / s[j];
        for (int r = 0; r < 6; r++) x[r] = x[r] + Va[r][j] * coef;
    }
}

/* real parts of the eigenvalues of a general 3x3 matrix: Householder
 * Hessenberg reduction, then Francis double-shift QR with deflation (the
 * published real-Schur method), in FP32 */
static void eig3_general_real(const float Min[3][3], float wr[3])
{
    float a[3][3];
    memcpy(a, Min, sizeof(a));
    {   /* Hessenberg: zero a[2][0] with a reflection on rows/cols 1, 2 */
        float x1 = a[1][0], x2 = a[2][0];
        float nrm = sqrtf(x1 * x1 + x2 * x2);
        if (x2 != 0.0f && nrm > 0.0f) {
            float alpha = x1 > 0.0f ? -nrm : nrm;
            float v1 = x1 - alpha, v2 = x2;
            float vv = v1 * v1 + v2 * v2, beta = 2.0f / vv;
            for (int j = 0; j < 3; j++) {               /* H a */
                float d = beta * (v1 * a[1][j] + v2 * a[2][j]);
                a[1][j] = a[1][j] - d * v1;
                a[2][j] = a[2][j] - d * v2;
            }
            for (int i = 0; i < 3; i++) {               /* (H a) H */
                float d = beta * (a[i][1] * v1 + a[i][2] * v2);
                a[i][1] = a[i][1] - d * v1;
                a[i][2] = a[i][2] - d * v2;
            }
            a[2][0] = 0.0f;
        }
    }
    int hi = 2, iter = 0;
    float exshift = 0.0f;
    while (hi >= 0) {
        /* negligible subdiagonal entry below hi */
        int lo = hi;
        while (lo > 0) {
            float sc = fabsf(a[lo - 1][lo - 1]) + fabsf(a[lo][lo]);
            if (sc == 0.0f) sc = 1.0f;
            if (fabsf(a[lo][lo - 1]) <= FLT_EPSILON * sc) { a[lo][lo - 1] = 0.0f; break; }
            lo--;
        }
        if (lo == hi) {                                 /* a 1x1 block */
            wr[hi] = a[hi][hi] + exshift;
            hi--;
            iter = 0;
        } else if (lo == hi - 1) {                      /* a 2x2 block */
            float p = 0.5f * (a[hi - 1][hi - 1] - a[hi][hi]);
            float q = p * p + a[hi][hi - 1] * a[hi - 1][hi];
            float base = a[hi][hi] + exshift;
            if (q >= 0.0f) {
                float z = sqrtf(q);
                z = p >= 0.0f ? p + z : p - z;
                wr[hi - 1] = base + z;
                wr[hi] = z != 0.0f ? base - a[hi][hi - 1] * a[hi - 1][hi] / z : base + z;
            } else {
                wr[hi - 1] = wr[hi] = base + p;         /* a complex pair: the common real part */
            }
            hi -= 2;
            iter = 0;
        } else {                                        /* a 3x3 block: a double-shift step */
            if (++iter > 60) {                          /* no convergence: take the diagonal */
                for (int k = lo; k <= hi; k++) wr[k] = a[k][k] + exshift;
                break;
            }
            float x = a[hi][hi], y = a[hi - 1][hi - 1], w = a[hi][hi - 1] * a[hi - 1][hi];
            if (iter == 10 || iter == 20) {             /* exceptional shift */
                exshift += x;
                for (int k = lo; k <= hi; k++) a[k][k] -= x;
                float sft = fabsf(a[hi][hi - 1]) + fabsf(a[hi - 1][hi - 2 >= 0 ? hi - 2 : 0]);
                x = y = 0.75f * sft;
                w = -0.4375f * sft * sft;
            }
            /* first column of (H - s1)(H - s2), then bulge chase (n = 3) */
            float z0 = a[lo][lo];
            float r = x - z0, s = y - z0;
            float p = (r * s - w) / a[lo + 1][lo] + a[lo][lo + 1];
            float q = a[lo + 1][lo + 1] - z0 - r - s;
            float rr = a[lo + 2][lo + 1];
            {
                float xx = fabsf(p) + fabsf(q) + fabsf(rr);
                if (xx > 0.0f) { p /= xx; q /= xx; rr /= xx; }
            }
            /* the bulge of the previous step (left in place below the
             * subdiagonal, zero by construction) */
            for (int i = lo + 2; i <= hi; i++) { a[i][i - 2] = 0.0f; if (i != lo + 2) a[i][i - 3] = 0.0f; }
            for (int k = lo; k <= hi - 1; k++) {
                float xx = 1.0f;
                if (k != lo) {
                    p = a[k][k - 1];
                    q = a[k + 1][k - 1];
                    rr = k != hi - 1 ? a[k + 2][k - 1] : 0.0f;
                    xx = fabsf(p) + fabsf(q) + fabsf(rr);
                    if (xx == 0.0f) continue;
                    p /= xx; q /= xx; rr /= xx;
                }
                float sgn = sqrtf(p * p + q * q + rr * rr);
                if (p < 0.0f) sgn = -sgn;
                if (sgn == 0.0f) continue;
                if (k != lo) a[k][k - 1] = -sgn * xx;
                p = p + sgn;
                float xk = p / sgn, yk = q / sgn, zk = rr / sgn;
                q = q / p; rr = rr / p;
                for (int j = k; j <= hi; j++) {         /* rows k, k+1, k+2 */
                    float t = a[k][j] + q * a[k + 1][j];
                    if (k != hi - 1) { t = t + rr * a[k + 2][j]; a[k + 2][j] = a[k + 2][j] - t * zk; }
                    a[k + 1][j] = a[k + 1][j] - t * yk;
                    a[k][j] = a[k][j] - t * xk;
                }
                int mm = k + 3 < hi ? k + 3 : hi;
                for (int i = lo; i <= mm; i++) {        /* columns k, k+1, k+2 */
                    float t = xk * a[i][k] + yk * a[i][k + 1];
                    if (k != hi - 1) { t = t + zk * a[i][k + 2]; a[i][k + 2] = a[i][k + 2] - t * rr; }
                    a[i][k + 1] = a[i][k + 1] - t * q;
                    a[i][k] = a[i][k] - t;
                }
            }
        }
    }
}

/* test hooks of the second restatement */
void orc_eig3_real(const float M9[9], float wr[3])
{
    float A[3][3];
    for (int i = 0; i < 9; i++) A[i / 3][i % 3] = M9[i];
    eig3_general_real(A, wr);
}

void orc_lsq_qrsvd(int m, const float *A6, const float *b, float x[6])
{
    float A[18][6];
    for (int i = 0; i < m; i++) for (int j = 0; j < 6; j++) A[i][j] = A6[6 * i + j];
    lsq_minnorm_qrsvd(m, A, b, x);
}

static int m6_negative_eig(const float M[6])
{
    const float A[3][3] = { { M[0], M[1], M[2] }, { M[1], M[3], M[4] }, { M[2], M[4], M[5] } };
    float wr[3] = { 0.0f, 0.0f, 0.0f };
    eig3_general_real(A, wr);
    return (wr[0] < 0.0f || wr[1] < 0.0f || wr[2] < 0.0f) ? 1 : 0;
}

/* nearest PSD in FP32: cyclic Jacobi eigenvectors, clip, V diag V^T */
static void m6_nearest_psd_f32(const float M[6], float out[6])
{
    float a[3][3] = { { M[0], M[1], M[2] }, { M[1], M[3], M[4] }, { M[2], M[4], M[5] } };
    float V[3][3] = { { 1, 0, 0 }, { 0, 1, 0 }, { 0, 0, 1 } };
    static const int P[3] = { 0, 0, 1 }, Q[3] = { 1, 2, 2 };
    for (int sw = 0; sw < 50; sw++) {
        int rot = 0;
        for (int k = 0; k < 3; k++) {
            int p = P[k], q = Q[k];
            float apq = a[p][q];
            if (fabsf(apq) <= FLT_EPSILON * (fabsf(a[p][p]) + fabsf(a[q][q])) || apq == 0.0f) continue;
            float th = (a[q][q] - a[p][p]) / (2.0f * apq);
            float t = 1.0f / (fabsf(th) + sqrtf(th * th + 1.0f));
            if (th < 0.0f) t = -t;
            float c = 1.0f / sqrtf(t * t + 1.0f), s = t * c;
            for (int r = 0; r < 3; r++) { float ap = a[r][p], aq = a[r][q]; a[r][p] = c * ap - s * aq; a[r][q] = s * ap + c * aq; }
            for (int r = 0; r < 3; r++) { float ap = a[p][r], aq = a[q][r]; a[p][r] = c * ap - s * aq; a[q][r] = s * ap + c * aq; }
            for (int r = 0; r < 3; r++) { float vp = V[r][p], vq = V[r][q]; V[r][p] = c * vp - s * vq; V[r][q] = s * vp + c * vq; }
            rot++;
        }
        if (!rot) break;
    }
    float w[3];
    for (int k = 0; k < 3; k++) w[k] = a[k][k] < 0.0f ? 0.0f : a[k][k];
    static const int R[6] = { 0, 0, 0, 1, 1, 2 }, C[6] = { 0, 1, 2, 1, 2, 2 };
    for (int e = 0; e < 6; e++) {
        int i = R[e], j = C[e];
        out[e] = (V[i][0] * w[0]) * V[j][0] + (V[i][1] * w[1]) * V[j][1] + (V[i][2] * w[2]) * V[j][2];
    }
}

static float round_half_up(float f) { return (float)floor((double)f + 0.5); } /* :901 */

int orc_metric_solve(const float *fwd, const float *bwd, int W, int H, int D, float sx, float sy,
                     int frame, float M[6])
{
    static const float expected_b[9] = { 3, 2, 3, 2, 1, 2, 3, 2, 3 };      /* :884 */
    float A[18][6], b[18];
    int m = 0, id_b = 0;
    for (int oy = -1; oy < 2; oy++)
        for (int ox = -1; ox < 2; ox++, id_b++) {
            int nx = (int)sx + ox, ny = (int)sy + oy;
            if (!(nx >= 0 && nx < W && ny >= 0 && ny < H)) continue;
            long o = 2 * IDX(nx, ny, frame);
            if (frame != D - 1) {                                            /* :898-913 */
                float dx = (float)ox + round_half_up(fwd[o]);
                float dy = (float)oy + round_half_up(fwd[o + 1]);
                A[m][0] = dx * dx; A[m][1] = 2.0f * dx * dy;
                A[m][2] = 2.0f * dx; A[m][3] = dy * dy;
                A[m][4] = 2.0f * dy; A[m][5] = 1.0f;
                b[m++] = expected_b[id_b];
            }
            if (frame != 0) {                                                /* :915-930 */
                float dx = round_half_up(bwd[o]) + (float)ox;
                float dy = round_half_up(bwd[o + 1]) + (float)oy;
                A[m][0] = dx * dx; A[m][1] = 2.0f * dx * dy;
                A[m][2] = -2.0f * dx; A[m][3] = dy * dy;
                A[m][4] = -2.0f * dy; A[m][5] = 1.0f;
                b[m++] = expected_b[id_b];
            }
        }
    float x[6];
    if (m == 0) { for (int k = 0; k < 6; k++) x[k] = 0.0f; }
    else if (g_solver & 1) lsq_minnorm_qrsvd(m, A, b, x);
    else lsq_minnorm(m, A, b, x);
    for (int k = 0; k < 6; k++) M[k] = x[k];
    return (g_solver & 2) ? m6_negative_eig(M) : m6_negative(M);
}

/* flow-angle filter of the plain reseed (Image.cpp:1406-1409); flow of the
 * last frame is the 4x4 zero Mat (:664-667), read as zero everywhere. */
static int angle_ok(const float *fwd, int W, int H, int D, int frame, int sx, int sy, int nx, int ny)
{
    float sfx = 0.0f, sfy = 0.0f, nfx = 0.0f, nfy = 0.0f;
    if (frame != D - 1) {
        long o = 2 * IDX(sx, sy, frame), p = 2 * IDX(nx, ny, frame);
        sfx = fwd[o]; sfy = fwd[o + 1]; nfx = fwd[p]; nfy = fwd[p + 1];
    }
    float num = sfx * nfx + sfy * nfy;
    double den = sqrt((double)sfx * (double)sfx + (double)sfy * (double)sfy) *
                 sqrt((double)nfx * (double)nfx + (double)nfy * (double)nfy);
    float c = (float)((double)num / den);
    return (c >= ORC_FLOW_COS_MIN && c <= 1.0f) ? 1 : 0;
}

static const int R1X[8] = { -1, 0, 1, -1, 1, -1, 0, 1 }, R1Y[8] = { -1, -1, -1, 0, 0, 1, 1, 1 };
static const int R2X[16] = { -2, -1, 0, 1, 2, -2, 2, -2, 2, -2, 2, -2, -1, 0, 1, 2 };
static const int R2Y[16] = { -2, -2, -2, -2, -2, -1, -1, 0, 0, 1, 1, 2, 2, 2, 2, 2 };

/* seed_matrix (Image.cpp:689-856, reseed == 0) and Ld_next_seeds_matrix
 * (Image.cpp:1351-1534, reseed == 1; angle filter in the plain form only). */
void orc_seed_metrics(const float *fwd, const float *bwd, int W, int H, int D, int Kp,
                      const float *pos3, int reseed, int angle_filter, float *M6, int *kind)
{
    int filt = reseed && angle_filter;
    for (int i = 0; i < Kp; i++) {
        float fx = floorf(pos3[3 * i]), fy = floorf(pos3[3 * i + 1]);
        int frame = (int)pos3[3 * i + 2];
        float self[6], nb[6], sum[6] = { 0, 0, 0, 0, 0, 0 };
        int k = 0;
        if (!orc_metric_solve(fwd, bwd, W, H, D, fx, fy, frame, self)) {
            memcpy(M6 + 6 * i, self, sizeof(self));
        } else {
            int n = 0;
            for (int ring = 1; ring <= 2 && n == 0; ring++) {
                int cnt = ring == 1 ? 8 : 16;
                for (int t = 0; t < cnt; t++) {
                    float nx = fx + (float)(ring == 1 ? R1X[t] : R2X[t]);
                    float ny = fy + (float)(ring == 1 ? R1Y[t] : R2Y[t]);
                    if (!(nx >= 0 && nx < W && ny >= 0 && ny < H)) continue;
                    if (filt && !angle_ok(fwd, W, H, D, frame, (int)fx, (int)fy, (int)nx, (int)ny))
                        continue;
                    if (!orc_metric_solve(fwd, bwd, W, H, D, nx, ny, frame, nb)) {
                        n++;
                        for (int e = 0; e < 6; e++) sum[e] = sum[e] + nb[e];
                    }
                }
                k = ring;
            }
            if (n > 0) {
                for (int e = 0; e < 6; e++) M6[6 * i + e] = sum[e] / (float)n;
            } else {
                if (g_solver & 4) m6_nearest_psd_f32(self, M6 + 6 * i);
                else m6_nearest_psd(self, M6 + 6 * i);
                k = 3;
            }
        }
        if (kind) kind[i] = k;
    }
}

/* ======================================================================
 * JFA ladder: GPU-AS/Image.cpp:1055-1190.
 * steps[] and the ratio multiplier of each pass; returns the pass count.
 * ==================================================================== */
int orc_ladder(int s, int full, int maxdim, int *steps, float *rmul, int cap)
{
    int n = 0;
#define PUSH(st, rm) do { if (n < cap) { steps[n] = (st); rmul[n] = (rm); } n++; } while (0)
    PUSH(1, 1.0f);                                                          /* :1096 */
    if (!full) {
        float st = (float)floor(0.5 * s);                                   /* :1057 */
        while (st > 0) {                                                    /* :1105-1140 */
            PUSH((int)st, 1.0f);
            if ((int)st == 1) st = 0;
            st = (float)floor(0.5 * st + 0.5);
        }
    } else {
        int p = 1;
        while (p * 2 <= maxdim) p *= 2;
        for (; p >= 1; p /= 2) PUSH(p, 1.0f);
    }
    PUSH(2, 2.0f);                                                          /* :1143-1181 */
    PUSH(1, 2.0f);
#undef PUSH
    return n;
}

/* ======================================================================
 * Seed drawing: draw_seeds.vs / draw_next_seeds.vs write the seed record at
 * the seed voxel, later seeds overwriting earlier ones (primitive order).
 * ==================================================================== */
void orc_draw_seeds(int W, int H, int D, int Kp, const float *pos3, int32_t *labels)
{
    long N = (long)W * H * D;
    for (long v = 0; v < N; v++) labels[v] = -1;
    for (int i = 0; i < Kp; i++) {
        float px = pos3[3 * i], py = pos3[3 * i + 1], pz = pos3[3 * i + 2];
        if (!(px >= 0.0f && py >= 0.0f && pz >= 0.0f)) continue;
        int x = (int)px, y = (int)py, z = (int)pz;
        if (x >= W || y >= H || z >= D) continue;
        labels[IDX(x, y, z)] = i;
    }
}

/* seed colour of the first iteration: LAB sampled at the seed voxel
 * (draw_seeds.vs:23-24). */
void orc_seed_lab(int W, int H, int D, int Kp, const float *pos3, const uint8_t *lab4, float *slab3)
{
    for (int i = 0; i < Kp; i++) {
        int x = clampi((int)floorf(pos3[3 * i]), 0, W - 1);
        int y = clampi((int)floorf(pos3[3 * i + 1]), 0, H - 1);
        int z = clampi((int)floorf(pos3[3 * i + 2]), 0, D - 1);
        const uint8_t *l = lab4 + 4 * IDX(x, y, z);
        slab3[3 * i] = l[0]; slab3[3 * i + 1] = l[1]; slab3[3 * i + 2] = l[2];
    }
}

/* ======================================================================
 * One JFA pass: GPU-AS/shaders/flood.gs:26-182.
 * ==================================================================== */
static void jfa_voxel(int W, int H, int D, const int32_t *in, int32_t *out, const uint8_t *lab4,
                      const float *pos3, const float *slab3, const float *M6, int step, float ratio,
                      int x, int y, int z)
{
    float vx = (float)x + 0.5f, vy = (float)y + 0.5f, vz = (float)z + 0.5f;  /* flood.vs:18 */
    const uint8_t *cl = lab4 + 4 * IDX(x, y, z);
    float cL = cl[0], ca = cl[1], cb = cl[2];
    float min_dist = 100000000.0f;                                            /* gs:63 */
    int32_t best = -1;
    int zs[3] = { z, clampi(z - step, 0, D - 1), clampi(z + step, 0, D - 1) }; /* gs:73,106,140 */
    for (int sl = 0; sl < 3; sl++)
        for (int oy = -1; oy <= 1; oy++)
            for (int ox = -1; ox <= 1; ox++) {                                /* gs:36-46 */
                int nx = clampi(x + ox * step, 0, W - 1), ny = clampi(y + oy * step, 0, H - 1);
                int32_t l = in[IDX(nx, ny, zs[sl])];
                if (l < 0) continue;                                          /* gs:77 */
                const float *sp = pos3 + 3 * l, *sc = slab3 + 3 * l, *m = M6 + 6 * l;
                float dx = vx - sp[0], dy = vy - sp[1], dz = vz - sp[2];
                float p1 = (dx * dx) * m[0] + ((2.0f * dx) * dy) * m[1];           /* gs:85 */
                p1 = p1 + ((2.0f * dx) * dz) * m[2];
                float p2 = (dy * dy) * m[3] + ((2.0f * dy) * dz) * m[4];
                p2 = p2 + (dz * dz) * m[5];
                float pos = p1 + p2;
                float eL = cL - sc[0], ea = ca - sc[1], eb = cb - sc[2];
                float col = eL * eL + ea * ea;                                /* gs:89 */
                col = col + eb * eb;
                if (pos < 0.0f) pos = 0.0f;                                   /* gs:90-93 */
                float dist = ratio * pos + col;                               /* gs:94 */
                if (dist < min_dist) { min_dist = dist; best = l; }           /* gs:95-99 */
            }
    out[IDX(x, y, z)] = best;
}

void orc_jfa_pass(int W, int H, int D, const int32_t *in, int32_t *out, const uint8_t *lab4,
                  const float *pos3, const float *slab3, const float *M6, int step, float ratio,
                  int nthreads)
{
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1) if (nthreads > 1)
#endif
    for (int z = 0; z < D; z++)
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++)
                jfa_voxel(W, H, D, in, out, lab4, pos3, slab3, M6, step, ratio, x, y, z);
    (void)nthreads;
}

/* ======================================================================
 * Centroid sums: centroids.vs:19-54 -- per label slot (label -1 -> slot
 * Kp): sum of (x+.5, y+.5, z+.5), count, sum of LAB.  Kept exactly as
 * integers: [0..2] = sum of (2x+1), (2y+1), (2z+1); [3] = count;
 * [4..6] = sum of L, a, b.
 * ==================================================================== */
void orc_centroid_sums(int W, int H, int D, int Kp, const int32_t *labels, const uint8_t *lab4,
                       int64_t *sums, int nthreads)
{
    long nsl = (long)(Kp + 1) * 7;
    memset(sums, 0, sizeof(int64_t) * nsl);
#ifdef _OPENMP
    if (nthreads > 1) {
#pragma omp parallel num_threads(nthreads)
        {
            int64_t *loc = calloc((size_t)nsl, sizeof(int64_t));
#pragma omp for schedule(static)
            for (int z = 0; z < D; z++)
                for (int y = 0; y < H; y++)
                    for (int x = 0; x < W; x++) {
                        long v = IDX(x, y, z);
                        int l = labels[v];
                        int64_t *s = loc + 7L * (l < 0 ? Kp : l);
                        s[0] += 2 * x + 1; s[1] += 2 * y + 1; s[2] += 2 * z + 1; s[3] += 1;
                        s[4] += lab4[4 * v]; s[5] += lab4[4 * v + 1]; s[6] += lab4[4 * v + 2];
                    }
#pragma omp critical
            for (long i = 0; i < nsl; i++) sums[i] += loc[i];
            free(loc);
        }
        return;
    }
#endif
    (void)nthreads;
    for (int z = 0; z < D; z++)
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++) {
                long v = IDX(x, y, z);
                int l = labels[v];
                int64_t *s = sums + 7L * (l < 0 ? Kp : l);
                s[0] += 2 * x + 1; s[1] += 2 * y + 1; s[2] += 2 * z + 1; s[3] += 1;
                s[4] += lab4[4 * v]; s[5] += lab4[4 * v + 1]; s[6] += lab4[4 * v + 2];
            }
}

/* ======================================================================
 * Reseed: aver_exception.vs:22-81 (run unless it is the last iteration).
 * ==================================================================== */
static void slot_mean(int W, int Kp, const int64_t *sums, int slot, float q[3])
{
    /* texel of a slot outside 0..Kp was cleared to zero (Image.cpp:1247-1248) */
    if (slot < 0 || slot > Kp) { q[0] = q[1] = q[2] = 0.0f; return; }
    (void)W;
    const int64_t *s = sums + 7L * slot;
    float cnt = (float)s[3];
    for (int a = 0; a < 3; a++) {
        float sf = (float)s[a] * 0.5f;
        q[a] = ((int)cnt != 0) ? sf / cnt : sf;                    /* vs:37-40, 51-54 */
    }
}

void orc_finalize(int W, int H, int D, int Kp, const int64_t *sums, const uint8_t *lab4,
                  float *pos3, float *slab3)
{
    for (int id = 0; id < Kp; id++) {
        const int64_t *s = sums + 7L * id;
        if (s[3] != 0) {                                           /* vs:63-70 */
            float cnt = (float)s[3];
            for (int a = 0; a < 3; a++) {
                float sf = (float)s[a] * 0.5f;
                pos3[3 * id + a] = floorf(sf / cnt) + 0.5f;
                slab3[3 * id + a] = (float)s[4 + a] / cnt;
            }
        } else {                                                   /* vs:25-62 */
            /* id-1 for id 0 is texel (W-1, -1) clamped to row 0 = slot W-1 */
            int s1 = id == 0 ? W - 1 : id - 1, s2 = id + 1;
            float q1[3], q2[3];
            slot_mean(W, Kp, sums, s1, q1);
            slot_mean(W, Kp, sums, s2, q2);
            for (int a = 0; a < 3; a++) pos3[3 * id + a] = floorf(0.5f * (q1[a] + q2[a])) + 0.5f;
            int x = clampi((int)floorf(pos3[3 * id]), 0, W - 1);
            int y = clampi((int)floorf(pos3[3 * id + 1]), 0, H - 1);
            int z = clampi((int)floorf(pos3[3 * id + 2]), 0, D - 1);
            const uint8_t *l = lab4 + 4 * IDX(x, y, z);
            slab3[3 * id] = l[0]; slab3[3 * id + 1] = l[1]; slab3[3 * id + 2] = l[2];
        }
    }
}

/* ======================================================================
 * Post-processing: check_dead_seeds + label_replace + sequence_label,
 * GPU-AS/Image.cpp:1579-1778.  stats = {dead, neg_count, final_label_num}.
 * ==================================================================== */
int orc_postprocess(int W, int H, int D, int Kp, const int64_t *sums, int32_t *labels, int *stats)
{
    long N = (long)W * H * D;
    int invalid = sums[7L * Kp + 3] > 0;                            /* :1590 */
    int dead = 0, valid = 0;
    int *dead_ids = malloc(sizeof(int) * (Kp + 1));
    int *rank = malloc(sizeof(int) * (Kp + 1));
    for (int i = 0; i < Kp; i++) {                                  /* :1603-1618 */
        if (sums[7L * i + 3] < 1) { dead_ids[dead++] = i; rank[i] = -1; }
        else rank[i] = valid++;
    }
    if (stats) { stats[0] = dead; stats[1] = (int)sums[7L * Kp + 3]; stats[2] = valid; }
    if (dead >= 1 && dead <= 3) {                                   /* :1648-1674 */
        int last = Kp;
        for (int k = 0; k < dead; k++) {
            last -= 1;
            for (long v = 0; v < N; v++) if (labels[v] == last) labels[v] = dead_ids[k];
        }
    }
    if (dead > 3) {                                                 /* :1727-1747 */
        int l0 = labels[0];
        int m = (l0 >= 0 && l0 < Kp && rank[l0] >= 0) ? rank[l0] : 0;
        labels[0] = m;
        for (long v = 1; v < N; v++) {
            int l = labels[v];
            if (l != l0 && l != -1) m = (l >= 0 && l < Kp && rank[l] >= 0) ? rank[l] : 0;
            labels[v] = m;
        }
    } else if (invalid) {                                           /* :1750-1776 */
        int last = 0;
        if (labels[0] >= 0) last = labels[0];
        for (long v = 1; v < N; v++) {
            if (labels[v] != last) {
                if (labels[v] == -1) labels[v] = last;
                last = labels[v];
            }
        }
    }
    free(dead_ids); free(rank);
    return dead;
}

/* ====================================================================
 * 3D connectivity enforcement: Image::EnforceLabelConnectivity3D
 * (GPU-AS/Image.cpp:1938-2063; the same loop is streamGPU-AS/Render.cpp:
 * 572-695 label_connected3D over a whole video).  Voxels are visited in
 * raster order; an unvisited voxel starts a new segment: first the label
 * `adj` is taken from the last already-labelled voxel among its 24
 * neighbours (slices z-1, z, z+1 x the 8 in-plane offsets; the voxel
 * straight above or below is not a neighbour), in the loop order dz
 * -1, 0, 1 and offsets (-1,0) (-1,-1) (0,-1) (1,-1) (1,0) (1,1) (0,1)
 * (-1,1); `adj` keeps its previous value when none is labelled (0 at the
 * start).  The segment grows over unvisited neighbours with the seed's input
 * label; a segment of fewer than supsz / 4 voxels takes `adj` and does not
 * consume a new label.  Returns the number of labels.
 * ==================================================================== */
int orc_enforce_connectivity(const int32_t *labels, int W, int H, int D, int supsz, int32_t *out)
{
    static const int dx8[8] = { -1, -1, 0, 1, 1, 1, 0, -1 };
    static const int dy8[8] = { 0, -1, -1, -1, 0, 1, 1, 1 };
    const long n = (long)W * H * D, sl = (long)W * H;
    long *q = (long *)malloc(sizeof(long) * (size_t)(n > 0 ? n : 1));
    if (!q) return -1;
    for (long i = 0; i < n; i++) out[i] = -1;
    int label = 0, adj = 0;
    for (long s = 0; s < n; s++) {
        if (out[s] >= 0) continue;
        const int sx = (int)(s % W), sy = (int)((s / W) % H), sz = (int)(s / sl);
        out[s] = label;
        for (int dz = -1; dz <= 1; dz++) {                           /* :1980-1999 */
            int z = sz + dz;
            if (z < 0 || z >= D) continue;
            for (int k = 0; k < 8; k++) {
                int x = sx + dx8[k], y = sy + dy8[k];
                if (x < 0 || x >= W || y < 0 || y >= H) continue;
                long v = z * sl + (long)y * W + x;
                if (out[v] >= 0) adj = out[v];
            }
        }
        long head = 0, tail = 0;                                      /* :2001-2037 */
        q[tail++] = s;
        while (head < tail) {
            long c = q[head++];
            const int cx = (int)(c % W), cy = (int)((c / W) % H), cz = (int)(c / sl);
            for (int dz = -1; dz <= 1; dz++) {
                int z = cz + dz;
                if (z < 0 || z >= D) continue;
                for (int k = 0; k < 8; k++) {
                    int x = cx + dx8[k], y = cy + dy8[k];
                    if (x < 0 || x >= W || y < 0 || y >= H) continue;
                    long v = z * sl + (long)y * W + x;
                    if (out[v] < 0 && labels[v] == labels[s]) {
                        out[v] = label;
                        q[tail++] = v;
                    }
                }
            }
        }
        if (tail < supsz / 4) {                                       /* :2042-2050 */
            for (long i = 0; i < tail; i++) out[q[i]] = adj;
            label--;
        }
        label++;
    }
    free(q);
    return label;
}

/* final centroids of alive seeds (streamGPU-AS/Image.cpp:1563-1582) */
void orc_final_centroids(int Kp, const int64_t *sums, float *seeds4_out, int *nalive)
{
    int n = 0;
    for (int i = 0; i < Kp; i++) {
        const int64_t *s = sums + 7L * i;
        int area = (int)s[3];
        if (area < 1) continue;
        for (int a = 0; a < 3; a++) {
            float sf = (float)s[a] * 0.5f;
            seeds4_out[4 * n + a] = (float)(floorf(sf / (float)area) + 0.5);
        }
        seeds4_out[4 * n + 3] = (float)i;
        n++;
    }
    *nalive = n;
}

/* ======================================================================
 * One segmentation of a volume from given seeds: seed_matrix, RGB2LAB and
 * the Lloyd loop (GPU-AS/Render.cpp:268-293; streamGPU-AS/Render.cpp:470-504).
 * ==================================================================== */
typedef struct seg_out {
    int32_t *labels;   /* post-processed */
    int32_t *raw;      /* last JFA output */
    int64_t *sums;     /* (Kp+1)*7 of the last iteration */
    float *pos3, *slab3, *M6;
    int stats[3];
} seg_out;

static void segment(int W, int H, int D, int Kp, const float *init_pos3, int s, float ratio,
                    int angle_filter, int iters, int full_ladder, const uint8_t *lab4,
                    const float *fwd, const float *bwd, int nthreads, seg_out *o)
{
    long N = (long)W * H * D;
    int steps[64]; float rmul[64];
    int maxdim = W > H ? W : H; if (D > maxdim) maxdim = D;
    int P = orc_ladder(s, full_ladder, maxdim, steps, rmul, 64);
    int32_t *bufA = malloc(sizeof(int32_t) * N), *bufB = malloc(sizeof(int32_t) * N);
    float *pos3 = o->pos3, *slab3 = o->slab3, *M6 = o->M6;
    memcpy(pos3, init_pos3, sizeof(float) * 3 * Kp);
    orc_seed_metrics(fwd, bwd, W, H, D, Kp, pos3, 0, angle_filter, M6, NULL);
    orc_seed_lab(W, H, D, Kp, pos3, lab4, slab3);
    int32_t *cur = NULL;
    for (int it = 1; it <= iters; it++) {
        if (it > 1) orc_seed_metrics(fwd, bwd, W, H, D, Kp, pos3, 1, angle_filter, M6, NULL);
        orc_draw_seeds(W, H, D, Kp, pos3, bufA);
        int32_t *src = bufA, *dst = bufB;
        for (int p = 0; p < P; p++) {
            float r = rmul[p] * ratio;
            orc_jfa_pass(W, H, D, src, dst, lab4, pos3, slab3, M6, steps[p], r, nthreads);
            int32_t *t = src; src = dst; dst = t;
        }
        cur = src;
        orc_centroid_sums(W, H, D, Kp, cur, lab4, o->sums, nthreads);
        if (it != iters) orc_finalize(W, H, D, Kp, o->sums, lab4, pos3, slab3);
    }
    memcpy(o->raw, cur, sizeof(int32_t) * N);
    memcpy(o->labels, cur, sizeof(int32_t) * N);
    orc_postprocess(W, H, D, Kp, o->sums, o->labels, o->stats);
    free(bufA); free(bufB);
}

int orc_run_clip(const orc_params *p, const uint8_t *rgb, const float *fwd, const float *bwd,
                 int32_t *labels_out, int32_t *raw_labels_out, float *seeds_out, int *info_out)
{
    int W = p->W, H = p->H, D = p->D;
    long N = (long)W * H * D;
    if (D < 2) return -1;
    orc_grid_info g;
    int Kp = orc_grid_seeds(W, H, D, p->K, p->middlebury, NULL, 0, &g);
    if (Kp <= 0) return -2;
    float *grid4 = malloc(sizeof(float) * 4 * Kp), *adj4 = malloc(sizeof(float) * 4 * Kp);
    orc_grid_seeds(W, H, D, p->K, p->middlebury, grid4, Kp, &g);
    int n = Kp;
    if (p->density_adjust) n = orc_density_adjust(rgb, W, H, D, grid4, &g, adj4, NULL);
    else memcpy(adj4, grid4, sizeof(float) * 4 * Kp);
    if (n != Kp) { free(grid4); free(adj4); return -3; }
    float *pos3 = malloc(sizeof(float) * 3 * Kp);
    for (int i = 0; i < Kp; i++) for (int a = 0; a < 3; a++) pos3[3 * i + a] = adj4[4 * i + a];
    uint8_t *lab4 = malloc((size_t)N * 4);
    orc_rgb2lab(rgb, N, lab4);
    seg_out o;
    o.labels = labels_out;
    o.raw = raw_labels_out ? raw_labels_out : malloc(sizeof(int32_t) * N);
    o.sums = malloc(sizeof(int64_t) * 7 * (Kp + 1));
    o.pos3 = malloc(sizeof(float) * 3 * Kp); o.slab3 = malloc(sizeof(float) * 3 * Kp);
    o.M6 = malloc(sizeof(float) * 6 * Kp);
    float compact = p->variant == 1 ? 6.0f : 8.0f;
    segment(W, H, D, Kp, pos3, g.s, orc_ratio(g.s, compact), p->variant == 0, p->iters,
            p->full_ladder, lab4, fwd, bwd, p->nthreads, &o);
    if (seeds_out)
        for (int i = 0; i < Kp; i++) {
            for (int a = 0; a < 3; a++) seeds_out[12 * i + a] = o.pos3[3 * i + a];
            for (int a = 0; a < 3; a++) seeds_out[12 * i + 3 + a] = o.slab3[3 * i + a];
            for (int a = 0; a < 6; a++) seeds_out[12 * i + 6 + a] = o.M6[6 * i + a];
        }
    if (info_out) {
        info_out[0] = Kp; info_out[1] = g.s; info_out[2] = o.stats[0];
        info_out[3] = o.stats[1]; info_out[4] = o.stats[2];
    }
    if (!raw_labels_out) free(o.raw);
    free(o.sums); free(o.pos3); free(o.slab3); free(o.M6);
    free(grid4); free(adj4); free(pos3); free(lab4);
    return Kp;
}

/* ======================================================================
 * Streaming form: streamGPU-AS/Render.cpp:156-569.
 * info_out = {blocks, seeds_num_placed}.
 * ==================================================================== */
/* post_and_next's kept seeds (streamGPU-AS/Render.cpp:519-540): the final
 * centroids (x, y, z, id) of a block with z > block_size - block_size/3, z
 * shifted back by the block's new frames (1.5 when it would fall below 1);
 * returns how many, written to kept (4 floats each). */
int orc_stream_keep(const float *info, int n, int bs, float *kept)
{
    const int one_third = bs / 3, two_third = bs - one_third;
    int k = 0;
    for (int i = 0; i < n; i++) {
        float z = info[4 * i + 2];
        if (z > (float)(bs - one_third)) {
            float nz = z - (float)two_third;
            if (nz < 1) nz = 1.5f;
            kept[4 * k + 0] = info[4 * i + 0];
            kept[4 * k + 1] = info[4 * i + 1];
            kept[4 * k + 2] = nz;
            kept[4 * k + 3] = info[4 * i + 3];
            k++;
        }
    }
    return k;
}

int orc_stream_blocks(int D_all, int block_size, int *intervals, int cap)
{
    int one_third = block_size / 3, two_third = 2 * block_size / 3;     /* :200-201 */
    int n = 0, last_end = block_size, done = 0;
#define PUSHB(a, b) do { if (n + 1 < cap) { intervals[n] = (a); intervals[n + 1] = (b); } n += 2; } while (0)
    if (D_all < block_size + one_third) { PUSHB(0, D_all); done = 1; }
    else {
        PUSHB(0, last_end);
        while (last_end + two_third < D_all) {
            if (D_all - last_end - two_third < one_third) { PUSHB(last_end - one_third, D_all); done = 1; }
            else PUSHB(last_end - one_third, last_end + two_third);
            last_end += two_third;
        }
        if (!done) PUSHB(last_end - one_third, D_all);
    }
#undef PUSHB
    return n / 2;
}

int orc_run_stream(const orc_stream_params *p, const uint8_t *rgb, const float *fwd,
                   const float *bwd, int32_t *labels_all, int *info_out)
{
    int W = p->W, H = p->H, Dall = p->D_all, bs = p->block_size > 0 ? p->block_size : 30;
    long slice = (long)W * H;
    int seeds100 = p->seeds_num_100 > 0 ? p->seeds_num_100 : p->K_video * 100 / Dall; /* :157 */
    int iv[512];
    int nb = orc_stream_blocks(Dall, bs, iv, 512);
    if (nb > 256) return -1;
    int one_third = bs / 3;
    int two_third = bs - one_third;                                      /* post_and_next :516 */
    float *kept = NULL; int kept_num = 0;
    int *prev_map = NULL; int prev_map_n = 0;
    int placed = 0;
    for (int b = 0; b < nb; b++) {
        int start = iv[2 * b], end = iv[2 * b + 1], Db = end - start;
        long Nb = slice * Db;
        int seeds_num;
        if (b == 0) seeds_num = nb > 1 ? seeds100 * (Db - 10) / 100 : seeds100 * Db / 100; /* :351-356 */
        else seeds_num = seeds100 * (Db - 10) / 100;                    /* :394 */
        const uint8_t *brgb = rgb + 3 * slice * start;
        const float *bf = fwd + 2 * slice * start, *bb = bwd + 2 * slice * start;
        orc_grid_info g;
        int Kn = orc_grid_seeds(W, H, Db, seeds_num, 0, NULL, 0, &g);
        if (Kn <= 0) return -2;
        float *grid4 = malloc(sizeof(float) * 4 * Kn), *adj4 = malloc(sizeof(float) * 4 * Kn);
        orc_grid_seeds(W, H, Db, seeds_num, 0, grid4, Kn, &g);
        int na = orc_density_adjust(brgb, W, H, Db, grid4, &g, adj4, NULL);
        int Kp = kept_num + na;
        float *pos3 = malloc(sizeof(float) * 3 * Kp);
        int *map = malloc(sizeof(int) * Kp);
        int added_id = placed;
        for (int i = 0; i < Kp; i++) {                                   /* :438-460 */
            if (i < kept_num) {
                for (int a = 0; a < 3; a++) pos3[3 * i + a] = kept[4 * i + a];
                int old = (int)kept[4 * i + 3];
                map[i] = (b > 0 && old >= 0 && old < prev_map_n) ? prev_map[old] : 0;
            } else {
                int j = i - kept_num;
                for (int a = 0; a < 3; a++) pos3[3 * i + a] = adj4[4 * j + a];
                map[i] = b == 0 ? i : added_id++;
            }
        }
        uint8_t *lab4 = malloc((size_t)Nb * 4);
        orc_rgb2lab(brgb, Nb, lab4);
        seg_out o;
        o.labels = malloc(sizeof(int32_t) * Nb); o.raw = malloc(sizeof(int32_t) * Nb);
        o.sums = malloc(sizeof(int64_t) * 7 * (Kp + 1));
        o.pos3 = malloc(sizeof(float) * 3 * Kp); o.slab3 = malloc(sizeof(float) * 3 * Kp);
        o.M6 = malloc(sizeof(float) * 6 * Kp);
        segment(W, H, Db, Kp, pos3, g.s, orc_ratio(g.s, 6.0f), 0, p->iters, 0, lab4, bf, bb,
                p->nthreads, &o);
        float *info = malloc(sizeof(float) * 4 * Kp);
        int nal = 0;
        orc_final_centroids(Kp, o.sums, info, &nal);
        placed += nal - kept_num;                                         /* :514 */
        int done_frames = Db;
        free(kept); kept = NULL; kept_num = 0;
        if (b < nb - 1) {                                                 /* :519-557 */
            kept = malloc(sizeof(float) * 4 * (nal > 0 ? nal : 1));
            kept_num = orc_stream_keep(info, nal, bs, kept);
            done_frames = Db - one_third;
        }
        long done = slice * done_frames;                                  /* :559-563 */
        for (long i = 0; i < done; i++) {
            int l = o.labels[i];
            labels_all[slice * start + i] = (l >= 0 && l < Kp) ? map[l] : 0;
        }
        free(prev_map); prev_map = map; prev_map_n = Kp;
        free(info); free(o.labels); free(o.raw); free(o.sums); free(o.pos3); free(o.slab3);
        free(o.M6); free(lab4); free(pos3); free(grid4); free(adj4);
    }
    free(kept); free(prev_map);
    if (info_out) { info_out[0] = nb; info_out[1] = placed; }
    return nb;
}
