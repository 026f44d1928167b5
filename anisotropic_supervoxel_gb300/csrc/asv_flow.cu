// asv_flow.cu -- dense optical flow on the device for the clip's metric.
//
// The reference computes the forward and backward flow of every frame with
// OpenCV's CUDA Farneback (GPU-AS/Image.cpp:643-686, cuda::FarnebackOpticalFlow
// with its default configuration: 5 pyramid levels at scale 0.5, polynomial
// neighbourhood 5 with sigma 1.1, a 13x13 averaging window, 10 iterations per
// level) on the grey frames of the preprocessed clip (GPU-AS/Render.cpp:
// 227-243).  OpenCV is not available here, so this is this project's
// implementation of the published method (G. Farneback, "Two-frame motion
// estimation based on polynomial expansion", SCIA 2003) with that
// configuration; its results are not bit-compared with OpenCV's.
//
// Per pyramid level, coarse to fine, for every frame pair of the clip at once
// (frame z -> z+1 and z -> z-1):
//   1. polynomial expansion of each frame: a weighted least-squares fit of
//      f(x+u, y+v) ~ c + b1 u + b2 v + a11 u^2 + a22 v^2 + 2 a12 u v over a
//      5x5 window with Gaussian weights, computed as six separable moment
//      filters and the inverse of the (constant) 6x6 normal matrix;
//   2. per iteration: A = (A_src(x) + A_dst(x + d)) / 2 and
//      db = -(b_dst(x + d) - b_src(x)) / 2 + A d (bilinear samples of the
//      destination expansion), the products A^T A and A^T db averaged over
//      the 13x13 window, and d = (A^T A)^-1 A^T db per pixel;
//   3. the flow is upsampled to the next finer level.
// The grey frames use the integer RGB -> grey of ITU-R BT.601 with 14-bit
// fixed-point weights (4899, 9617, 1868).
#include "asv_flow.cuh"

#include <math.h>

#define FL_T 256
#define FL_N 2          // polynomial window half-size (neighbourhood 5)
#define FL_BOX 6        // averaging window half-size (13x13)
#define FL_MAX_LEVELS 5

__constant__ float c_fl_g[3][2 * FL_N + 1];   // g(t), t g(t), t^2 g(t), t = -N..N
__constant__ float c_fl_ginv[5][6];           // rows b1, b2, a11, a22, 2*a12 of the normal-matrix inverse

// ---------------------------------------------------------------------------
__global__ void k_fl_gray(const uint8_t *__restrict__ rgb, float *__restrict__ out, long long n)
{
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const uint8_t *p = rgb + 3 * v;
    out[v] = (float)((p[0] * 4899 + p[1] * 9617 + p[2] * 1868 + 8192) >> 14);
}

// 5x5 binomial blur ([1 4 6 4 1]^2 / 256, clamp to edge) and decimation by 2
__global__ void k_fl_down(const float *__restrict__ in, int Wi, int Hi, float *__restrict__ out, int Wo,
                          int Ho, int D)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long fo = (long long)Wo * Ho;
    if (t >= fo * D) return;
    const int z = (int)(t / fo), p = (int)(t - z * fo), y = p / Wo, x = p - y * Wo;
    const float w[5] = { 1.f, 4.f, 6.f, 4.f, 1.f };
    const float *src = in + (long long)Wi * Hi * z;
    float acc = 0.f;
    for (int j = -2; j <= 2; j++) {
        const int yy = min(max(2 * y + j, 0), Hi - 1);
        float row = 0.f;
        for (int i = -2; i <= 2; i++) row += w[i + 2] * src[(long long)yy * Wi + min(max(2 * x + i, 0), Wi - 1)];
        acc += w[j + 2] * row;
    }
    out[t] = acc * (1.f / 256.f);
}

// horizontal moments: h_p(x, y) = sum_u t^p g(u) f(x + u, y), p = 0, 1, 2
__global__ void k_fl_poly_h(const float *__restrict__ img, int W, int H, int D, float *__restrict__ h)
{
    const long long plane = (long long)W * H * D;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= plane) return;
    const int x = (int)(t % W);
    const long long row = t - x;
    float s0 = 0.f, s1 = 0.f, s2 = 0.f;
#pragma unroll
    for (int u = -FL_N; u <= FL_N; u++) {
        const float f = img[row + min(max(x + u, 0), W - 1)];
        s0 += c_fl_g[0][u + FL_N] * f;
        s1 += c_fl_g[1][u + FL_N] * f;
        s2 += c_fl_g[2][u + FL_N] * f;
    }
    h[t] = s0;
    h[plane + t] = s1;
    h[2 * plane + t] = s2;
}

// vertical moments and the fit: per pixel (b1, b2, a11, a22) in polyA and
// a12 in polyB, so a bilinear tap of the expansion is two loads
__global__ void k_fl_poly_v(const float *__restrict__ h, int W, int H, int D, float4 *__restrict__ polyA,
                            float *__restrict__ polyB)
{
    const long long plane = (long long)W * H * D;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= plane) return;
    const long long fr = (long long)W * H;
    const int z = (int)(t / fr);
    const int p = (int)(t - z * fr), y = p / W, x = p - y * W;
    float m[6] = { 0.f, 0.f, 0.f, 0.f, 0.f, 0.f };   // 1, u, v, u^2, v^2, uv
#pragma unroll
    for (int v = -FL_N; v <= FL_N; v++) {
        const long long q = fr * z + (long long)min(max(y + v, 0), H - 1) * W + x;
        const float h0 = h[q], h1 = h[plane + q], h2 = h[2 * plane + q];
        const float g = c_fl_g[0][v + FL_N], vg = c_fl_g[1][v + FL_N], vvg = c_fl_g[2][v + FL_N];
        m[0] += g * h0;
        m[1] += g * h1;
        m[2] += vg * h0;
        m[3] += g * h2;
        m[4] += vvg * h0;
        m[5] += vg * h1;
    }
    float r[5];
#pragma unroll
    for (int k = 0; k < 5; k++) {
        r[k] = 0.f;
#pragma unroll
        for (int e = 0; e < 6; e++) r[k] += c_fl_ginv[k][e] * m[e];
    }
    polyA[t] = make_float4(r[0], r[1], r[2], r[3]);
    polyB[t] = 0.5f * r[4];
}

// frame pair p: source and destination frames (forward pairs first)
__device__ __forceinline__ void fl_pair(int p, int D, int &src, int &dst)
{
    if (p < D - 1) { src = p; dst = p + 1; }
    else { src = p - (D - 1) + 1; dst = src - 1; }
}

// the per-pixel products A^T A (g11, g12, g22) and A^T db (h1, h2) at pixel
// (x, y) of the frame with the current flow (dx, dy), from the expansions
// sA/sB of the source frame and dA/dB of the destination frame; zero when
// x + d falls outside the frame
__device__ __forceinline__ void fl_matrix(const float4 *__restrict__ sA, const float *__restrict__ sB,
                                          const float4 *__restrict__ dA, const float *__restrict__ dB, int W,
                                          int H, int x, int y, float dx, float dy, float o[5])
{
    // no early exit: the sample indices are clamped into the frame whatever
    // the flow (also NaN), every load is issued, and the result is zeroed by
    // a select, so a thread's evaluations overlap their loads
    const float qx = (float)x + dx, qy = (float)y + dy;
    const bool inside = qx >= 0.f && qy >= 0.f && qx <= (float)(W - 1) && qy <= (float)(H - 1);
    const int x0 = min(max((int)qx, 0), W - 2 < 0 ? 0 : W - 2), y0 = min(max((int)qy, 0), H - 2 < 0 ? 0 : H - 2);
    const int x1 = min(x0 + 1, W - 1), y1 = min(y0 + 1, H - 1);
    const float fx = qx - (float)x0, fy = qy - (float)y0;
    const float w00 = (1.f - fx) * (1.f - fy), w01 = fx * (1.f - fy), w10 = (1.f - fx) * fy, w11 = fx * fy;
    const int s = y * W + x;                                   // frames hold < 2^31 pixels
    const int i00 = y0 * W + x0, i01 = y0 * W + x1, i10 = y1 * W + x0, i11 = y1 * W + x1;
    const float4 t00 = __ldg(dA + i00), t01 = __ldg(dA + i01), t10 = __ldg(dA + i10), t11 = __ldg(dA + i11);
    const float u00 = __ldg(dB + i00), u01 = __ldg(dB + i01), u10 = __ldg(dB + i10), u11 = __ldg(dB + i11);
    const float4 sa = __ldg(sA + s);
    const float sb = __ldg(sB + s);
    float q[5];
    q[0] = w00 * t00.x + w01 * t01.x + w10 * t10.x + w11 * t11.x;
    q[1] = w00 * t00.y + w01 * t01.y + w10 * t10.y + w11 * t11.y;
    q[2] = w00 * t00.z + w01 * t01.z + w10 * t10.z + w11 * t11.z;
    q[3] = w00 * t00.w + w01 * t01.w + w10 * t10.w + w11 * t11.w;
    q[4] = w00 * u00 + w01 * u01 + w10 * u10 + w11 * u11;
    const float a11 = 0.5f * (sa.z + q[2]);
    const float a22 = 0.5f * (sa.w + q[3]);
    const float a12 = 0.5f * (sb + q[4]);
    const float db1 = -0.5f * (q[0] - sa.x) + a11 * dx + a12 * dy;
    const float db2 = -0.5f * (q[1] - sa.y) + a12 * dx + a22 * dy;
    o[0] = inside ? a11 * a11 + a12 * a12 : 0.f;
    o[1] = inside ? a11 * a12 + a12 * a22 : 0.f;
    o[2] = inside ? a12 * a12 + a22 * a22 : 0.f;
    o[3] = inside ? a11 * db1 + a12 * db2 : 0.f;
    o[4] = inside ? a12 * db1 + a22 * db2 : 0.f;
}

// One iteration for a TW x TH tile of one frame pair: the five matrix planes
// of the tile and its 6-pixel halo are computed from the flow `fin` straight
// into shared memory (zero outside the frame), summed over the 13x13 window
// -- rows along x, then the row sums along y, both in ascending index order,
// so the sums equal those of separate x and y passes -- and each pixel's 2x2
// system is solved into `fout`.  fin and fout are separate buffers: halo
// pixels read flow that neighbouring tiles overwrite.
template <int TW, int TH, int NT>
__global__ void __launch_bounds__(NT) k_fl_iter(const float4 *__restrict__ polyA, const float *__restrict__ polyB,
                                                const float *__restrict__ fin, float *__restrict__ fout, int W,
                                                int H, int D, int P)
{
    constexpr int RPT = TH / (NT / 32);              // output rows per thread
    static_assert(TW % 32 == 0 && RPT >= 1 && RPT * (NT / 32) == TH, "tile shape");
    extern __shared__ float fl_sm[];
    constexpr int RW = TW + 2 * FL_BOX, RH = TH + 2 * FL_BOX, SP = RW + 1, TP = TW + 1;
    float *S = fl_sm;                                  // [5][RH][SP]
    float *T = fl_sm + 5 * RH * SP;                    // [RH][TP]
    const long long fr = (long long)W * H, mplane = fr * P;
    const int tiles_x = (W + TW - 1) / TW, tiles_y = (H + TH - 1) / TH;
    // blocks take the pairs as z -> z+1, z+1 -> z, z+1 -> z+2, ...: the two
    // pairs of a frame pair read the same two expansions while both are in L2
    const int j = blockIdx.x / (tiles_x * tiles_y);
    const int pr = (j & 1) ? D - 1 + (j >> 1) : (j >> 1);
    const int rem = blockIdx.x - j * tiles_x * tiles_y;
    const int x0 = (rem % tiles_x) * TW, y0 = (rem / tiles_x) * TH;
    int src, dst;
    fl_pair(pr, D, src, dst);
    const float4 *sA = polyA + fr * src, *dA = polyA + fr * dst;
    const float *sB = polyB + fr * src, *dB = polyB + fr * dst;
    const float *fx_in = fin + fr * pr, *fy_in = fin + mplane + fr * pr;
    for (int i0 = threadIdx.x; i0 < RW * RH; i0 += 2 * NT) {     // two pixels per trip
        int cell[2];
        bool keep[2];
        float o[2][5];
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const int i = i0 + u * NT;
            cell[u] = i < RW * RH ? i : 0;
            const int r = cell[u] / RW, q = cell[u] - r * RW;
            const int gy = y0 - FL_BOX + r, gx = x0 - FL_BOX + q;
            keep[u] = gx >= 0 && gx < W && gy >= 0 && gy < H;       // zero outside the frame
            const int cx = min(max(gx, 0), W - 1), cy = min(max(gy, 0), H - 1);
            const int e = cy * W + cx;
            fl_matrix(sA, sB, dA, dB, W, H, cx, cy, __ldg(fx_in + e), __ldg(fy_in + e), o[u]);
        }
#pragma unroll
        for (int u = 0; u < 2; u++) {
            if (i0 + u * NT >= RW * RH) continue;
            const int r = cell[u] / RW, q = cell[u] - r * RW;
#pragma unroll
            for (int c = 0; c < 5; c++) S[(c * RH + r) * SP + q] = keep[u] ? o[u][c] : 0.f;
        }
    }
    __syncthreads();
    const int tx = threadIdx.x % 32, ty = threadIdx.x / 32;            // 32 x NT/32 threads
    float acc[TW / 32][RPT][5];
    // window sums several at a time from registers: a thread loads the
    // values of adjacent windows once (horizontal: four windows, one column
    // group per warp with lanes on rows, so with the odd row pitches a
    // warp's loads and stores fall in distinct banks; vertical: RPT rows)
#pragma unroll
    for (int c = 0; c < 5; c++) {
        const float *Sc = S + c * RH * SP;
        for (int g = threadIdx.x / 32; g < TW / 4; g += NT / 32)
            for (int r = threadIdx.x % 32; r < RH; r += 32) {
                const int q = 4 * g;
                float w[16];
#pragma unroll
                for (int k = 0; k < 16; k++) w[k] = Sc[r * SP + q + k];
#pragma unroll
                for (int m = 0; m < 4; m++) {
                    float v = 0.f;
#pragma unroll
                    for (int k = 0; k <= 2 * FL_BOX; k++) v += w[m + k];
                    T[r * TP + q + m] = v;
                }
            }
        __syncthreads();
#pragma unroll
        for (int a = 0; a < TW / 32; a++) {
            const int q = tx + 32 * a;
            float w[RPT + 2 * FL_BOX];
#pragma unroll
            for (int k = 0; k < RPT + 2 * FL_BOX; k++) w[k] = T[(RPT * ty + k) * TP + q];
#pragma unroll
            for (int j = 0; j < RPT; j++) {
                float v = 0.f;
#pragma unroll
                for (int k = 0; k <= 2 * FL_BOX; k++) v += w[j + k];
                acc[a][j][c] = v;
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < TW / 32; a++)
#pragma unroll
        for (int j = 0; j < RPT; j++) {
            const int x = x0 + tx + 32 * a, y = y0 + RPT * ty + j;
            if (x >= W || y >= H) continue;
            const float g11 = acc[a][j][0], g12 = acc[a][j][1], g22 = acc[a][j][2];
            const float h1 = acc[a][j][3], h2 = acc[a][j][4];
            const float idet = 1.f / (g11 * g22 - g12 * g12 + 1e-3f);
            const long long e = fr * pr + (long long)y * W + x;
            fout[e] = (g22 * h1 - g12 * h2) * idet;
            fout[mplane + e] = (g11 * h2 - g12 * h1) * idet;
        }
}

#define FL_TW 64
#define FL_TH 32
#define FL_NT 512
static constexpr size_t fl_iter_smem(int tw, int th)
{
    return sizeof(float) * (size_t)(5 * (th + 2 * FL_BOX) * (tw + 2 * FL_BOX + 1) + (th + 2 * FL_BOX) * (tw + 1));
}

// flow of level k from level k+1: bilinear, scaled by the size ratio
__global__ void k_fl_up(const float *__restrict__ coarse, int Wc, int Hc, float *__restrict__ fine, int W, int H,
                        int P)
{
    const long long fr = (long long)W * H, mplane = fr * P, cfr = (long long)Wc * Hc, cplane = cfr * P;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= mplane) return;
    const int pr = (int)(t / fr);
    const int pix = (int)(t - pr * fr), y = pix / W, x = pix - y * W;
    const float sx = (float)Wc / (float)W, sy = (float)Hc / (float)H;
    const float cx = fminf(fmaxf(((float)x + 0.5f) * sx - 0.5f, 0.f), (float)(Wc - 1));
    const float cy = fminf(fmaxf(((float)y + 0.5f) * sy - 0.5f, 0.f), (float)(Hc - 1));
    const int x0 = (int)cx, y0 = (int)cy, x1 = min(x0 + 1, Wc - 1), y1 = min(y0 + 1, Hc - 1);
    const float fx = cx - (float)x0, fy = cy - (float)y0;
    const long long b = cfr * pr;
    for (int c = 0; c < 2; c++) {
        const float *F = coarse + c * cplane + b;
        const float v = (1.f - fx) * (1.f - fy) * F[(long long)y0 * Wc + x0] + fx * (1.f - fy) * F[(long long)y0 * Wc + x1] +
                        (1.f - fx) * fy * F[(long long)y1 * Wc + x0] + fx * fy * F[(long long)y1 * Wc + x1];
        fine[c * mplane + t] = v / (c == 0 ? sx : sy);
    }
}

// level-0 flow of the pairs into the clip's interleaved fwd / bwd volumes
__global__ void k_fl_store(const float *__restrict__ flow, int W, int H, int D, float2 *__restrict__ fwd,
                           float2 *__restrict__ bwd, int keep_first_bwd)
{
    const long long fr = (long long)W * H, vox = fr * D, mplane = fr * 2 * (D - 1);
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= vox) return;
    const int z = (int)(t / fr);
    const long long pix = t - z * fr;
    float2 f = make_float2(0.f, 0.f), b = make_float2(0.f, 0.f);
    if (z < D - 1) {
        const long long e = fr * z + pix;
        f = make_float2(flow[e], flow[mplane + e]);
    }
    if (z > 0) {
        const long long e = fr * (D - 1 + z - 1) + pix;
        b = make_float2(flow[e], flow[mplane + e]);
    }
    fwd[t] = f;
    if (z > 0 || !keep_first_bwd) bwd[t] = b;
}

// ---------------------------------------------------------------------------
static int fl_levels(int W, int H, int *Ws, int *Hs)
{
    int L = 0, w = W, h = H;
    while (L < FL_MAX_LEVELS) {
        Ws[L] = w; Hs[L] = h;
        L++;
        const int nw = (w + 1) / 2, nh = (h + 1) / 2;
        if (nw < 16 || nh < 16) break;
        w = nw; h = nh;
    }
    return L;
}

size_t asv_flow_scratch_bytes(int W, int H, int D)
{
    if (D < 2) return 0;
    int Ws[FL_MAX_LEVELS], Hs[FL_MAX_LEVELS];
    const int L = fl_levels(W, H, Ws, Hs);
    const long long P = 2LL * (D - 1);
    size_t b = 0;
    for (int k = 0; k < L; k++) {
        const long long fr = (long long)Ws[k] * Hs[k];
        b += (size_t)fr * D * (1 + 3 + 5) * 4;     // image, horizontal moments, expansion
        b += (size_t)fr * P * 2 * 4;               // flow
    }
    const long long fr0 = (long long)W * H;
    b += (size_t)fr0 * P * 2 * 4;                  // second flow buffer (iterations alternate)
    return b + 64 * 256;
}

struct FlConsts {
    float g[3][2 * FL_N + 1];
    float ginv[5][6];
};

// Gaussian applicability (sigma 1.1) t^p g(t), and rows 1..5 of the inverse
// of the 6x6 normal matrix sum w B B^T of the basis B = (1, u, v, u^2, v^2, uv)
static FlConsts fl_consts()
{
    FlConsts K;
    const double sigma = 1.1;
    double g[2 * FL_N + 1];
    for (int u = -FL_N; u <= FL_N; u++) {
        g[u + FL_N] = exp(-(double)(u * u) / (2.0 * sigma * sigma));
        K.g[0][u + FL_N] = (float)g[u + FL_N];
        K.g[1][u + FL_N] = (float)(u * g[u + FL_N]);
        K.g[2][u + FL_N] = (float)(u * u * g[u + FL_N]);
    }
    double G[6][12] = {};
    for (int v = -FL_N; v <= FL_N; v++)
        for (int u = -FL_N; u <= FL_N; u++) {
            const double w = g[u + FL_N] * g[v + FL_N];
            const double B[6] = { 1.0, (double)u, (double)v, (double)(u * u), (double)(v * v), (double)(u * v) };
            for (int i = 0; i < 6; i++)
                for (int j = 0; j < 6; j++) G[i][j] += w * B[i] * B[j];
        }
    for (int i = 0; i < 6; i++) G[i][6 + i] = 1.0;
    for (int c = 0; c < 6; c++) {                               // Gauss-Jordan, partial pivoting
        int piv = c;
        for (int r = c + 1; r < 6; r++) if (fabs(G[r][c]) > fabs(G[piv][c])) piv = r;
        for (int j = 0; j < 12; j++) { const double tmp = G[c][j]; G[c][j] = G[piv][j]; G[piv][j] = tmp; }
        const double d = G[c][c];
        for (int j = 0; j < 12; j++) G[c][j] /= d;
        for (int r = 0; r < 6; r++)
            if (r != c) {
                const double f = G[r][c];
                for (int j = 0; j < 12; j++) G[r][j] -= f * G[c][j];
            }
    }
    for (int k = 0; k < 5; k++)
        for (int e = 0; e < 6; e++) K.ginv[k][e] = (float)G[k + 1][6 + e];
    return K;
}

static float *fl_carve(unsigned char *&p, size_t floats)
{
    float *r = (float *)p;
    p += (floats * 4 + 255) & ~(size_t)255;
    return r;
}

static unsigned fl_blocks(long long n) { return (unsigned)((n + FL_T - 1) / FL_T); }

int asv_launch_flow(const uint8_t *rgb, int W, int H, int D, float2 *fwd, float2 *bwd, void *scratch,
                    cudaStream_t st, int keep_first_bwd)
{
    if (D < 2) return -1;
    // filter constants: computed once (thread-safe static), copied to this
    // device's constant memory on the stream before the kernels that read them
    static const FlConsts K = fl_consts();
    if (cudaMemcpyToSymbolAsync(c_fl_g, K.g, sizeof(K.g), 0, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyToSymbolAsync(c_fl_ginv, K.ginv, sizeof(K.ginv), 0, cudaMemcpyHostToDevice, st) != cudaSuccess)
        return -1;
    int Ws[FL_MAX_LEVELS], Hs[FL_MAX_LEVELS];
    const int L = fl_levels(W, H, Ws, Hs);
    const int P = 2 * (D - 1);
    unsigned char *p = (unsigned char *)scratch;
    float *img[FL_MAX_LEVELS], *hm[FL_MAX_LEVELS], *polyB[FL_MAX_LEVELS], *flow[FL_MAX_LEVELS];
    float4 *polyA[FL_MAX_LEVELS];
    for (int k = 0; k < L; k++) {
        const size_t fr = (size_t)Ws[k] * Hs[k];
        img[k] = fl_carve(p, fr * D);
        hm[k] = fl_carve(p, fr * D * 3);
        polyA[k] = (float4 *)fl_carve(p, fr * D * 4);      // 256-byte aligned
        polyB[k] = fl_carve(p, fr * D);
        flow[k] = fl_carve(p, fr * P * 2);
    }
    const size_t fr0 = (size_t)W * H;
    float *alt = fl_carve(p, fr0 * P * 2);
    const size_t smem = fl_iter_smem(FL_TW, FL_TH);
    if (cudaFuncSetAttribute(k_fl_iter<FL_TW, FL_TH, FL_NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return -1;

    k_fl_gray<<<fl_blocks((long long)fr0 * D), FL_T, 0, st>>>(rgb, img[0], (long long)fr0 * D);
    for (int k = 1; k < L; k++)
        k_fl_down<<<fl_blocks((long long)Ws[k] * Hs[k] * D), FL_T, 0, st>>>(img[k - 1], Ws[k - 1], Hs[k - 1], img[k],
                                                                          Ws[k], Hs[k], D);
    for (int k = 0; k < L; k++) {
        const long long n = (long long)Ws[k] * Hs[k] * D;
        k_fl_poly_h<<<fl_blocks(n), FL_T, 0, st>>>(img[k], Ws[k], Hs[k], D, hm[k]);
        k_fl_poly_v<<<fl_blocks(n), FL_T, 0, st>>>(hm[k], Ws[k], Hs[k], D, polyA[k], polyB[k]);
    }
    for (int k = L - 1; k >= 0; k--) {
        const int w = Ws[k], h = Hs[k];
        const long long mplane = (long long)w * h * P;
        if (k == L - 1) cudaMemsetAsync(flow[k], 0, sizeof(float) * mplane * 2, st);
        else k_fl_up<<<fl_blocks(mplane), FL_T, 0, st>>>(flow[k + 1], Ws[k + 1], Hs[k + 1], flow[k], w, h, P);
        const unsigned tiles = (unsigned)(((w + FL_TW - 1) / FL_TW) * ((h + FL_TH - 1) / FL_TH) * P);
        for (int it = 0; it < 10; it++) {                 // even count: the result ends in flow[k]
            const float *fin = (it & 1) ? alt : flow[k];
            float *fout = (it & 1) ? flow[k] : alt;
            k_fl_iter<FL_TW, FL_TH, FL_NT><<<tiles, FL_NT, smem, st>>>(polyA[k], polyB[k], fin, fout, w, h, D, P);
        }
    }
    k_fl_store<<<fl_blocks((long long)fr0 * D), FL_T, 0, st>>>(flow[0], W, H, D, fwd, bwd, keep_first_bwd);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}
