// asv_metric.cu -- per-seed anisotropic metric tensor from the flow field.
//
// Replaces the reference's CPU solve (GPU-AS/Image.cpp:689-1009 seed_matrix /
// matrix_slover, :1300-1534 Ld_next_seeds_matrix) and its GPU->CPU->GPU
// round trip every Lloyd iteration.  For each seed, the 3x3 neighbourhood of
// its voxel gives up to 18 rows d^T M d = b (forward rows d = (dx, dy, 1),
// backward rows d = (dx, dy, -1), b = n^2 + m^2 + 1); M is the min-norm
// least-squares solution in FP32 like the reference's Eigen float solve
// (one-sided Jacobi SVD, rank rule of Eigen's SVD solve: keep
// sigma >= max(sigma_max * min(rows,6) * FLT_EPSILON, FLT_MIN)); the 3x3
// PSD test is exact (principal minors, error-free FP64 expansion) and the
// nearest-PSD projection runs in FP64.  A non-PSD M falls back to the mean of
// the PSD metrics of the 1-ring, then 2-ring neighbours, then to the nearest
// PSD matrix.
//
// One warp per solve: lane i holds row i of the system; column dot products
// are butterfly sums over the lanes (asv_lane_sum), which leave the same bits
// on every lane, so all lanes apply the same rotations.
// Launches: k_metric_self (a warp per seed), k_metric_psd (a thread per
// solve: the FP64 PSD tests), k_metric_ring (a warp per seed and neighbour,
// only for non-PSD seeds), k_metric_psd again, k_metric_combine (a thread per
// seed).  A reseed solve is skipped when the seed's voxel is the one of its
// previous reseed solve in this Lloyd run: the metric is a function of that
// voxel and the flow only, so the stored result is the solve's result.
// Compiled with -fmad=false.
#include "asv_common.cuh"

#include <float.h>

#define SVD_SWEEPS 30
#define FULL 0xffffffffu

// Sum of a per-lane value over the warp as a butterfly: at each level a lane
// adds its partner's partial sum (lane ^ 16, 8, 4, 2, 1) to its own.  Both
// partners add the same two operands and IEEE addition commutes, so every
// lane ends with the same bits: slot i takes t[i] + t[i + off] for
// off = 16, 8, 4, 2, 1 over the 32 slots (rows 0..m-1, then +0), the order
// the oracle restates.  Lanes at or beyond m hold +0 (their rows are zero).
__device__ __forceinline__ float asv_lane_sum(float v)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = v + __shfl_xor_sync(FULL, v, off);
    return v;
}

// min-norm least squares in FP32; u = this lane's row (zero beyond m),
// bl = its rhs.  Returns x[0..5] on every lane.
__device__ void asv_lsq_minnorm_warp(int m, float u[6], float bl, float x[6])
{
    const int lane = threadIdx.x & 31;
    float v[6];
#pragma unroll
    for (int c = 0; c < 6; c++) v[c] = lane == c ? 1.0f : 0.0f;   // lane r < 6 holds row r of V
    for (int sw = 0; sw < SVD_SWEEPS; sw++) {
        int rot = 0;
#pragma unroll
        for (int p = 0; p < 5; p++)
#pragma unroll
            for (int q = p + 1; q < 6; q++) {
                const float al = asv_lane_sum(u[p] * u[p]);
                const float be = asv_lane_sum(u[q] * u[q]);
                const float ga = asv_lane_sum(u[p] * u[q]);
                if (ga == 0.0f) continue;
                if (fabsf(ga) <= FLT_EPSILON * sqrtf(al * be)) continue;
                float zeta = (be - al) / (2.0f * ga);
                float t = 1.0f / (fabsf(zeta) + sqrtf(1.0f + zeta * zeta));
                if (zeta < 0.0f) t = -t;
                float c = 1.0f / sqrtf(1.0f + t * t);
                float s = c * t;
                float up = u[p], uq = u[q];
                u[p] = c * up - s * uq;
                u[q] = s * up + c * uq;
                float vp = v[p], vq = v[q];
                v[p] = c * vp - s * vq;
                v[q] = s * vp + c * vq;
                rot++;
            }
        if (!rot) break;
    }
    float sig[6], smax = 0.0f;
#pragma unroll
    for (int j = 0; j < 6; j++) {
        sig[j] = sqrtf(asv_lane_sum(u[j] * u[j]));
        if (sig[j] > smax) smax = sig[j];
    }
    float thr = smax * ((float)(m < 6 ? m : 6) * FLT_EPSILON);
    if (thr < FLT_MIN) thr = FLT_MIN;
    float xr = 0.0f;   // lane r < 6 accumulates x[r]
#pragma unroll
    for (int j = 0; j < 6; j++) {
        if (!(sig[j] >= thr)) continue;
        float ub = asv_lane_sum(u[j] * bl);
        float coef = (ub / sig[j]) / sig[j];
        xr = xr + v[j] * coef;
    }
#pragma unroll
    for (int r = 0; r < 6; r++) x[r] = __shfl_sync(FULL, xr, r);
}

// symmetric 3x3 eigen-decomposition, cyclic Jacobi
__device__ void asv_sym3_eig(const float M[6], double w[3], double V[3][3])
{
    double a[3][3] = { { M[0], M[1], M[2] }, { M[1], M[3], M[4] }, { M[2], M[4], M[5] } };
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) V[r][c] = r == c ? 1.0 : 0.0;
    const int P[3] = { 0, 0, 1 }, Q[3] = { 1, 2, 2 };
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

// error-free transformations (Knuth's TwoSum, the FMA TwoProduct)
__device__ __forceinline__ void asv_two_sum(double a, double b, double &s, double &e)
{
    s = a + b;
    const double bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ void asv_two_prod(double a, double b, double &p, double &e)
{
    p = a * b;
    e = fma(a, b, -p);
}

// Exact "some eigenvalue is negative" test of the symmetric 3x3 matrix M
// (GPU-AS/Image.cpp:997-1006 asks eigenvalues() for a real part < 0): a
// symmetric matrix has no negative eigenvalue iff all its principal minors
// are >= 0.  Products of two floats are exact in double; the determinant's
// five triple products are split into exact (hi, lo) pairs and summed as a
// nonoverlapping expansion (Shewchuk's Grow-Expansion), whose last non-zero
// component carries the exact sign.  Entries that are not finite count as
// no negative eigenvalue.
__device__ int asv_m6_negative(const float M[6])
{
    const double a = M[0], b = M[1], c = M[2], d = M[3], e = M[4], f = M[5];
    if (!(isfinite(a) && isfinite(b) && isfinite(c) && isfinite(d) && isfinite(e) && isfinite(f)))
        return 0;
    if (a < 0.0 || d < 0.0 || f < 0.0) return 1;
    if (a * d < b * b || a * f < c * c || d * f < e * e) return 1;
    double t[10];
    asv_two_prod(a * d, f, t[0], t[1]);                 // a d f
    asv_two_prod(2.0 * (b * c), e, t[2], t[3]);         // 2 b c e
    asv_two_prod(-(a * e), e, t[4], t[5]);              // - a e e
    asv_two_prod(-(d * c), c, t[6], t[7]);              // - d c c
    asv_two_prod(-(f * b), b, t[8], t[9]);              // - f b b
    double x[10];
    int n = 0;
    for (int k = 0; k < 10; k++) {                      // Grow-Expansion
        double q = t[k];
        for (int i = 0; i < n; i++) {
            double h;
            asv_two_sum(q, x[i], q, h);
            x[i] = h;
        }
        x[n++] = q;
    }
    for (int i = n - 1; i >= 0; i--)
        if (x[i] != 0.0) return x[i] < 0.0 ? 1 : 0;
    return 0;
}

__device__ void asv_m6_nearest_psd(const float M[6], float out[6])
{
    double w[3], V[3][3];
    asv_sym3_eig(M, w, V);
    for (int k = 0; k < 3; k++) if (w[k] < 0.0) w[k] = 0.0;
    const int R[6] = { 0, 0, 0, 1, 1, 2 }, C[6] = { 0, 1, 2, 1, 2, 2 };
    for (int e = 0; e < 6; e++) {
        int i = R[e], j = C[e];
        double acc = (V[i][0] * w[0]) * V[j][0];
        acc = acc + (V[i][1] * w[1]) * V[j][1];
        acc = acc + (V[i][2] * w[2]) * V[j][2];
        out[e] = (float)acc;
    }
}

// floor(f + 0.5) of the reference's round (GPU-AS/Image.cpp:901), exactly:
// f + 0.5 can round in FP32, but f - floorf(f) cannot change which side of
// 0.5 the fraction lies on, and the result is the reference's value for every
// float (the +0.0f turns the -0 of f = -0 into +0, as floor(-0 + 0.5) is +0).
__device__ __forceinline__ float asv_round_half_up(float f)
{
    const float r = floorf(f);
    return (f - r >= 0.5f ? r + 1.0f : r) + 0.0f;
}

// matrix_slover (GPU-AS/Image.cpp:874-1009) for one warp; M valid on every
// lane (its PSD test, :997-1006, is k_metric_psd).  Rows are numbered in the
// reference's order (neighbour y outer, x inner; forward row, then backward).
__device__ void asv_metric_solve_warp(const float2 *__restrict__ fwd, const float2 *__restrict__ bwd,
                                      int W, int H, int D, float sx, float sy, int frame, float M[6])
{
    const int lane = threadIdx.x & 31;
    // rows: each in-bounds neighbour in order gives a forward row (unless
    // the last frame) then a backward row (unless the first frame); lane r
    // finds its row's neighbour and direction, so all flow reads issue at once
    const bool hf = frame != D - 1, hb = frame != 0;     // D >= 2: at least one
    const int per = (int)hf + (int)hb;
    unsigned inb = 0;
#pragma unroll
    for (int k = 0; k < 9; k++) {
        const int nx = (int)sx + (k % 3 - 1), ny = (int)sy + (k / 3 - 1);
        if (nx >= 0 && nx < W && ny >= 0 && ny < H) inb |= 1u << k;
    }
    const int m = per * __popc(inb);
    float u[6] = { 0, 0, 0, 0, 0, 0 }, bl = 0.0f;
    if (lane < m) {
        const int j = per == 2 ? lane >> 1 : lane;
        const bool back = per == 2 ? (lane & 1) != 0 : hb;
        unsigned rest = inb;
        for (int k = 0; k < j; k++) rest &= rest - 1;    // drop the j lower neighbours
        const int id_b = __ffs(rest) - 1;
        const int ox = id_b % 3 - 1, oy = id_b / 3 - 1;
        const long long o = ((long long)frame * H + ((int)sy + oy)) * W + ((int)sx + ox);
        const float2 f = __ldg((back ? bwd : fwd) + o);
        if (!back) {
            float dx = (float)ox + asv_round_half_up(f.x);
            float dy = (float)oy + asv_round_half_up(f.y);
            u[0] = dx * dx; u[1] = 2.0f * dx * dy;
            u[2] = 2.0f * dx; u[3] = dy * dy;
            u[4] = 2.0f * dy; u[5] = 1.0f;
        } else {
            float dx = asv_round_half_up(f.x) + (float)ox;
            float dy = asv_round_half_up(f.y) + (float)oy;
            u[0] = dx * dx; u[1] = 2.0f * dx * dy;
            u[2] = -2.0f * dx; u[3] = dy * dy;
            u[4] = -2.0f * dy; u[5] = 1.0f;
        }
        bl = (float)(ox * ox + oy * oy + 1);             // expected_b of :884: 3 2 3 / 2 1 2 / 3 2 3
    }
    float x[6];
    if (m == 0) {
        for (int k = 0; k < 6; k++) x[k] = 0.0f;
    } else {
        asv_lsq_minnorm_warp(m, u, bl, x);
    }
    for (int k = 0; k < 6; k++) M[k] = x[k];
}

// plain reseed flow-angle filter (GPU-AS/Image.cpp:1406-1409): accept iff
// the float cosine c satisfies T <= c <= 1, T the smallest float with
// float(double(acosf(T)) * (180 / 3.141592653)) < 90 (bits 0x328885a3).
// The last frame's flow is the reference's 4x4 zero Mat: read as zero.
__device__ int asv_angle_ok(const float2 *__restrict__ fwd, int W, int H, int D, int frame, int sx,
                            int sy, int nx, int ny)
{
    float sfx = 0.0f, sfy = 0.0f, nfx = 0.0f, nfy = 0.0f;
    if (frame != D - 1) {
        sx = min(max(sx, 0), W - 1);
        sy = min(max(sy, 0), H - 1);
        float2 a = __ldg(fwd + ((long long)frame * H + sy) * W + sx);
        float2 c = __ldg(fwd + ((long long)frame * H + ny) * W + nx);
        sfx = a.x; sfy = a.y; nfx = c.x; nfy = c.y;
    }
    float num = sfx * nfx + sfy * nfy;
    double den = sqrt((double)sfx * (double)sfx + (double)sfy * (double)sfy) *
                 sqrt((double)nfx * (double)nfx + (double)nfy * (double)nfy);
    float c = (float)((double)num / den);
    return (c >= 1.5893254712295857e-08f && c <= 1.0f) ? 1 : 0;
}

__constant__ int c_ringx[ASV_RING] = { -1, 0, 1, -1, 1, -1, 0, 1,
                                       -2, -1, 0, 1, 2, -2, 2, -2, 2, -2, 2, -2, -1, 0, 1, 2 };
__constant__ int c_ringy[ASV_RING] = { -1, -1, -1, 0, 0, 1, 1, 1,
                                       -2, -2, -2, -2, -2, -1, -1, 0, 0, 1, 1, 2, 2, 2, 2, 2 };

struct SeedRef { int si, i, g; };

__device__ __forceinline__ bool asv_seed_ref(const AsvDev &d, int g, SeedRef &r)
{
    if (g >= d.total_seeds) return false;
    r.g = g;
    r.si = asv_find_seg(d.seed_prefix, d.nseg, g);
    r.i = g - d.seed_prefix[r.si];
    return r.i < d.segs[r.si].Kp;
}

// voxel key of a seed position (the memo key of the reseed solve)
__device__ __forceinline__ int asv_seed_key(const SegDesc &S, float4 p)
{
    int frame = min(max((int)p.z, 0), S.D - 1);
    int x = min(max((int)floorf(p.x), 0), S.W - 1), y = min(max((int)floorf(p.y), 0), S.H - 1);
    return (frame * S.H + y) * S.W + x;
}

// neg[g]: 0 = PSD, 1 = non-PSD (fallbacks run), 2 = memo hit (reseed only),
// 3 = solved, PSD test pending (k_metric_psd).  Which seed positions:
// reseed 0 -> pos0 (seed_matrix), 1 -> pos (reseed).
__global__ void __launch_bounds__(128) k_metric_self(AsvDev d, int reseed)
{
    const int lane = threadIdx.x & 31;
    SeedRef r;
    if (!asv_seed_ref(d, (blockIdx.x * blockDim.x + threadIdx.x) >> 5, r)) return;   // warp-uniform
    const SegDesc &S = d.segs[r.si];
    float4 p = reseed ? d.pos[r.g] : d.pos0[r.g];
    if (reseed && d.mkey[r.g] == asv_seed_key(S, p)) {
        if (lane == 0) d.neg[r.g] = 2;
        return;
    }
    float fx = floorf(p.x), fy = floorf(p.y);
    int frame = min(max((int)p.z, 0), S.D - 1);   // positions are inside; keep reads in bounds
    float M[6];
    asv_metric_solve_warp(d.fwd + S.vox_off, d.bwd + S.vox_off, S.W, S.H, S.D, fx, fy, frame, M);
    if (lane < 6) d.Mself[8 * r.g + lane] = M[lane];
    if (lane == 0) d.neg[r.g] = 3;
}

// The FP64 PSD tests of the solves, one thread per solve: the warp solves
// leave them pending so that each 3x3 eigen-decomposition runs on one lane
// of a full warp instead of on all 32 lanes of the solving warp (GB300's FP64
// pipe is narrow).  flag 3 (self) / 2 (ring) marks a pending test.
__global__ void k_metric_psd(AsvDev d)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long nself = d.total_seeds;
    SeedRef r;
    if (t < nself) {
        if (asv_seed_ref(d, (int)t, r) && d.neg[t] == 3) d.neg[t] = asv_m6_negative(d.Mself + 8 * t);
        return;
    }
    const long long k = t - nself;                       // ring task: seed * ASV_RING + neighbour
    if (k >= nself * ASV_RING || !asv_seed_ref(d, (int)(k / ASV_RING), r)) return;
    if (d.ringok[k] == 2) d.ringok[k] = asv_m6_negative(d.Mring + 8 * k) ? 0 : 1;
}

__global__ void __launch_bounds__(128) k_metric_ring(AsvDev d, int reseed)
{
    const int lane = threadIdx.x & 31;
    int task = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int g = task / ASV_RING, t = task - g * ASV_RING;
    SeedRef r;
    if (!asv_seed_ref(d, g, r)) return;
    int *ok = d.ringok + ASV_RING * g + t;
    if (d.neg[g] != 1) { if (lane == 0) *ok = 0; return; }
    const SegDesc &S = d.segs[r.si];
    float4 p = reseed ? d.pos[g] : d.pos0[g];
    float fx = floorf(p.x), fy = floorf(p.y);
    int frame = min(max((int)p.z, 0), S.D - 1);
    float nx = fx + (float)c_ringx[t], ny = fy + (float)c_ringy[t];
    if (!(nx >= 0 && nx < S.W && ny >= 0 && ny < S.H)) { if (lane == 0) *ok = 0; return; }
    const float2 *fwd = d.fwd + S.vox_off, *bwd = d.bwd + S.vox_off;
    if (reseed && S.angle_filter &&
        !asv_angle_ok(fwd, S.W, S.H, S.D, frame, (int)fx, (int)fy, (int)nx, (int)ny)) {
        if (lane == 0) *ok = 0;
        return;
    }
    float M[6];
    asv_metric_solve_warp(fwd, bwd, S.W, S.H, S.D, nx, ny, frame, M);
    float *dst = d.Mring + 8 * (ASV_RING * g + t);
    if (lane < 6) dst[lane] = M[lane];
    if (lane == 0) *ok = 2;                              // PSD test pending (k_metric_psd)
}

// writes M0 (reseed 0) or M (reseed 1, and the memo)
__global__ void k_metric_combine(AsvDev d, int reseed)
{
    SeedRef r;
    if (!asv_seed_ref(d, blockIdx.x * blockDim.x + threadIdx.x, r)) return;
    const int g = r.g;
    float *out = (reseed ? d.M : d.M0) + 8 * g;
    const int neg = d.neg[g];
    if (neg == 2) {
        for (int e = 0; e < 6; e++) out[e] = d.Mmemo[8 * g + e];
        return;
    }
    float res[6];
    float self[6];
    for (int e = 0; e < 6; e++) self[e] = d.Mself[8 * g + e];
    bool done = false;
    if (!neg) {
        for (int e = 0; e < 6; e++) res[e] = self[e];
        done = true;
    }
    for (int ring = 0; ring < 2 && !done; ring++) {
        int t0 = ring == 0 ? 0 : 8, t1 = ring == 0 ? 8 : ASV_RING;
        float sum[6] = { 0, 0, 0, 0, 0, 0 };
        int n = 0;
        for (int t = t0; t < t1; t++) {
            if (!d.ringok[ASV_RING * g + t]) continue;
            const float *m = d.Mring + 8 * (ASV_RING * g + t);
            n++;
            for (int e = 0; e < 6; e++) sum[e] = sum[e] + m[e];
        }
        if (n > 0) {
            for (int e = 0; e < 6; e++) res[e] = sum[e] / (float)n;
            done = true;
        }
    }
    if (!done) asv_m6_nearest_psd(self, res);
    for (int e = 0; e < 6; e++) out[e] = res[e];
    if (reseed) {
        for (int e = 0; e < 6; e++) d.Mmemo[8 * g + e] = res[e];
        d.mkey[g] = asv_seed_key(d.segs[r.si], d.pos[g]);
    }
}

void asv_launch_metric(const AsvDev &d, int reseed, cudaStream_t st)
{
    long long warps = d.total_seeds;
    k_metric_self<<<(int)((warps * 32 + 127) / 128), 128, 0, st>>>(d, reseed);
    long long rw = (long long)d.total_seeds * ASV_RING;
    k_metric_psd<<<(int)((warps + 127) / 128), 128, 0, st>>>(d);     // self tests
    k_metric_ring<<<(int)((rw * 32 + 127) / 128), 128, 0, st>>>(d, reseed);
    k_metric_psd<<<(int)((warps + rw + 127) / 128), 128, 0, st>>>(d); // ring tests
    k_metric_combine<<<(d.total_seeds + 63) / 64, 64, 0, st>>>(d, reseed);
}
