// asv_noalloc.cu -- check_dead_seeds post-processing over caller-owned
// device buffers, with no device allocation at all.
//
// Some hosts of this library cannot let it call cudaMalloc: a media
// pipeline or inference server that hands every byte of device memory out
// of its own pool (and audits that nothing else allocates), or a
// latency-bound stage where cudaMalloc/cudaFree would synchronize the device
// in the middle of other work.  For them this entry point takes a raw label
// volume and writes the post-processed one, using as scratch a fixed array
// that lives in the library's own device image: it is allocated when the
// library is loaded on a device and held until the process exits.
//
// The scratch is shared by every call on a device and keeps the last call's
// contents; the per-label counts are cleared at the start of each call, the
// other regions are fully rewritten before they are read.  Calls whose work
// overlaps on the GPU (different streams, or host threads without ordering)
// race on the scratch and must be serialized by the caller.
//
// The semantics are those of asv_check_dead_seeds (GPU-AS/Image.cpp:
// 1579-1778): count the voxels of each label, then relabel dead seeds
// (<= 3 dead: label_replace.gs in order; > 3: sequence_label's raster remap)
// and forward-fill label -1.  A label outside [-1, Kp) (which the JFA never
// writes) is read as -1 by every stage: counted in the -1 slot and filled.
#include "asv.h"

#include <cuda_runtime.h>

#include <mutex>

#define NA_CHUNK 2048
#define NA_FULL 0xffffffffu
#define NA_MAX_VOXELS (1LL << 25)
#define NA_MAX_SEEDS 32767
#define NA_MAX_CHUNKS (int)(NA_MAX_VOXELS / NA_CHUNK)

// scratch regions (bytes): counts (Kp+1 u32), rank (Kp i32), record, scan carries
#define NA_OFF_COUNTS 0
#define NA_OFF_RANK (NA_OFF_COUNTS + 4 * (NA_MAX_SEEDS + 1))
#define NA_OFF_REC (((NA_OFF_RANK + 4 * NA_MAX_SEEDS) + 255) & ~255)
#define NA_OFF_SCAN (NA_OFF_REC + 256)
#define NA_SCRATCH_BYTES (NA_OFF_SCAN + 4 * NA_MAX_CHUNKS)

static __device__ __align__(256) unsigned char g_asv_noalloc_scratch[NA_SCRATCH_BYTES];

enum { R_DEAD = 0, R_MODE = 1, R_INVALID = 2, R_L0 = 3, R_M0 = 4, R_DEAD0 = 5 };

struct NaScratch {
    unsigned int *counts;
    int *rank;
    int *rec;
    int *scan;
};

// a raw label as every stage reads it: outside [-1, Kp) -> -1
static __device__ __forceinline__ int na_label(const int32_t *__restrict__ raw, long long v, int Kp)
{
    const int l = raw[v];
    return (l >= 0 && l < Kp) ? l : -1;
}

static __device__ __forceinline__ int na_relabel(const int *rec, int Kp, int l)
{
    if (rec[R_MODE] != 1 || l < 0) return l;
    int last = Kp;
    for (int k = 0; k < rec[R_DEAD]; k++) {
        last -= 1;
        if (l == last) l = rec[R_DEAD0 + k];
    }
    return l;
}

static __device__ __forceinline__ long long na_src(const int *rec, int Kp, long long v, int l)
{
    if (rec[R_MODE] == 2) {
        if (v == 0) return 0;
        return (l != rec[R_L0] && l != -1) ? v : -1;
    }
    if (v == 0) return 0;
    return na_relabel(rec, Kp, l) != -1 ? v : -1;
}

static __device__ __forceinline__ bool na_scan_needed(const int *rec)
{
    return rec[R_MODE] == 2 || rec[R_INVALID] != 0;
}

__global__ void __launch_bounds__(256) k_na_count(NaScratch s, const int32_t *__restrict__ raw,
                                                  long long n, int Kp)
{
    for (int i = 0; i < NA_CHUNK / 256; i++) {
        long long v = (long long)blockIdx.x * NA_CHUNK + i * 256 + threadIdx.x;
        int key = -1;
        if (v < n) {
            const int l = na_label(raw, v, Kp);
            key = l < 0 ? Kp : l;
        }
        unsigned grp = __match_any_sync(NA_FULL, key);
        if (key >= 0 && (threadIdx.x & 31) == __ffs(grp) - 1) atomicAdd(s.counts + key, __popc(grp));
    }
}

__global__ void __launch_bounds__(1024) k_na_stats(NaScratch s, const int32_t *__restrict__ raw, int Kp)
{
    __shared__ int warp_tot[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int b0 = 0; b0 < Kp; b0 += blockDim.x) {
        int i = b0 + threadIdx.x;
        int alive = (i < Kp && s.counts[i] >= 1) ? 1 : 0;
        unsigned bal = __ballot_sync(NA_FULL, alive);
        int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        int pre = __popc(bal & ((1u << lane) - 1u));
        if (lane == 0) warp_tot[w] = __popc(bal);
        __syncthreads();
        if (threadIdx.x < 32) {
            int v = warp_tot[threadIdx.x];
            int incl = v;
            for (int o = 1; o < 32; o <<= 1) {
                int m = __shfl_up_sync(NA_FULL, incl, o);
                if (threadIdx.x >= o) incl += m;
            }
            warp_tot[threadIdx.x] = incl - v;
        }
        __syncthreads();
        if (i < Kp) {
            const int live_before = carry + warp_tot[w] + pre;
            s.rank[i] = alive ? live_before : -1;
            const int dead_before = i - live_before;        // the first four dead seeds, in order
            if (!alive && dead_before < 4) s.rec[R_DEAD0 + dead_before] = i;
        }
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry += warp_tot[w] + pre + alive;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        int dead = Kp - carry;
        s.rec[R_DEAD] = dead;
        s.rec[R_MODE] = dead == 0 ? 0 : (dead <= 3 ? 1 : 2);
        s.rec[R_INVALID] = s.counts[Kp] > 0 ? 1 : 0;
        const int l0 = na_label(raw, 0, Kp);
        s.rec[R_L0] = l0;
        s.rec[R_M0] = (l0 >= 0 && s.rank[l0] >= 0) ? s.rank[l0] : 0;
    }
}

__global__ void __launch_bounds__(256) k_na_chunk_max(NaScratch s, const int32_t *__restrict__ raw,
                                                      long long n, int Kp)
{
    if (!na_scan_needed(s.rec)) return;
    long long m = -1;
    for (int i = 0; i < NA_CHUNK / 256; i++) {
        long long v = (long long)blockIdx.x * NA_CHUNK + i * 256 + threadIdx.x;
        if (v < n) { long long q = na_src(s.rec, Kp, v, na_label(raw, v, Kp)); if (q > m) m = q; }
    }
    for (int o = 16; o; o >>= 1) { long long q = __shfl_xor_sync(NA_FULL, m, o); if (q > m) m = q; }
    __shared__ long long wm[8];
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long r = wm[0];
        for (int k = 1; k < 8; k++) if (wm[k] > r) r = wm[k];
        s.scan[blockIdx.x] = (int)(r + 1);
    }
}

__global__ void __launch_bounds__(1024) k_na_prefix(NaScratch s, int nchunks)
{
    if (!na_scan_needed(s.rec)) return;
    __shared__ int carry;
    __shared__ int wmax[32];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int b0 = 0; b0 < nchunks; b0 += blockDim.x) {
        int c = b0 + threadIdx.x;
        int v = c < nchunks ? s.scan[c] : 0;
        int incl = v;
        int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        for (int o = 1; o < 32; o <<= 1) { int q = __shfl_up_sync(NA_FULL, incl, o); if (lane >= o && q > incl) incl = q; }
        if (lane == 31) wmax[w] = incl;
        __syncthreads();
        if (threadIdx.x < 32) {
            int ix = wmax[threadIdx.x];
            for (int o = 1; o < 32; o <<= 1) { int q = __shfl_up_sync(NA_FULL, ix, o); if (threadIdx.x >= o && q > ix) ix = q; }
            wmax[threadIdx.x] = ix;
        }
        __syncthreads();
        int before = w > 0 ? wmax[w - 1] : 0;
        int ew = __shfl_up_sync(NA_FULL, incl, 1);
        if (lane == 0) ew = 0;
        int ex = max(max(carry, before), ew);
        int tot = max(carry, wmax[31]);
        __syncthreads();
        if (c < nchunks) s.scan[c] = ex;
        if (threadIdx.x == 0) carry = tot;
        __syncthreads();
    }
}

// The chunk's raw labels are staged through shared memory with coalesced
// loads (voxel base + i * 256 + thread), then every thread scans its 8
// consecutive voxels from there; the results go back through shared memory
// and out with coalesced stores.
__global__ void __launch_bounds__(256) k_na_apply(NaScratch s, const int32_t *__restrict__ raw,
                                                  int32_t *__restrict__ out, long long n, int Kp)
{
    __shared__ int32_t tile[NA_CHUNK + NA_CHUNK / 32];      // one pad word per 32: no bank conflicts
    const int *rec = s.rec;
    const bool scan = na_scan_needed(rec);
    const int mode = rec[R_MODE];
    const int per = NA_CHUNK / 256;
    const long long base = (long long)blockIdx.x * NA_CHUNK;
#define NA_PAD(i) ((i) + ((i) >> 5))
    for (int i = 0; i < per; i++) {
        const int k = i * 256 + threadIdx.x;
        tile[NA_PAD(k)] = base + k < n ? na_label(raw, base + k, Kp) : -1;
    }
    __syncthreads();
    const int k0 = threadIdx.x * per;
    const long long v0 = base + k0;
    long long excl = -1;
    if (scan) {
        long long carry = (long long)s.scan[blockIdx.x] - 1;
        long long m = -1;
        for (int k = 0; k < per; k++) {
            long long v = v0 + k;
            if (v < n) { long long q = na_src(rec, Kp, v, tile[NA_PAD(k0 + k)]); if (q > m) m = q; }
        }
        long long incl = m;
        int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        for (int o = 1; o < 32; o <<= 1) { long long q = __shfl_up_sync(NA_FULL, incl, o); if (lane >= o && q > incl) incl = q; }
        __shared__ long long wmx[8];
        if (lane == 31) wmx[w] = incl;
        __syncthreads();
        long long before = -1;
        for (int k = 0; k < w; k++) if (wmx[k] > before) before = wmx[k];
        long long ew = __shfl_up_sync(NA_FULL, incl, 1);
        if (lane == 0) ew = -1;
        excl = max(max(before, ew), carry);
    }
    int res[NA_CHUNK / 256];
    long long src = excl;
    for (int k = 0; k < per; k++) {
        long long v = v0 + k;
        res[k] = -1;
        if (v >= n) continue;
        int l = tile[NA_PAD(k0 + k)];
        int r;
        if (!scan) {
            r = na_relabel(rec, Kp, l);
        } else {
            long long q = na_src(rec, Kp, v, l);
            if (q > src) src = q;
            if (mode == 2) {
                if (src <= 0) r = rec[R_M0];
                else {
                    // the source voxel can lie in an earlier chunk: read it from global memory
                    int ls = src >= base ? tile[NA_PAD((int)(src - base))] : na_label(raw, src, Kp);
                    r = (ls >= 0 && s.rank[ls] >= 0) ? s.rank[ls] : 0;
                }
            } else {
                int rl = na_relabel(rec, Kp, l);
                if (v == 0 || rl != -1) r = rl;
                else if (src >= 1) {
                    int ls = src >= base ? tile[NA_PAD((int)(src - base))] : na_label(raw, src, Kp);
                    r = na_relabel(rec, Kp, ls);
                } else {
                    int r0 = na_relabel(rec, Kp, na_label(raw, 0, Kp));
                    r = r0 >= 0 ? r0 : 0;
                }
            }
        }
        res[k] = r;
    }
    __syncthreads();                                        // every read of the staged labels is done
    for (int k = 0; k < per; k++) tile[NA_PAD(k0 + k)] = res[k];
    __syncthreads();
    for (int i = 0; i < per; i++) {
        const int k = i * 256 + threadIdx.x;
        if (base + k < n) out[base + k] = tile[NA_PAD(k)];
    }
#undef NA_PAD
}

// Device address of the scratch array, resolved once per device (the first
// call on a device makes this runtime call; do that first call before any
// stream capture).  The array's name in host code is only a host-side
// stand-in, never a device address.
static std::mutex g_na_mu;
static void *g_na_ptr[256];

static cudaError_t na_scratch(int dev, void **out)
{
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_na_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_asv_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_na_ptr[dev] = p;
    }
    *out = g_na_ptr[dev];
    return cudaSuccess;
}

extern "C" asv_status asv_check_dead_seeds_noalloc(const int32_t *d_raw, int32_t *d_out, int W, int H,
                                                   int D, int Kp, void *stream)
{
    if (!d_raw || !d_out || W < 1 || H < 1 || D < 1 || Kp < 1) return ASV_ERR_BAD_ARG;
    if ((long long)W * H > NA_MAX_VOXELS || (long long)W * H * D > NA_MAX_VOXELS || Kp > NA_MAX_SEEDS)
        return ASV_ERR_BAD_ARG;
    long long n = (long long)W * H * D;
    // in and out must not overlap: blocks read labels of other chunks (the
    // fill source) while others write theirs
    const uintptr_t r0 = (uintptr_t)d_raw, o0 = (uintptr_t)d_out, nb = 4 * (uintptr_t)n;
    if (r0 < o0 + nb && o0 < r0 + nb) return ASV_ERR_BAD_ARG;
    // an error left pending by earlier work of the caller is returned as
    // ASV_ERR_CUDA and left pending for its owner (not cleared, not mixed
    // with this call's launches)
    if (cudaPeekAtLastError() != cudaSuccess) return ASV_ERR_CUDA;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) { cudaGetLastError(); return ASV_ERR_NO_DEVICE; }
    void *base = nullptr;
    if (na_scratch(dev, &base) != cudaSuccess) { cudaGetLastError(); return ASV_ERR_CUDA; }
    cudaStream_t st = (cudaStream_t)stream;
    unsigned char *b = (unsigned char *)base;
    NaScratch s;
    s.counts = (unsigned int *)(b + NA_OFF_COUNTS);
    s.rank = (int *)(b + NA_OFF_RANK);
    s.rec = (int *)(b + NA_OFF_REC);
    s.scan = (int *)(b + NA_OFF_SCAN);
    int nchunks = (int)((n + NA_CHUNK - 1) / NA_CHUNK);
    if (cudaMemsetAsync(s.counts, 0, sizeof(unsigned int) * (size_t)(Kp + 1), st) != cudaSuccess) {
        cudaGetLastError();
        return ASV_ERR_CUDA;
    }
    k_na_count<<<nchunks, 256, 0, st>>>(s, d_raw, n, Kp);
    k_na_stats<<<1, 1024, 0, st>>>(s, d_raw, Kp);
    k_na_chunk_max<<<nchunks, 256, 0, st>>>(s, d_raw, n, Kp);
    k_na_prefix<<<1, 1024, 0, st>>>(s, nchunks);
    k_na_apply<<<nchunks, 256, 0, st>>>(s, d_raw, d_out, n, Kp);
    if (cudaGetLastError() != cudaSuccess) return ASV_ERR_CUDA;
    return ASV_OK;
}
