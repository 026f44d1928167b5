// asv_connect.cu -- 3D connectivity enforcement on the device.
//
// Replaces Image::EnforceLabelConnectivity3D (GPU-AS/Image.cpp:1938-2063,
// called by enforce_connectivity_3d :1808-1837) and Render::label_connected3D
// (streamGPU-AS/Render.cpp:572-695), a sequential raster scan with a flood
// fill per segment.  What the scan computes, restated for a parallel build:
//
//  * segments are the connected components of equal input label under the
//    24-neighbourhood (slices z-1, z, z+1 x the 8 in-plane offsets; the
//    voxel straight above or below is not a neighbour);
//  * segments are numbered in the raster order of their first voxel (the
//    scan's seed), which is the component's smallest voxel index;
//  * a segment of fewer than supsz / 4 voxels takes the label `adj` read at
//    its seed: the label, at that moment, of the last neighbour of the seed
//    (in the reference's loop order) that belongs to an earlier segment; if
//    none does, `adj` keeps the value of the previous segment's scan (0 at
//    the start).  Other segments get consecutive labels.
//
// Build: union-find over voxels (each voxel links to its 12 earlier
// neighbours of equal label; the smaller root always wins, so the root of a
// component is its smallest index = the scan's seed), root compaction by a
// chunked prefix scan, per-root `adj` from the seed's neighbours, and the
// labels of merged segments resolved by pointer jumping over two node kinds:
// F_j (the label of segment j) and A_j (the scan's `adj` after segment j).
// Compiled with -fmad=false (integer work only).
#include "asv_connect.cuh"

#define CC_CHUNK 2048
#define CC_THREADS 256
#define CC_SPIN_LIMIT (1 << 24)     // retry bound of a union / find; exceeding it flags an error

__constant__ int c_dx8[8] = { -1, -1, 0, 1, 1, 1, 0, -1 };
__constant__ int c_dy8[8] = { 0, -1, -1, -1, 0, 1, 1, 1 };

// Root of x with path halving (reads bypass L1: parents change while the
// union kernel runs).  Only non-roots are rewritten, and only to one of
// their ancestors, which stays correct under concurrent links: a root's
// parent changes only through the CAS in cc_union, and a non-root never
// becomes a root again.
__device__ __forceinline__ int cc_find(int *par, int x, int *err)
{
    for (int it = 0; it < CC_SPIN_LIMIT; it++) {
        const int p = __ldcg(par + x);
        if (p == x) return x;
        const int gp = __ldcg(par + p);
        if (gp != p) par[x] = gp;
        x = gp;
    }
    atomicOr(err, 1);
    return x;
}

// links the larger root under the smaller; retries when another thread
// re-linked the root first (each failed CAS means another link succeeded)
__device__ __forceinline__ void cc_union(int *par, int a, int b, int *err)
{
    for (int it = 0; it < CC_SPIN_LIMIT; it++) {
        a = cc_find(par, a, err);
        b = cc_find(par, b, err);
        if (a == b) return;
        if (a > b) { const int t = a; a = b; b = t; }
        const int old = atomicCAS(par + b, b, a);
        if (old == b) return;
        b = old;
    }
    atomicOr(err, 1);
}

__global__ void k_cc_init(int *par, int *cnt, long long n)
{
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    par[v] = (int)v;
    cnt[v] = 0;
}

// union with the earlier half of the 24-neighbourhood: slice z-1 (8 offsets)
// and, in slice z, (-1,0) (-1,-1) (0,-1) (1,-1)
__global__ void k_cc_union(const int32_t *__restrict__ lab, int *par, int W, int H, int D, int *err)
{
    const long long sl = (long long)W * H, n = sl * D;
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const int x = (int)(v % W), y = (int)((v / W) % H), z = (int)(v / sl);
    const int l = lab[v];
    if (z > 0) {
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const int xx = x + c_dx8[k], yy = y + c_dy8[k];
            if (xx < 0 || xx >= W || yy < 0 || yy >= H) continue;
            const long long u = v - sl + (long long)c_dy8[k] * W + c_dx8[k];
            if (lab[u] == l) cc_union(par, (int)u, (int)v, err);
        }
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {                       // offsets 0..3 of dx8/dy8 are earlier
        const int xx = x + c_dx8[k], yy = y + c_dy8[k];
        if (xx < 0 || xx >= W || yy < 0) continue;
        const long long u = v + (long long)c_dy8[k] * W + c_dx8[k];
        if (lab[u] == l) cc_union(par, (int)u, (int)v, err);
    }
}

// root of x by reading only: after the union kernel no links change, so the
// walk ends at the true root
__device__ __forceinline__ int cc_root(const int *par, int x, int *err)
{
    for (int it = 0; it < CC_SPIN_LIMIT; it++) {
        const int p = __ldcg(par + x);
        if (p == x) return x;
        x = p;
    }
    atomicOr(err, 1);
    return x;
}

// par[v] = root; component sizes at the roots.  Only thread v writes par[v]:
// a path-halving write by another thread could land after it and leave an
// ancestor that is not the root.
__global__ void k_cc_flatten(int *par, int *cnt, long long n, int *err)
{
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const int r = cc_root(par, (int)v, err);
    par[v] = r;
    atomicAdd(cnt + r, 1);
}

// roots per chunk of CC_CHUNK voxels
__global__ void __launch_bounds__(CC_THREADS) k_cc_count(const int *__restrict__ par, long long n, int *chunk)
{
    __shared__ int tot;
    if (threadIdx.x == 0) tot = 0;
    __syncthreads();
    const long long base = (long long)blockIdx.x * CC_CHUNK;
    int c = 0;
    for (int i = threadIdx.x; i < CC_CHUNK; i += CC_THREADS) {
        const long long v = base + i;
        if (v < n && par[v] == (int)v) c++;
    }
    atomicAdd(&tot, c);
    __syncthreads();
    if (threadIdx.x == 0) chunk[blockIdx.x] = tot;
}

// exclusive prefix of chunk[0..m) in place, total in chunk[m] (one block)
__global__ void __launch_bounds__(1024) k_cc_prefix(int *chunk, int m)
{
    __shared__ int part[1024];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int b0 = 0; b0 < m; b0 += 1024) {
        const int i = b0 + threadIdx.x;
        const int v = i < m ? chunk[i] : 0;
        part[threadIdx.x] = v;
        __syncthreads();
        for (int off = 1; off < 1024; off <<= 1) {       // inclusive Hillis-Steele scan
            const int t = threadIdx.x >= off ? part[threadIdx.x - off] : 0;
            __syncthreads();
            part[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < m) chunk[i] = carry + part[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry += part[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0) chunk[m] = carry;
}

// compact ids of the roots in raster order: rvox[id] = root voxel,
// rsize[id] = its size, cid[root] = id (cid overwrites the size array)
__global__ void __launch_bounds__(CC_THREADS) k_cc_compact(const int *__restrict__ par, int *cnt_cid,
                                                           const int *__restrict__ chunk, long long n,
                                                           int *rvox, int *rsize)
{
    __shared__ int wsum[CC_THREADS / 32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = chunk[blockIdx.x];
    __syncthreads();
    const long long base = (long long)blockIdx.x * CC_CHUNK;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int i0 = 0; i0 < CC_CHUNK; i0 += CC_THREADS) {
        const long long v = base + i0 + threadIdx.x;
        const bool root = v < n && par[v] == (int)v;
        const unsigned bal = __ballot_sync(0xffffffffu, root);
        if (lane == 0) wsum[w] = __popc(bal);
        __syncthreads();
        int before = carry;
        for (int k = 0; k < w; k++) before += wsum[k];
        if (root) {
            const int id = before + __popc(bal & ((1u << lane) - 1u));
            rvox[id] = (int)v;
            rsize[id] = cnt_cid[v];
            cnt_cid[v] = id;
        }
        __syncthreads();
        if (threadIdx.x == 0) for (int k = 0; k < CC_THREADS / 32; k++) carry += wsum[k];
        __syncthreads();
    }
}

// kept flag per segment, into chunk-sized groups for the rank scan
__global__ void __launch_bounds__(CC_THREADS) k_cc_kept_count(const int *__restrict__ rsize, const int *R,
                                                              int minsz, int *chunk)
{
    __shared__ int tot;
    if (threadIdx.x == 0) tot = 0;
    __syncthreads();
    const int base = blockIdx.x * CC_CHUNK, r = *R;
    int c = 0;
    for (int i = threadIdx.x; i < CC_CHUNK; i += CC_THREADS) {
        const int j = base + i;
        if (j < r && rsize[j] >= minsz) c++;
    }
    atomicAdd(&tot, c);
    __syncthreads();
    if (threadIdx.x == 0) chunk[blockIdx.x] = tot;
}

// Per segment j: its node F_j and the scan's node A_j.  node encoding:
// >= 0 pointer to a node (F_j = j, A_j = R + j), < 0 final value -1 - v.
__global__ void __launch_bounds__(CC_THREADS) k_cc_nodes(const int *__restrict__ par, const int *__restrict__ cid,
                                                         const int *__restrict__ rvox,
                                                         const int *__restrict__ rsize,
                                                         const int *__restrict__ chunk, const int *R, int minsz,
                                                         int W, int H, int D, int *node)
{
    __shared__ int wsum[CC_THREADS / 32];
    __shared__ int carry;
    const int r = *R;
    if (threadIdx.x == 0) carry = chunk[blockIdx.x];
    __syncthreads();
    const int base = blockIdx.x * CC_CHUNK;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const long long sl = (long long)W * H;
    for (int i0 = 0; i0 < CC_CHUNK; i0 += CC_THREADS) {
        const int j = base + i0 + threadIdx.x;
        const bool kept = j < r && rsize[j] >= minsz;
        const unsigned bal = __ballot_sync(0xffffffffu, kept);
        if (lane == 0) wsum[w] = __popc(bal);
        __syncthreads();
        int before = carry;
        for (int k = 0; k < w; k++) before += wsum[k];
        if (j < r) {
            const int s = rvox[j];
            if (kept) node[j] = -1 - (before + __popc(bal & ((1u << lane) - 1u)));   // its label
            else node[j] = r + j;                                                    // = A_j
            // the scan of segment j: last neighbour of the seed in an earlier segment
            const int x = (int)(s % W), y = (int)((s / W) % H), z = (int)(s / sl);
            int adj = -1;
            for (int dz = -1; dz <= 1; dz++) {
                const int zz = z + dz;
                if (zz < 0 || zz >= D) continue;
                for (int k = 0; k < 8; k++) {
                    const int xx = x + c_dx8[k], yy = y + c_dy8[k];
                    if (xx < 0 || xx >= W || yy < 0 || yy >= H) continue;
                    const int root = par[(long long)zz * sl + (long long)yy * W + xx];
                    if (root < s) adj = root;
                }
            }
            if (adj >= 0) node[r + j] = cid[adj];        // A_j -> F of that segment
            else if (j > 0) node[r + j] = r + j - 1;     // A_j -> A_{j-1}
            else node[r + j] = -1;                       // initial value 0
        }
        __syncthreads();
        if (threadIdx.x == 0) for (int k = 0; k < CC_THREADS / 32; k++) carry += wsum[k];
        __syncthreads();
    }
}

// one pointer-jumping round over the 2R nodes (chains point to smaller
// segments, so log2(2R) + 1 rounds resolve every node)
__global__ void k_cc_jump(int *node, const int *R)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 2LL * *R) return;
    const int p = node[t];
    if (p < 0) return;
    node[t] = node[p];
}

__global__ void k_cc_output(const int *__restrict__ par, const int *__restrict__ cid,
                            const int *__restrict__ node, long long n, int32_t *out)
{
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const int f = node[cid[par[v]]];
    out[v] = f < 0 ? -1 - f : 0x7fffffff;                // unresolved cannot happen; marked if it does
}

size_t asv_connect_scratch_bytes(long long n)
{
    const long long chunks = (n + CC_CHUNK - 1) / CC_CHUNK;
    // par, cid/size, rvox, rsize, node (2 per segment), chunk sums (+1), R, error word
    return (size_t)(4 * n * 6 + 4 * (chunks + 2) + 256 * 8);
}

static int *carve(unsigned char *&p, long long count)
{
    int *r = (int *)p;
    p += ((size_t)count * 4 + 255) & ~(size_t)255;
    return r;
}

int asv_launch_connect(const int32_t *lab, int W, int H, int D, int supsz, int32_t *out, void *scratch,
                       cudaStream_t st, int *host_R, int *host_num)
{
    const long long n = (long long)W * H * D;
    const long long chunks = (n + CC_CHUNK - 1) / CC_CHUNK;
    unsigned char *p = (unsigned char *)scratch;
    int *par = carve(p, n), *cid = carve(p, n), *rvox = carve(p, n), *rsize = carve(p, n);
    int *node = carve(p, 2 * n), *chunk = carve(p, chunks + 1), *meta = carve(p, 4);
    const int minsz = supsz / 4;
    const int blocks = (int)((n + CC_THREADS - 1) / CC_THREADS);
    cudaMemsetAsync(meta, 0, 16, st);
    k_cc_init<<<blocks, CC_THREADS, 0, st>>>(par, cid, n);
    k_cc_union<<<blocks, CC_THREADS, 0, st>>>(lab, par, W, H, D, meta + 1);
    k_cc_flatten<<<blocks, CC_THREADS, 0, st>>>(par, cid, n, meta + 1);
    k_cc_count<<<(int)chunks, CC_THREADS, 0, st>>>(par, n, chunk);
    k_cc_prefix<<<1, 1024, 0, st>>>(chunk, (int)chunks);
    k_cc_compact<<<(int)chunks, CC_THREADS, 0, st>>>(par, cid, chunk, n, rvox, rsize);
    cudaMemcpyAsync(meta, chunk + chunks, sizeof(int), cudaMemcpyDeviceToDevice, st);    // R
    int R = 0, err = 0;
    cudaMemcpyAsync(&R, meta, sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&err, meta + 1, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
    if (err) return -2;
    if (R > (1 << 30)) return -3;                        // node ids (2 per segment) are int
    const int rchunks = (R + CC_CHUNK - 1) / CC_CHUNK;
    if (R > 0) {
        k_cc_kept_count<<<rchunks, CC_THREADS, 0, st>>>(rsize, meta, minsz, chunk);
        k_cc_prefix<<<1, 1024, 0, st>>>(chunk, rchunks);
        k_cc_nodes<<<rchunks, CC_THREADS, 0, st>>>(par, cid, rvox, rsize, chunk, meta, minsz, W, H, D, node);
        int rounds = 1;
        while ((1LL << (rounds - 1)) < 2LL * R) rounds++;
        const int jb = (int)((2LL * R + CC_THREADS - 1) / CC_THREADS);
        for (int k = 0; k < rounds; k++) k_cc_jump<<<jb, CC_THREADS, 0, st>>>(node, meta);
        k_cc_output<<<blocks, CC_THREADS, 0, st>>>(par, cid, node, n, out);
    }
    int num = 0;
    cudaMemcpyAsync(&num, chunk + rchunks, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return -1;
    if (cudaGetLastError() != cudaSuccess) return -1;
    *host_R = R;
    *host_num = R > 0 ? num : 0;
    return 0;
}
