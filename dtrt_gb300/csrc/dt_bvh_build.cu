// dtrt_gb300 — BVH build on the device: a linear BVH in the traversal's 2-wide layout.
//
// Replaces the Embree scene build of the reference (src/scene.cpp:17-43). Steps, all on
// one stream:
//   1. per triangle: bounds, centroid; the centroid bounds of the scene (block reduction,
//      one atomic per block on order-preserving integer images of the floats)
//   2. 30-bit Morton code of each centroid in those bounds
//   3. stable LSD radix sort of (code, triangle) pairs, 8 bits per pass: block digit
//      histograms, an exclusive scan of each digit's row (one block per digit) and of the
//      row totals, a scatter whose in-block ranks come from __match_any_sync (so equal
//      digits keep their order)
//   4. the binary radix tree of the sorted codes (one thread per inner node; equal codes
//      are told apart by their sorted position), each node covering a contiguous range
//   5. node boxes bottom-up: one thread per leaf climbs while it is the second child to
//      arrive (arrival counter per node), so every box is written exactly once
//   6. subtrees of at most kLeafMax triangles become leaves (their triangles are already
//      contiguous in sorted order); the remaining inner nodes are compacted by a scan and
//      written as BvhNode (child boxes + child codes), triangles as (v0, id) (e1) (e2)
//      in sorted order — the same records the host builder writes
// A tree deeper than the traversal stack can hold is reported (the caller then builds
// on the host instead).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "dt_bvh.h"
#include "dt_common.cuh"

namespace dt {
namespace {

constexpr int kLeafMax = 4;         // triangles per leaf (3-bit count field allows 8)
constexpr int kSortThreads = 256;   // radix sort block
constexpr int kSortRounds = 8;      // elements per thread per block tile
constexpr int kTile = kSortThreads * kSortRounds;
constexpr int kDigitBits = 8;       // 8-bit digits: 3 passes for the Li and primary-edge sort keys, 4 for Morton codes
constexpr int kDigits = 1 << kDigitBits;
constexpr int kScanThreads = 1024;

// order-preserving unsigned image of a float (for atomicMin / atomicMax)
__device__ __forceinline__ unsigned f2o(float f) {
    const unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ __forceinline__ float o2f(unsigned u) {
    const unsigned v = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
#ifdef __CUDA_ARCH__
    return __uint_as_float(v);
#else
    float f;
    std::memcpy(&f, &v, 4);
    return f;
#endif
}

__device__ __forceinline__ void tri_box(const float *tv, int t, float lo[3], float hi[3]) {
    const float *v = tv + 9 * (size_t)t;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        lo[a] = fminf(v[a], fminf(v[3 + a], v[6 + a]));
        hi[a] = fmaxf(v[a], fmaxf(v[3 + a], v[6 + a]));
    }
}

// 1. centroid bounds: bounds[0..2] = min (ordered images), bounds[3..5] = max
__global__ void k_centroid_bounds(const float *tv, int n, unsigned *bounds) {
    __shared__ unsigned s_lo[3][32], s_hi[3][32];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned lo[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, hi[3] = {0u, 0u, 0u};
    if (i < n) {
        float l[3], h[3];
        tri_box(tv, i, l, h);
        for (int a = 0; a < 3; ++a) lo[a] = hi[a] = f2o(0.5f * (l[a] + h[a]));
    }
    for (int a = 0; a < 3; ++a)
        for (int off = 16; off > 0; off >>= 1) {
            lo[a] = min(lo[a], __shfl_down_sync(0xffffffffu, lo[a], off));
            hi[a] = max(hi[a], __shfl_down_sync(0xffffffffu, hi[a], off));
        }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
        for (int a = 0; a < 3; ++a) { s_lo[a][w] = lo[a]; s_hi[a][w] = hi[a]; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int ww = 1; ww < (int)(blockDim.x >> 5); ++ww)
            for (int a = 0; a < 3; ++a) { lo[a] = min(lo[a], s_lo[a][ww]); hi[a] = max(hi[a], s_hi[a][ww]); }
        for (int a = 0; a < 3; ++a) {
            atomicMin(bounds + a, lo[a]);
            atomicMax(bounds + 3 + a, hi[a]);
        }
    }
}

__device__ __forceinline__ unsigned expand_bits(unsigned v) {  // 10 bits -> every third bit
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

// 2. Morton codes of the centroids
__global__ void k_morton(const float *tv, int n, const unsigned *bounds, unsigned *keys, int *vals) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float l[3], h[3];
    tri_box(tv, i, l, h);
    unsigned q[3];
    for (int a = 0; a < 3; ++a) {
        const float lo = o2f(bounds[a]), hi = o2f(bounds[3 + a]);
        const float ext = hi - lo;
        const float u = ext > 0.f ? (0.5f * (l[a] + h[a]) - lo) / ext : 0.5f;
        q[a] = (unsigned)fminf(fmaxf(u * 1024.f, 0.f), 1023.f);
    }
    keys[i] = (expand_bits(q[0]) << 2) | (expand_bits(q[1]) << 1) | expand_bits(q[2]);
    vals[i] = i;
}

// 3a. digit histogram of each block tile: hist[digit * nblocks + block]
__global__ void __launch_bounds__(kSortThreads) k_radix_hist(const unsigned *keys, int n, int shift, unsigned *hist) {
    __shared__ unsigned s_cnt[kDigits];
    for (int q = threadIdx.x; q < kDigits; q += kSortThreads) s_cnt[q] = 0;
    __syncthreads();
    const long long base = (long long)blockIdx.x * kTile;
    for (int r = 0; r < kSortRounds; ++r) {
        const long long i = base + (long long)r * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&s_cnt[(keys[i] >> shift) & (kDigits - 1)], 1u);
    }
    __syncthreads();
    for (int q = threadIdx.x; q < kDigits; q += kSortThreads) hist[(size_t)q * gridDim.x + blockIdx.x] = s_cnt[q];
}

// exclusive scan of m entries per block (m is at most a few hundred thousand): block b scans
// a[b m, (b + 1) m) and writes its sum to total[b] (when total is given)
__global__ void __launch_bounds__(kScanThreads) k_scan_excl(unsigned *a, int m, unsigned *total) {
    __shared__ unsigned s[kScanThreads];
    a += (size_t)blockIdx.x * m;
    const int per = (m + kScanThreads - 1) / kScanThreads;
    const int b0 = threadIdx.x * per, b1 = min(m, b0 + per);
    unsigned sum = 0;
    for (int i = b0; i < b1; ++i) sum += a[i];
    s[threadIdx.x] = sum;
    __syncthreads();
    for (int off = 1; off < kScanThreads; off <<= 1) {  // Hillis-Steele inclusive scan of the chunk sums
        const unsigned v = threadIdx.x >= off ? s[threadIdx.x - off] : 0u;
        __syncthreads();
        s[threadIdx.x] += v;
        __syncthreads();
    }
    unsigned run = threadIdx.x ? s[threadIdx.x - 1] : 0u;
    for (int i = b0; i < b1; ++i) {
        const unsigned v = a[i];
        a[i] = run;
        run += v;
    }
    if (threadIdx.x == kScanThreads - 1 && total) total[blockIdx.x] = s[kScanThreads - 1];
}

// 3b. stable scatter of each tile by digit, rounds in element order, ranks within a warp
// from __match_any_sync and across warps from per-warp digit counts. hist holds each
// digit's row of block counts scanned within the row, then the digits' exclusive offsets
// (the row totals scanned).
__global__ void __launch_bounds__(kSortThreads) k_radix_scatter(const unsigned *keys, const int *vals, int n, int shift,
                                                                const unsigned *hist, unsigned *keys_out,
                                                                int *vals_out) {
    constexpr int kWarps = kSortThreads / 32;
    __shared__ unsigned s_base[kDigits];
    __shared__ unsigned s_wcnt[kWarps][kDigits];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int q = threadIdx.x; q < kDigits; q += kSortThreads)
        s_base[q] = hist[(size_t)q * gridDim.x + blockIdx.x] + hist[(size_t)kDigits * gridDim.x + q];
    const long long base = (long long)blockIdx.x * kTile;
    for (int r = 0; r < kSortRounds; ++r) {
        const long long i = base + (long long)r * kSortThreads + threadIdx.x;
        const bool live = i < n;
        const unsigned k = live ? keys[i] : 0u;
        const int d = live ? (int)((k >> shift) & (kDigits - 1)) : kDigits;  // kDigits: not counted
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const unsigned rank = __popc(peers & ((1u << lane) - 1u));
        __syncthreads();  // s_base / s_wcnt of the previous round consumed
        for (int q = lane; q < kDigits; q += 32) s_wcnt[w][q] = 0;
        __syncwarp();
        if (live && rank == 0) s_wcnt[w][d] = __popc(peers);
        __syncthreads();
        unsigned off = 0;
        if (live) {
            off = s_base[d];
            for (int ww = 0; ww < w; ++ww) off += s_wcnt[ww][d];
        }
        __syncthreads();
        for (int q = threadIdx.x; q < kDigits; q += kSortThreads) {
            unsigned tot = 0;
            for (int ww = 0; ww < kWarps; ++ww) tot += s_wcnt[ww][q];
            s_base[q] += tot;
        }
        if (live) {
            keys_out[off + rank] = k;
            vals_out[off + rank] = vals[i];
        }
    }
}

// common prefix length of sorted codes i and j; equal codes compare their positions
__device__ __forceinline__ int delta(const unsigned *keys, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const unsigned a = keys[i], b = keys[j];
    return a == b ? 32 + __clz((unsigned)(i ^ j)) : __clz(a ^ b);
}

// 4. binary radix tree (Karras 2012): children (>= 0 inner node, < 0 ~leaf), parents, ranges
__global__ void k_radix_tree(const unsigned *keys, int n, int *left, int *right, int *parent_inner, int *parent_leaf,
                             int2 *range) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1) >= 0 ? 1 : -1;
    const int dmin = delta(keys, n, i, i - d);
    int lmax = 2;
    while (delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = delta(keys, n, i, j);
    int s = 0;
    for (int div = 2;; div <<= 1) {
        const int t = (l + div - 1) / div;
        if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
        if (t <= 1) break;
    }
    const int gamma = i + s * d + min(d, 0);
    const int lo = min(i, j), hi = max(i, j);
    const int lc = lo == gamma ? ~gamma : gamma;
    const int rc = hi == gamma + 1 ? ~(gamma + 1) : gamma + 1;
    left[i] = lc;
    right[i] = rc;
    range[i] = make_int2(lo, hi);
    if (lc >= 0) parent_inner[lc] = i; else parent_leaf[~lc] = i;
    if (rc >= 0) parent_inner[rc] = i; else parent_leaf[~rc] = i;
    if (i == 0) parent_inner[0] = -1;
}

// 5. boxes bottom-up; also the depth of each leaf (for the stack check)
__global__ void k_bottom_up(const float *tv, const int *vals, int n, const int *left, const int *right,
                            const int *parent_inner, const int *parent_leaf, float4 *leaf_box, float4 *node_box,
                            unsigned *arrivals, unsigned *max_depth) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    float lo[3], hi[3];
    tri_box(tv, vals[k], lo, hi);
    leaf_box[2 * k] = make_float4(lo[0], lo[1], lo[2], 0.f);
    leaf_box[2 * k + 1] = make_float4(hi[0], hi[1], hi[2], 0.f);
    unsigned depth = 1;
    for (int p = parent_leaf[k]; p >= 0; p = parent_inner[p]) ++depth;
    atomicMax(max_depth, depth);
    int p = parent_leaf[k];
    while (p >= 0) {
        __threadfence();
        if (atomicAdd(arrivals + p, 1u) == 0) return;  // the sibling's subtree is not done yet
        __threadfence();
        const int c[2] = {left[p], right[p]};
        float4 blo = make_float4(3.4e38f, 3.4e38f, 3.4e38f, 0.f), bhi = make_float4(-3.4e38f, -3.4e38f, -3.4e38f, 0.f);
        for (int q = 0; q < 2; ++q) {
            const float4 *src = c[q] >= 0 ? node_box + 2 * c[q] : leaf_box + 2 * (~c[q]);
            const float4 a = __ldcg(src), b = __ldcg(src + 1);
            blo = make_float4(fminf(blo.x, a.x), fminf(blo.y, a.y), fminf(blo.z, a.z), 0.f);
            bhi = make_float4(fmaxf(bhi.x, b.x), fmaxf(bhi.y, b.y), fmaxf(bhi.z, b.z), 0.f);
        }
        __stcg(node_box + 2 * p, blo);
        __stcg(node_box + 2 * p + 1, bhi);
        p = parent_inner[p];
    }
}

// 6a. inner nodes kept as BvhNode: more than kLeafMax triangles below them
__global__ void k_mark(const int2 *range, int m, unsigned *kept) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    kept[i] = (range[i].y - range[i].x + 1) > kLeafMax ? 1u : 0u;
}

// 6b. the compacted nodes: child codes (kept inner node: its new index; anything else: a
// leaf over its contiguous sorted range) and child boxes
__global__ void k_write_nodes(int m, const int *left, const int *right, const int2 *range, const unsigned *kept,
                              const unsigned *newidx, const float4 *leaf_box, const float4 *node_box, BvhNode *nodes) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m || !kept[i]) return;
    const int c[2] = {left[i], right[i]};
    int code[2];
    float4 lo[2], hi[2];
    for (int q = 0; q < 2; ++q) {
        if (c[q] >= 0) {
            lo[q] = node_box[2 * c[q]];
            hi[q] = node_box[2 * c[q] + 1];
            const int2 r = range[c[q]];
            code[q] = kept[c[q]] ? (int)newidx[c[q]] : ~((r.x << 3) | (r.y - r.x));
        } else {
            const int k = ~c[q];
            lo[q] = leaf_box[2 * k];
            hi[q] = leaf_box[2 * k + 1];
            code[q] = ~(k << 3);
        }
    }
    BvhNode nd;
    nd.x = make_float4(lo[0].x, hi[0].x, lo[1].x, hi[1].x);
    nd.y = make_float4(lo[0].y, hi[0].y, lo[1].y, hi[1].y);
    nd.z = make_float4(lo[0].z, hi[0].z, lo[1].z, hi[1].z);
    nd.child = make_int4(code[0], code[1], 0, 0);
    nodes[newidx[i]] = nd;
}

// 6c. triangle records in sorted (leaf) order: (v0, id) (v1 - v0) (v2 - v0)
__global__ void k_write_tris(const float *tv, const int *vals, int n, float4 *leaf_tris) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int t = vals[k];
    const float *v = tv + 9 * (size_t)t;
    leaf_tris[3 * (size_t)k] = make_float4(v[0], v[1], v[2], __int_as_float(t));
    leaf_tris[3 * (size_t)k + 1] = make_float4(v[3] - v[0], v[4] - v[1], v[5] - v[2], 0.f);
    leaf_tris[3 * (size_t)k + 2] = make_float4(v[6] - v[0], v[7] - v[1], v[8] - v[2], 0.f);
}

struct DevBuf {
    std::vector<void *> ptrs;
    cudaError_t err = cudaSuccess;
    template <class T>
    T *get(size_t count) {
        void *p = nullptr;
        if (err == cudaSuccess) err = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
        if (p) ptrs.push_back(p);
        return (T *)p;
    }
    ~DevBuf() {
        for (void *p : ptrs) cudaFree(p);
    }
};

}  // namespace

int build_bvh_device(const std::vector<float> &tri_verts, int num_tris, DeviceBvh &out, std::string &err) {
    out = DeviceBvh();
    const int n = num_tris;
    if (n < 2) {
        err = "device BVH build needs at least two triangles";
        return 1;
    }
    const int m = n - 1;
    const int nblk = (n + kTile - 1) / kTile;
    cudaStream_t st = 0;
    DevBuf tmp;
    float *tv = tmp.get<float>((size_t)9 * n);
    unsigned *bounds = tmp.get<unsigned>(8);
    unsigned *keys = tmp.get<unsigned>(n), *keys2 = tmp.get<unsigned>(n);
    int *vals = tmp.get<int>(n), *vals2 = tmp.get<int>(n);
    unsigned *hist = tmp.get<unsigned>((size_t)kDigits * (nblk + 1));  // rows of block counts, row totals
    int *left = tmp.get<int>(m), *right = tmp.get<int>(m), *par_in = tmp.get<int>(m), *par_leaf = tmp.get<int>(n);
    int2 *range = tmp.get<int2>(m);
    float4 *leaf_box = tmp.get<float4>((size_t)2 * n), *node_box = tmp.get<float4>((size_t)2 * m);
    unsigned *arrivals = tmp.get<unsigned>(m), *kept = tmp.get<unsigned>((size_t)m + 1);
    unsigned *newidx = tmp.get<unsigned>((size_t)m + 1), *counters = tmp.get<unsigned>(4);
    if (tmp.err != cudaSuccess) {
        err = std::string("device BVH build: ") + cudaGetErrorString(tmp.err);
        return 2;
    }
    const unsigned init[8] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u, 0u, 0u};
    cudaError_t e = cudaMemcpyAsync(tv, tri_verts.data(), (size_t)9 * n * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(bounds, init, sizeof(init), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(arrivals, 0, (size_t)m * sizeof(unsigned), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(counters, 0, 4 * sizeof(unsigned), st);
    const int T = 256;
    const unsigned g = (unsigned)((n + T - 1) / T), gm = (unsigned)((m + T - 1) / T);
    if (e == cudaSuccess) {
        k_centroid_bounds<<<g, T, 0, st>>>(tv, n, bounds);
        k_morton<<<g, T, 0, st>>>(tv, n, bounds, keys, vals);
        for (int shift = 0; shift < 32; shift += kDigitBits) {  // 32 key bits
            k_radix_hist<<<nblk, kSortThreads, 0, st>>>(keys, n, shift, hist);
            k_scan_excl<<<kDigits, kScanThreads, 0, st>>>(hist, nblk, hist + (size_t)kDigits * nblk);
            k_scan_excl<<<1, kScanThreads, 0, st>>>(hist + (size_t)kDigits * nblk, kDigits, nullptr);
            k_radix_scatter<<<nblk, kSortThreads, 0, st>>>(keys, vals, n, shift, hist, keys2, vals2);
            std::swap(keys, keys2);
            std::swap(vals, vals2);
        }
        k_radix_tree<<<gm, T, 0, st>>>(keys, n, left, right, par_in, par_leaf, range);
        k_bottom_up<<<g, T, 0, st>>>(tv, vals, n, left, right, par_in, par_leaf, leaf_box, node_box, arrivals,
                                     counters);
        k_mark<<<gm, T, 0, st>>>(range, m, kept);
        e = cudaMemcpyAsync(newidx, kept, (size_t)m * sizeof(unsigned), cudaMemcpyDeviceToDevice, st);
    }
    if (e == cudaSuccess) {
        k_scan_excl<<<1, kScanThreads, 0, st>>>(newidx, m, counters + 1);
        e = cudaGetLastError();
    }
    unsigned hc[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(hc, counters, 2 * sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        err = std::string("device BVH build: ") + cudaGetErrorString(e);
        return 2;
    }
    out.max_depth = (int)hc[0];
    out.num_nodes = (int)hc[1];
    if (out.max_depth > kStackDepth - 2 || out.num_nodes < 1) return 3;  // the caller builds on the host
    e = cudaMalloc(&out.nodes, (size_t)out.num_nodes * sizeof(BvhNode));
    if (e == cudaSuccess) e = cudaMalloc(&out.leaf_tris, (size_t)3 * n * sizeof(float4));
    if (e == cudaSuccess) {
        k_write_nodes<<<gm, T, 0, st>>>(m, left, right, range, kept, newidx, leaf_box, node_box, out.nodes);
        k_write_tris<<<g, T, 0, st>>>(tv, vals, n, out.leaf_tris);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaFree(out.nodes);
        cudaFree(out.leaf_tris);
        out = DeviceBvh();
        err = std::string("device BVH build: ") + cudaGetErrorString(e);
        return 2;
    }
    out.leaf_tris_bytes = (size_t)3 * n * sizeof(float4);
    return 0;
}

int radix_sort_launches(int bits) { return 4 * ((bits + kDigitBits - 1) / kDigitBits); }

size_t radix_hist_entries(long long n) { return (size_t)kDigits * (size_t)((n + kTile - 1) / kTile + 1); }

int *radix_sort_bits(unsigned *keys, int *vals, unsigned *keys2, int *vals2, unsigned *hist, int n, int bits,
                     cudaStream_t st) {
    if (n <= 1) return vals;
    const unsigned nblk = (unsigned)((n + kTile - 1) / kTile);
    for (int shift = 0; shift < bits; shift += kDigitBits) {
        k_radix_hist<<<nblk, kSortThreads, 0, st>>>(keys, n, shift, hist);
        k_scan_excl<<<kDigits, kScanThreads, 0, st>>>(hist, (int)nblk, hist + (size_t)kDigits * nblk);
        k_scan_excl<<<1, kScanThreads, 0, st>>>(hist + (size_t)kDigits * nblk, kDigits, nullptr);
        k_radix_scatter<<<nblk, kSortThreads, 0, st>>>(keys, vals, n, shift, hist, keys2, vals2);
        std::swap(keys, keys2);
        std::swap(vals, vals2);
    }
    return vals;
}

}  // namespace dt
