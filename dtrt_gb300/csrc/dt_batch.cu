// dtrt_gb300 — many scenes of uneven size in one persistent launch under a CUDA graph.
//
// No counterpart in the reference (one scene per blocking render call,
// integratorAD.cpp:19-166, parallel over pixels of that scene only). Every item of a batch
// is one scene with its own render options and device buffers; the work is the density
// adjoint replay of dtrt_render_adjoint (image + density gradient) for each item.
//
// Work distribution: the camera paths of all items are cut into chunks of `chunk` paths
// (a multiple of 32), laid out item after item in a tuned item order. A persistent grid
// (resident blocks only) lets each warp take the next chunk from one global counter, so
// long and short scenes share the GPU until the last chunk; the item of a chunk is a
// binary search over the chunk prefix. The launch and its memsets are captured once in a
// CUDA graph; dtrt_batch_launch replays it.
//
// Autotuner: (1) a probe launch per item on a sample of its paths measures the cost per
// path; items are then ordered longest-total-cost first (or kept in input order, whichever
// times faster); (2) the schedule is timed on a strided sample of every item's paths: the
// persistent launch with chunks of 32..512 paths, or one launch per item (scene data as
// kernel parameters) dealt over 1, 2 or 4 streams so that one item's tail overlaps the
// next item; the fastest is captured.
#include <algorithm>
#include <cstring>
#include <memory>
#include <numeric>
#include <vector>

#include "dt_adjoint.cuh"
#include "dt_host.h"

namespace dt {

// chunk c belongs to the item at position i of the order with cbeg[i] <= c < cbeg[i+1]
__global__ void __launch_bounds__(kBlock) k_batch(const BatchItemDev *items, const long long *cbeg, const int *order,
                                                  int n, long long total_chunks, int chunk, long long sample_stride,
                                                  unsigned long long *next) {
    __shared__ int s_stack[kStackDepth * kBlock];
    // the current item's scene and parameters, one copy per warp: the path code reads them
    // at every step, and shared memory serves those uniform reads like kernel parameters do
    __shared__ DevScene s_sc[kBlock / 32];
    __shared__ RenderParams s_rp[kBlock / 32];
    int *stack = s_stack + threadIdx.x;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int cur = -1;
    const float *dimg = nullptr;
    float *grad = nullptr;
    double *img_acc = nullptr;
    for (;;) {
        unsigned long long c = 0;
        if (lane == 0) c = atomicAdd(next, 1ull);
        c = __shfl_sync(full, c, 0);
        if (c >= (unsigned long long)total_chunks) break;
        int lo = 0, hi = n - 1;  // largest i with cbeg[i] <= c
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if ((unsigned long long)cbeg[mid] <= c) lo = mid;
            else hi = mid - 1;
        }
        const int item = order[lo];
        if (item != cur) {  // warp-uniform: copy the item's scene and parameters into shared memory
            __syncwarp();
            const BatchItemDev &it = items[item];
            const uint32_t *src = reinterpret_cast<const uint32_t *>(&it.sc);
            uint32_t *dst = reinterpret_cast<uint32_t *>(&s_sc[warp]);
            for (int k = lane; k < (int)(sizeof(DevScene) / 4); k += 32) dst[k] = src[k];
            src = reinterpret_cast<const uint32_t *>(&it.rp);
            dst = reinterpret_cast<uint32_t *>(&s_rp[warp]);
            for (int k = lane; k < (int)(sizeof(RenderParams) / 4); k += 32) dst[k] = src[k];
            dimg = it.dimg;
            grad = it.grad;
            img_acc = it.img_acc;
            cur = item;
            __syncwarp();
        }
        const long long base = ((long long)c - cbeg[lo]) * chunk;
        Ctr ctr;
        for (int k = lane; k < chunk; k += 32)  // sample_stride > 1 (tuning): every stride-th path
            adjoint_one<1>(s_sc[warp], s_rp[warp], stack, base + k, dimg, grad, img_acc, ctr, sample_stride);
    }
}

// FP64 image accumulators -> float images of every item (integratorAD.cpp:59-87 write rule)
struct BatchImageDev {
    const double *acc;
    float *out;
    long long pix_begin;
};
__global__ void k_batch_image(const BatchImageDev *imgs, int n, long long total_pix) {
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= total_pix) return;
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (imgs[mid].pix_begin <= p) lo = mid;
        else hi = mid - 1;
    }
    const long long q = p - imgs[lo].pix_begin;
    const double *a = imgs[lo].acc + q * 3;
    const bool nonneg = a[0] >= 0.0 && a[1] >= 0.0 && a[2] >= 0.0;
    for (int c = 0; c < 3; ++c) imgs[lo].out[q * 3 + c] = nonneg ? (float)a[c] : 0.f;
}

}  // namespace dt

struct dtrt_batch {
    int device = 0;
    int n = 0;
    std::vector<dtrt_batch_item> items;
    std::vector<dt::BatchItemDev> host_items;
    std::vector<size_t> npix, nvox;
    std::vector<long long> paths;
    // device memory
    dt::BatchItemDev *d_items = nullptr;
    long long *d_cbeg = nullptr;
    int *d_order = nullptr;
    dt::BatchImageDev *d_imgs = nullptr;
    unsigned long long *d_next = nullptr;
    unsigned int *d_err = nullptr;
    std::vector<double *> img_acc;
    std::vector<int> vert_items;  // items with d_vertices: the vertex replay after the captured launch
    // launch shape
    int grid = 0, chunk = 128, n_img = 0;
    long long total_chunks = 0, total_pix = 0;
    std::vector<int> order;
    std::vector<long long> cbeg;
    // schedule: 0 persistent launch, 1 one launch per item spread over `nstreams` streams,
    // 2 one wavefront over all items
    int schedule = 0, nstreams = 1;
    std::vector<cudaStream_t> side;  // streams 1.. of the per-item schedule
    std::vector<cudaEvent_t> side_ev;
    cudaEvent_t fork_ev = nullptr;
    // wavefront replay workspaces of the per-item schedule, one per stream (empty: megakernel)
    std::vector<void *> wave_mem;
    std::vector<dt::AdjWave> wave;
    // the batch wavefront (schedule 2): one replay wavefront over the paths of all items
    void *bw_mem = nullptr;
    dt::AdjWave bw;
    int wave_items = 0;  // items in the uploaded wavefront numbering
    int max_levels = 1;
    bool any_grad = false;
    // tuning: best strided-sample time of the persistent launch, the per-item schedule on
    // 1, 2 and 4 streams, and the batch wavefront
    float sampled_best[5] = {1e30f, 1e30f, 1e30f, 1e30f, 1e30f};
    int sms = 0;
    // graph
    cudaStream_t cap_stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    dtrt_batch_stats stats{};
};

namespace dt {
namespace {

// paths per workspace of the batch wavefront (about 780 B of replay state per path)
constexpr long long kBatchWaveCap = 1ll << 23;

#define DT_BCK(call)                                                                 \
    do {                                                                             \
        cudaError_t e_ = (call);                                                     \
        if (e_ != cudaSuccess) {                                                     \
            set_last_error(std::string(#call) + ": " + cudaGetErrorString(e_));      \
            return DTRT_ERR_CUDA;                                                    \
        }                                                                            \
    } while (0)

void free_batch(dtrt_batch *b) {
    for (cudaStream_t x : b->side) cudaStreamDestroy(x);
    for (cudaEvent_t x : b->side_ev) cudaEventDestroy(x);
    if (b->fork_ev) cudaEventDestroy(b->fork_ev);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
    for (void *p : b->wave_mem) cudaFree(p);
    if (b->bw_mem) cudaFree(b->bw_mem);
    void *ptrs[] = {b->d_items, b->d_cbeg, b->d_order, b->d_imgs, b->d_next, b->d_err};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    for (double *p : b->img_acc)
        if (p) cudaFree(p);
}

// chunk layout for an item order and chunk size (sample_stride > 1: sampled path counts)
void layout(dtrt_batch *b, const std::vector<int> &order, int chunk, long long stride, std::vector<long long> &cbeg,
            long long &total) {
    cbeg.assign(b->n + 1, 0);
    for (int i = 0; i < b->n; ++i) {
        const long long p = (b->paths[order[i]] + stride - 1) / stride;
        cbeg[i + 1] = cbeg[i] + (p + chunk - 1) / chunk;
    }
    total = cbeg[b->n];
}

// upload a chunk layout (blocking copies: never inside a stream capture)
int upload_layout(dtrt_batch *b, const std::vector<int> &order, int chunk, long long stride, long long &total) {
    std::vector<long long> cbeg;
    layout(b, order, chunk, stride, cbeg, total);
    DT_BCK(cudaMemcpy(b->d_cbeg, cbeg.data(), cbeg.size() * 8, cudaMemcpyHostToDevice));
    DT_BCK(cudaMemcpy(b->d_order, order.data(), order.size() * 4, cudaMemcpyHostToDevice));
    return DTRT_OK;
}

// counter reset + one k_batch launch over the uploaded layout; the caller zeroes outputs
int launch_kernel(dtrt_batch *b, long long total, int chunk, long long stride, cudaStream_t st) {
    DT_BCK(cudaMemsetAsync(b->d_next, 0, 8, st));
    if (total > 0) k_batch<<<b->grid, kBlock, 0, st>>>(b->d_items, b->d_cbeg, b->d_order, b->n, total, chunk, stride, b->d_next);
    DT_BCK(cudaGetLastError());
    return DTRT_OK;
}

int launch_once(dtrt_batch *b, const std::vector<int> &order, int chunk, long long stride, cudaStream_t st) {
    long long total = 0;
    DT_BCK(cudaStreamSynchronize(st));  // the layout buffers may still be read by a previous launch
    int rc = upload_layout(b, order, chunk, stride, total);
    return rc ? rc : launch_kernel(b, total, chunk, stride, st);
}

// one k_adjoint launch per item (every stride-th path), items taken in `order`, each dealt to
// the least-loaded of st and S-1 side streams that fork from and join back into st (graph-
// capturable); an item's load is its measured cost estimate, else its path count
int launch_items(dtrt_batch *b, const std::vector<int> &order, int S, long long stride, cudaStream_t st,
                 bool zero = false) {
    S = std::max(1, std::min(S, 1 + (int)b->side.size()));
    if (S > 1) {
        DT_BCK(cudaEventRecord(b->fork_ev, st));
        for (int k = 1; k < S; ++k) DT_BCK(cudaStreamWaitEvent(b->side[k - 1], b->fork_ev, 0));
    }
    std::vector<double> load(S, 0.0);
    for (size_t i = 0; i < order.size(); ++i) {
        const int item = order[i];
        const BatchItemDev &it = b->host_items[item];
        const int s = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        const double est = b->stats.item_ms_estimate[std::min(item, DTRT_BATCH_MAX_ITEMS - 1)];
        load[s] += est > 0.0 ? est : (double)b->paths[item];
        cudaStream_t q = s == 0 ? st : b->side[s - 1];
        if (zero) {  // each item's outputs are cleared just before its own launches, on its stream
            if (it.img_acc) DT_BCK(cudaMemsetAsync(it.img_acc, 0, b->npix[item] * 3 * 8, q));
            if (it.grad) DT_BCK(cudaMemsetAsync(it.grad, 0, b->nvox[item] * 4, q));
        }
        if (stride > 1) {
            DT_BCK(launch_adjoint(it.sc, it.rp, it.dimg, it.grad, it.img_acc, nullptr, stride, q));
            continue;
        }
        if (!b->wave.empty()) {  // the wavefront replay of dtrt_render_adjoint, on this stream's workspace
            DT_BCK(launch_adjoint_wave(it.sc, it.rp, it.dimg, it.grad, it.img_acc, nullptr, b->wave[s], b->sms, q,
                                       nullptr));
            continue;
        }
        RenderParams rp = it.rp;  // launches of at most 2^24 paths, as dtrt_render_adjoint
        for (long long b0 = 0; b0 < it.rp.path_count; b0 += 1ll << 24) {
            rp.path_begin = b0;
            rp.path_count = std::min(1ll << 24, it.rp.path_count - b0);
            DT_BCK(launch_adjoint(it.sc, rp, it.dimg, it.grad, it.img_acc, nullptr, 1, q));
        }
    }
    for (int k = 1; k < S; ++k) {
        DT_BCK(cudaEventRecord(b->side_ev[k - 1], b->side[k - 1]));
        DT_BCK(cudaStreamWaitEvent(st, b->side_ev[k - 1], 0));
    }
    return DTRT_OK;
}

// the batch wavefront's path numbering: the items in `order` (all of them, or a subset),
// every stride-th path (blocking copies: never inside a stream capture). Returns the number
// of global paths.
int upload_wave_layout(dtrt_batch *b, const std::vector<int> &order, long long stride, long long &total) {
    const int m = (int)order.size();
    std::vector<long long> gbeg(m + 1, 0);
    for (int i = 0; i < m; ++i) gbeg[i + 1] = gbeg[i] + (b->paths[order[i]] + stride - 1) / stride;
    total = gbeg[m];
    b->wave_items = m;
    DT_BCK(cudaMemcpy(b->d_cbeg, gbeg.data(), gbeg.size() * 8, cudaMemcpyHostToDevice));
    DT_BCK(cudaMemcpy(b->d_order, order.data(), order.size() * 4, cudaMemcpyHostToDevice));
    return DTRT_OK;
}

// One replay wavefront over the uploaded numbering, in chunks of a workspace's capacity:
// pass A (start, one launch per vertex kind and level, totals), then, when an item asks
// for a density gradient, pass B. Every level launch covers live paths of all items; a
// chunk spans item boundaries. Chunks are independent: they are dealt round-robin to the
// caller's stream and the side streams, each with its own workspace, so that one chunk's
// last, sparse levels overlap the next chunk's work.
int enqueue_chunk(dtrt_batch *b, const AdjWave &w, BatchWave bw, cudaStream_t st) {
    const int levels = b->max_levels;
    auto blocks = [](long long n) { return (unsigned)((n + kBlock - 1) / kBlock); };
    AdjState<1> *states = (AdjState<1> *)w.states;
    VertexIn<1> *vins = (VertexIn<1> *)w.vins;
    int *qa = w.q, *qb = qa + w.cap, *qv = qb + w.cap, *qs = qv + w.cap;
    {
        const unsigned gw = std::min<unsigned>(blocks(bw.count), (unsigned)std::max(1, b->sms) * 16u);
        DT_BCK(cudaMemsetAsync(w.cnt, 0, (size_t)6 * (levels + 1) * sizeof(unsigned long long), st));
        for (int pass = 0; pass < (b->any_grad ? 2 : 1); ++pass) {
            const bool pb = pass == 1;
            // per level: volume, interface front-end and back-end counts (as launch_adjoint_wave)
            unsigned long long *vc = w.cnt + pass * 3 * (levels + 1), *scn = vc + (levels + 1);
            const QueueEnds qx{w.cap, levels + 1};
            k_badj_start<1><<<blocks(bw.count), kBlock, 0, st>>>(bw, states, vins, qa, vc, qv, vc + 1, qs, scn + 1,
                                                                w.tots, w.ev, qx, pb);
            for (int L = 0; L < levels; ++L) {
                int *qvl = (L & 1) ? qv : qa, *qsl = (L & 1) ? qs : qb;
                int *qvn = (L & 1) ? qa : qv, *qsn = (L & 1) ? qb : qs;
                k_badj_vertex<1, true><<<gw, kBlock, 0, st>>>(bw, states, vins, qvl, vc + L, qvn, vc + L + 1, qsn,
                                                             scn + L + 1, w.tots, w.ev, qx, pb);
                if (L > 0)
                    k_badj_vertex<1, false><<<gw, kBlock, 0, st>>>(bw, states, vins, qsl, scn + L, qvn, vc + L + 1,
                                                                  qsn, scn + L + 1, w.tots, w.ev, qx, pb);
            }
            if (pass == 0) k_badj_totals<1><<<blocks(bw.count), kBlock, 0, st>>>(bw, states, w.tots);
        }
        DT_BCK(cudaGetLastError());
    }
    return DTRT_OK;
}

int enqueue_wave(dtrt_batch *b, long long total, long long stride, cudaStream_t st) {
    // workspaces: the per-stream ones of the per-item schedule when they hold the deepest
    // item's levels, else the single batch workspace
    const bool multi = b->wave.size() == 4 && b->wave[0].levels >= b->max_levels;
    const int S = multi ? 4 : 1;
    const long long cap = multi ? b->wave[0].cap : b->bw.cap;
    if (S > 1) {
        DT_BCK(cudaEventRecord(b->fork_ev, st));
        for (int k = 1; k < S; ++k) DT_BCK(cudaStreamWaitEvent(b->side[k - 1], b->fork_ev, 0));
    }
    BatchWave bw{b->d_items, b->d_cbeg, b->d_order, b->wave_items, 0, 0, stride};
    int k = 0;
    for (long long b0 = 0; b0 < total; b0 += cap, k = (k + 1) % S) {
        bw.begin = b0;
        bw.count = std::min(cap, total - b0);
        cudaStream_t q = k == 0 ? st : b->side[k - 1];
        int rc = enqueue_chunk(b, multi ? b->wave[k] : b->bw, bw, q);
        if (rc) return rc;
    }
    for (int j = 1; j < S; ++j) {
        DT_BCK(cudaEventRecord(b->side_ev[j - 1], b->side[j - 1]));
        DT_BCK(cudaStreamWaitEvent(st, b->side_ev[j - 1], 0));
    }
    return DTRT_OK;
}

int launch_wave(dtrt_batch *b, const std::vector<int> &order, long long stride, cudaStream_t st) {
    long long total = 0;
    DT_BCK(cudaStreamSynchronize(st));  // the numbering buffers may still be read by a previous launch
    int rc = upload_wave_layout(b, order, stride, total);
    return rc ? rc : enqueue_wave(b, total, stride, st);
}

int launch_schedule(dtrt_batch *b, cudaStream_t st, long long stride) {
    if (b->schedule == 1) return launch_items(b, b->order, b->nstreams, stride, st, true);
    if (b->schedule == 2) return launch_wave(b, b->order, stride, st);
    return launch_once(b, b->order, b->chunk, stride, st);
}

// clear every item's outputs (the per-item schedule clears each item just before it instead)
int zero_outputs(dtrt_batch *b, cudaStream_t st) {
    for (int i = 0; i < b->n && b->schedule != 1; ++i) {
        if (b->host_items[i].img_acc) DT_BCK(cudaMemsetAsync(b->host_items[i].img_acc, 0, b->npix[i] * 3 * 8, st));
        if (b->host_items[i].grad) DT_BCK(cudaMemsetAsync(b->host_items[i].grad, 0, b->nvox[i] * 4, st));
    }
    DT_BCK(cudaMemsetAsync(b->d_err, 0, 4, st));
    return DTRT_OK;
}

// time fn() on st with events (ms)
template <class F>
int timed(cudaStream_t st, F &&fn, float &ms) {
    cudaEvent_t e0, e1;
    DT_BCK(cudaEventCreate(&e0));
    DT_BCK(cudaEventCreate(&e1));
    cudaEventRecord(e0, st);
    int rc = fn();
    cudaEventRecord(e1, st);
    cudaError_t e = cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if (e != cudaSuccess) {
        set_last_error(std::string("batch timing: ") + cudaGetErrorString(e));
        return DTRT_ERR_CUDA;
    }
    return DTRT_OK;
}

int autotune(dtrt_batch *b, cudaStream_t st) {
    const long long kProbePaths = 16384;
    // (1) cost per path of every item, from a strided probe of about kProbePaths paths
    std::vector<double> cost(b->n, 0.0);
    for (int i = 0; i < b->n; ++i) {
        const long long stride = std::max<long long>(1, b->paths[i] / kProbePaths);
        std::vector<int> one = {i};
        // a one-item layout: other items get no chunks
        std::vector<long long> cbeg = {0, ((b->paths[i] + stride - 1) / stride + 127) / 128};
        float ms = 0.f;
        DT_BCK(cudaStreamSynchronize(st));
        DT_BCK(cudaMemcpy(b->d_cbeg, cbeg.data(), 16, cudaMemcpyHostToDevice));
        DT_BCK(cudaMemcpy(b->d_order, one.data(), 4, cudaMemcpyHostToDevice));
        int rc = timed(st, [&]() -> int {
            DT_BCK(cudaMemsetAsync(b->d_next, 0, 8, st));
            k_batch<<<b->grid, kBlock, 0, st>>>(b->d_items, b->d_cbeg, b->d_order, 1, cbeg[1], 128, stride, b->d_next);
            DT_BCK(cudaGetLastError());
            return DTRT_OK;
        }, ms);
        if (rc) return rc;
        const double sampled = (double)((b->paths[i] + stride - 1) / stride);
        cost[i] = ms / std::max(1.0, sampled) * (double)b->paths[i];  // ms for the whole item
        b->stats.item_ms_estimate[std::min(i, DTRT_BATCH_MAX_ITEMS - 1)] = cost[i];
    }
    std::vector<int> natural(b->n), longest(b->n);
    std::iota(natural.begin(), natural.end(), 0);
    std::iota(longest.begin(), longest.end(), 0);
    std::stable_sort(longest.begin(), longest.end(), [&](int a, int c) { return cost[a] > cost[c]; });
    // (2) chunk size x order on a strided sample of the whole batch
    long long total_paths = 0;
    for (long long p : b->paths) total_paths += p;
    const long long stride = std::max<long long>(1, total_paths / (1ll << 22));
    const int chunks[] = {32, 64, 128, 256, 512};
    float best = 1e30f;
    int trial = 0;
    for (int oi = 0; oi < 2; ++oi) {
        const std::vector<int> &ord = oi == 0 ? longest : natural;
        for (int ch : chunks) {
            float ms = 0.f;
            long long total = 0;
            DT_BCK(cudaStreamSynchronize(st));
            int rc = upload_layout(b, ord, ch, stride, total);
            if (rc) return rc;
            rc = timed(st, [&]() { return launch_kernel(b, total, ch, stride, st); }, ms);
            if (rc) return rc;
            if (trial < DTRT_BATCH_MAX_TRIALS) {
                b->stats.trial_chunk[trial] = ch;
                b->stats.trial_order[trial] = oi;
                b->stats.trial_ms[trial] = ms;
            }
            ++trial;
            if (ms < best) {
                best = ms;
                b->chunk = ch;
                b->order = ord;
                b->stats.order_longest_first = oi == 0;
            }
        }
    }
    b->sampled_best[0] = best;
    // one launch per item over 1, 2 or 4 streams (longest first)
    for (int S : {1, 2, 4}) {
        float ms = 0.f;
        DT_BCK(cudaStreamSynchronize(st));
        int rc = timed(st, [&]() { return launch_items(b, longest, S, stride, st); }, ms);
        if (rc) return rc;
        if (trial < DTRT_BATCH_MAX_TRIALS) {
            b->stats.trial_chunk[trial] = -S;  // negative: per-item launches over S streams
            b->stats.trial_order[trial] = 0;
            b->stats.trial_ms[trial] = ms;
        }
        ++trial;
        b->sampled_best[S == 1 ? 1 : S == 2 ? 2 : 3] = ms;
        if (ms < best) {
            best = ms;
            b->schedule = 1;
            b->nstreams = S;
            b->order = longest;
            b->stats.order_longest_first = 1;
        }
    }
    // one wavefront over all items (input order)
    if (b->bw_mem) {
        float ms = 0.f;
        DT_BCK(cudaStreamSynchronize(st));
        int rc = timed(st, [&]() { return launch_wave(b, natural, stride, st); }, ms);
        if (rc) return rc;
        if (trial < DTRT_BATCH_MAX_TRIALS) {
            b->stats.trial_chunk[trial] = 0;  // 0: the batch wavefront
            b->stats.trial_order[trial] = 1;
            b->stats.trial_ms[trial] = ms;
        }
        ++trial;
        b->sampled_best[4] = ms;
        if (ms < best) {
            best = ms;
            b->schedule = 2;
            b->order = natural;
            b->stats.order_longest_first = 0;
        }
    }
    b->stats.num_trials = std::min(trial, DTRT_BATCH_MAX_TRIALS);
    b->stats.tune_sample_stride = stride;
    return DTRT_OK;
}

// Full-size confirmation (DTRT_BATCH_TUNE_FULL): a strided sample shrinks every per-item
// launch to a few waves, which understates that schedule on large items. The two
// candidates (persistent, per-item on 1, 2 or 4 streams, batch wavefront) that were
// fastest on the sample run once each on whole items, every fourth in cost order; the
// faster one is kept.
int autotune_full(dtrt_batch *b, cudaStream_t st) {
    const int saved_chunk = b->chunk;
    const std::vector<int> saved_order = b->order;
    std::vector<int> longest(b->n);
    std::iota(longest.begin(), longest.end(), 0);
    std::stable_sort(longest.begin(), longest.end(), [&](int a, int c) {
        return b->stats.item_ms_estimate[std::min(a, DTRT_BATCH_MAX_ITEMS - 1)] >
               b->stats.item_ms_estimate[std::min(c, DTRT_BATCH_MAX_ITEMS - 1)];
    });
    float best = 1e30f;
    int best_sched = 0, best_streams = 1;
    std::vector<int> natural(b->n);
    std::iota(natural.begin(), natural.end(), 0);
    // whole items (not a strided sample of paths), every fourth in cost order from 8 items
    // on: the wavefront schedules see full-size launches at a quarter of the batch's work
    std::vector<int> sub_longest, sub_natural;
    for (int i = 0; i < b->n; i += b->n >= 8 ? 4 : 1) sub_longest.push_back(longest[i]);
    sub_natural = sub_longest;
    std::sort(sub_natural.begin(), sub_natural.end());
    // the two best candidates on the strided sample are confirmed on those items. With items
    // large enough for the wavefront replay the persistent megakernel is left out: the
    // strided sample understates the wavefront schedules (a sample of a large item is a few
    // short launches) and overstates the megakernel, which the replay wavefront outpaces
    // several times at full size (7.3 s against 1.86 s on the 64-scene C4 batch)
    std::vector<int> rank;
    for (int cand = 0; cand < 5; ++cand)
        if (!(cand == 0 && !b->wave.empty()) && !(cand == 4 && !b->bw_mem)) rank.push_back(cand);
    std::stable_sort(rank.begin(), rank.end(), [&](int a, int c) { return b->sampled_best[a] < b->sampled_best[c]; });
    rank.resize(std::max<size_t>(rank.size(), 2), -1);
    for (int cand = 0; cand < 5; ++cand) {
        if (cand == 4 && !b->bw_mem) continue;
        if (cand != rank[0] && cand != rank[1]) {
            if (cand < 4) b->stats.full_ms[cand] = -1.f;
            else b->stats.full_ms_wavefront = -1.f;
            continue;
        }
        float ms = 0.f;
        DT_BCK(cudaStreamSynchronize(st));
        int rc;
        if (cand == 4) {
            rc = timed(st, [&]() { return launch_wave(b, sub_natural, 1, st); }, ms);
        } else if (cand == 0) {  // the persistent layout covers every item
            long long total = 0;
            rc = upload_layout(b, saved_order, saved_chunk, 1, total);
            if (rc) return rc;
            rc = timed(st, [&]() { return launch_kernel(b, total, saved_chunk, 1, st); }, ms);
            double all = 0.0, part = 0.0;  // scaled to the subset's share of the estimated cost
            for (int i = 0; i < b->n; ++i) all += b->stats.item_ms_estimate[std::min(i, DTRT_BATCH_MAX_ITEMS - 1)];
            for (int i : sub_longest) part += b->stats.item_ms_estimate[std::min(i, DTRT_BATCH_MAX_ITEMS - 1)];
            if (all > 0.0) ms = (float)(ms * part / all);
        } else {
            rc = timed(st, [&]() { return launch_items(b, sub_longest, 1 << (cand - 1), 1, st); }, ms);
        }
        if (rc) return rc;
        if (cand < 4) b->stats.full_ms[cand] = ms;
        else b->stats.full_ms_wavefront = ms;
        if (ms < best) {
            best = ms;
            best_sched = cand == 0 ? 0 : cand == 4 ? 2 : 1;
            best_streams = (cand == 0 || cand == 4) ? 1 : 1 << (cand - 1);
        }
    }
    b->schedule = best_sched;
    b->nstreams = best_streams;
    b->chunk = saved_chunk;
    b->order = best_sched == 0 ? saved_order : best_sched == 2 ? natural : longest;
    b->stats.order_longest_first = best_sched == 1 ? 1 : best_sched == 2 ? 0 : b->stats.order_longest_first;
    return DTRT_OK;
}

// capture zero + launch + image conversion into a graph (the layout is uploaded first and
// stays fixed: every replay runs the tuned order and chunk size)
int capture(dtrt_batch *b) {
    cudaStream_t cs = b->cap_stream;
    long long total = 0;
    int rc = b->schedule == 2 ? upload_wave_layout(b, b->order, 1, total) : upload_layout(b, b->order, b->chunk, 1, total);
    if (rc) return rc;
    DT_BCK(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    rc = zero_outputs(b, cs);
    if (!rc) rc = b->schedule == 1 ? launch_items(b, b->order, b->nstreams, 1, cs, true)
                  : b->schedule == 2 ? enqueue_wave(b, total, 1, cs)
                                     : launch_kernel(b, total, b->chunk, 1, cs);
    if (!rc && b->n_img > 0) {
        k_batch_image<<<(unsigned)((b->total_pix + 255) / 256), 256, 0, cs>>>(b->d_imgs, b->n_img, b->total_pix);
        if (cudaGetLastError() != cudaSuccess) rc = DTRT_ERR_CUDA;
    }
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(cs, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) {
        set_last_error(std::string("batch graph capture: ") + cudaGetErrorString(e));
        return DTRT_ERR_CUDA;
    }
    b->graph = g;
    DT_BCK(cudaGraphInstantiate(&b->exec, g, 0));
    return DTRT_OK;
}

}  // namespace
}  // namespace dt

extern "C" {

int dtrt_batch_create(const dtrt_batch_item *items, int n, unsigned flags, void *stream, dtrt_batch **out) {
    using namespace dt;
    if (!items || !out || n <= 0) {
        set_last_error("null argument or empty batch");
        return DTRT_ERR_INVALID;
    }
    *out = nullptr;
    std::unique_ptr<dtrt_batch, void (*)(dtrt_batch *)> b(new dtrt_batch(), [](dtrt_batch *p) {
        free_batch(p);
        delete p;
    });
    cudaStream_t st = (cudaStream_t)stream;
    b->n = n;
    b->items.assign(items, items + n);
    cudaGetDevice(&b->device);
    DT_BCK(cudaMalloc(&b->d_err, 4));
    for (int i = 0; i < n; ++i) {
        const dtrt_batch_item &it = items[i];
        if (!it.scene || it.opts.spp < 0 || it.opts.max_bounces < 0 || (!it.image && !it.d_density && !it.d_vertices)) {
            set_last_error("batch item " + std::to_string(i) + ": needs a scene, spp/max_bounces >= 0 and an output");
            return DTRT_ERR_INVALID;
        }
        if (it.scene->device != b->device) {
            set_last_error("batch items must live on the current device");
            return DTRT_ERR_INVALID;
        }
        if ((it.d_density || it.d_vertices) && !it.d_image) {
            set_last_error("batch item " + std::to_string(i) + ": d_density and d_vertices need d_image");
            return DTRT_ERR_INVALID;
        }
        if (it.d_vertices && it.d_density) {
            set_last_error("batch item " + std::to_string(i) + ": d_vertices takes no d_density");
            return DTRT_ERR_INVALID;
        }
        // a vertex item has no paths in the batch's launch: the vertex replay renders it
        const bool vertex_item = it.d_vertices != nullptr;
        if (vertex_item) b->vert_items.push_back(i);
        DevScene sc = it.scene->dev;
        sc.vert_der = nullptr;
        sc.face_n_der = nullptr;
        sc.normal_der = nullptr;
        sc.moving_geometry = 0;
        std::memset(sc.cam.d_cpos, 0, sizeof(sc.cam.d_cpos));
        std::memset(sc.cam.d_cframe, 0, sizeof(sc.cam.d_cframe));
        sc.error_flags = b->d_err;
        const DevCamera &cam = sc.cam;
        const bool cropped = cam.crop_w > 0 && cam.crop_h > 0;
        RenderParams rp{};
        rp.seed = it.opts.seed;
        rp.spp = it.opts.spp;
        rp.max_bounces = it.opts.max_bounces;
        rp.mode = it.opts.mode >= 0 ? it.opts.mode : MODE_ALL;
        rp.jitter = it.opts.sppe >= 0 ? 1 : 0;
        rp.ddist = it.opts.ddist_coeff;
        rp.inv_spp = it.opts.spp > 0 ? 1.0f / (float)it.opts.spp : 0.f;
        rp.out_w = cropped ? cam.crop_w : cam.width;
        rp.out_h = cropped ? cam.crop_h : cam.height;
        rp.crop_x = cropped ? cam.crop_x : 0;
        rp.crop_y = cropped ? cam.crop_y : 0;
        rp.npix = rp.out_w * rp.out_h;
        const long long paths = vertex_item ? 0 : (long long)rp.npix * std::max(0, it.opts.spp);
        rp.path_begin = 0;
        rp.path_count = paths;
        BatchItemDev d{};
        d.sc = sc;
        d.rp = rp;
        d.dimg = it.d_image;
        d.grad = (it.d_density && it.scene->density_voxels > 0) ? it.d_density : nullptr;
        d.img_acc = nullptr;
        double *acc = nullptr;
        if (it.image && !vertex_item) {
            DT_BCK(cudaMalloc(&acc, (size_t)rp.npix * 3 * 8));
            d.img_acc = acc;
        }
        b->img_acc.push_back(acc);
        b->host_items.push_back(d);
        b->npix.push_back((size_t)rp.npix);
        b->nvox.push_back((size_t)it.scene->density_voxels);
        b->paths.push_back(paths);
    }
    DT_BCK(cudaMalloc(&b->d_items, sizeof(BatchItemDev) * n));
    DT_BCK(cudaMemcpy(b->d_items, b->host_items.data(), sizeof(BatchItemDev) * n, cudaMemcpyHostToDevice));
    DT_BCK(cudaMalloc(&b->d_cbeg, 8 * (n + 1)));
    DT_BCK(cudaMalloc(&b->d_order, 4 * n));
    DT_BCK(cudaMalloc(&b->d_next, 8));
    std::vector<BatchImageDev> imgs;
    long long pix = 0;
    for (int i = 0; i < n; ++i)
        if (items[i].image && b->img_acc[i]) {
            imgs.push_back({b->img_acc[i], items[i].image, pix});
            pix += (long long)b->npix[i];
        }
    b->n_img = (int)imgs.size();
    b->total_pix = pix;
    if (!imgs.empty()) {
        DT_BCK(cudaMalloc(&b->d_imgs, sizeof(BatchImageDev) * imgs.size()));
        DT_BCK(cudaMemcpy(b->d_imgs, imgs.data(), sizeof(BatchImageDev) * imgs.size(), cudaMemcpyHostToDevice));
    }
    // persistent grid: resident blocks only
    int sms = 0, per_sm = 0;
    DT_BCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device));
    DT_BCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch, kBlock, 0));
    b->grid = std::max(1, sms * std::max(1, per_sm));
    DT_BCK(cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming));
    for (int k = 0; k < 3; ++k) {
        cudaStream_t x;
        cudaEvent_t ev;
        DT_BCK(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
        b->side.push_back(x);
        DT_BCK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        b->side_ev.push_back(ev);
    }
    // wavefront workspaces for the per-item schedule (4 streams), as dtrt_render_adjoint's
    {
        long long maxp = 0;
        int maxl = 1;
        for (int i = 0; i < n; ++i) {
            maxp = std::max(maxp, b->paths[i]);
            maxl = std::max(maxl, items[i].opts.max_bounces + 1);
        }
        b->sms = sms;
        if (maxp >= kWavefrontMinPaths) {
            const long long cap = std::min<long long>(1ll << 22, maxp);
            for (int k = 0; k < 4; ++k) {
                void *p = nullptr;
                if (cudaMalloc(&p, AdjWave::bytes(cap, maxl)) != cudaSuccess) {
                    cudaGetLastError();  // no room: the per-item schedule runs the megakernel
                    for (void *x : b->wave_mem) cudaFree(x);
                    b->wave_mem.clear();
                    b->wave.clear();
                    break;
                }
                b->wave_mem.push_back(p);
                AdjWave w;
                w.carve(p, cap, maxl);
                b->wave.push_back(w);
            }
        }
    }
    // workspace of the batch wavefront: one replay wavefront over the paths of all items
    {
        long long tp = 0;
        for (int i = 0; i < n; ++i) {
            tp += b->paths[i];
            b->max_levels = std::max(b->max_levels, items[i].opts.max_bounces + 1);
            b->any_grad = b->any_grad || b->host_items[i].grad != nullptr;
        }
        const long long cap = std::max<long long>(1, std::min<long long>(kBatchWaveCap, tp));
        if (cudaMalloc(&b->bw_mem, AdjWave::bytes(cap, b->max_levels)) == cudaSuccess) {
            b->bw.carve(b->bw_mem, cap, b->max_levels);
        } else {
            cudaGetLastError();  // no room: the other schedules only
            b->bw_mem = nullptr;
        }
    }
    b->order.resize(n);
    std::iota(b->order.begin(), b->order.end(), 0);
    b->chunk = 128;
    b->stats.grid_blocks = b->grid;
    b->stats.blocks_per_sm = per_sm;
    if (flags & DTRT_BATCH_WAVEFRONT) {
        if (!b->bw_mem) {
            set_last_error("batch wavefront: no device memory for its workspace");
            return DTRT_ERR_CUDA;
        }
        b->schedule = 2;
    } else if (flags & (DTRT_BATCH_AUTOTUNE | DTRT_BATCH_TUNE_FULL)) {
        int rc = autotune(b.get(), st);
        if (!rc && (flags & DTRT_BATCH_TUNE_FULL)) rc = autotune_full(b.get(), st);
        if (rc) return rc;
        DT_BCK(cudaStreamSynchronize(st));
    }
    b->stats.chunk_paths = b->chunk;
    b->stats.schedule = b->schedule;
    b->stats.streams = b->schedule == 1 ? b->nstreams : 1;
    b->stats.wave_capacity = b->bw_mem ? b->bw.cap : 0;
    for (int i = 0; i < n && i < DTRT_BATCH_MAX_ITEMS; ++i) b->stats.order[i] = b->order[i];
    b->stats.num_items = n;
    b->stats.vertex_items = (int)b->vert_items.size();
    long long tp = 0;
    for (long long p : b->paths) tp += p;
    b->stats.total_paths = (uint64_t)tp;
    std::vector<long long> cbeg;
    long long total = 0;
    layout(b.get(), b->order, b->chunk, 1, cbeg, total);
    b->total_chunks = total;
    if (flags & DTRT_BATCH_GRAPH) {
        DT_BCK(cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking));
        int rc = capture(b.get());
        if (rc) return rc;
        b->stats.graph = 1;
    }
    *out = b.release();
    return DTRT_OK;
}

int dtrt_batch_launch(dtrt_batch *b, void *stream) {
    using namespace dt;
    if (!b) {
        set_last_error("null batch");
        return DTRT_ERR_INVALID;
    }
    cudaStream_t st = (cudaStream_t)stream;
    if (b->exec) {
        DT_BCK(cudaGraphLaunch(b->exec, st));
    } else {
        int rc = zero_outputs(b, st);
        if (!rc) rc = launch_schedule(b, st, 1);
        if (rc) return rc;
        if (b->n_img > 0) {
            k_batch_image<<<(unsigned)((b->total_pix + 255) / 256), 256, 0, st>>>(b->d_imgs, b->n_img, b->total_pix);
            DT_BCK(cudaGetLastError());
        }
    }
    // vertex items: the vertex-position replay of each (its chunking reads queue counts on
    // the host, so it runs outside the captured graph), on the same stream
    for (int i : b->vert_items) {
        const dtrt_batch_item &it = b->items[i];
        const int rc = render_vertex_adjoint(it.scene, &it.opts, it.d_image, it.image, it.d_vertices, 1, st);
        if (rc) return rc;
    }
    unsigned int herr = 0;
    DT_BCK(cudaMemcpyAsync(&herr, b->d_err, 4, cudaMemcpyDeviceToHost, st));
    DT_BCK(cudaStreamSynchronize(st));
    if (herr & ERR_STACK) {
        set_last_error("BVH traversal stack overflow");
        return DTRT_ERR_INVALID;
    }
    if (herr & ERR_TRACK_CAP) {
        set_last_error("a delta/ratio tracking loop hit its iteration cap");
        return DTRT_ERR_STEP_CAP;
    }
    return DTRT_OK;
}

int dtrt_batch_stats_get(const dtrt_batch *b, dtrt_batch_stats *out) {
    if (!b || !out) {
        dt::set_last_error("null argument");
        return DTRT_ERR_INVALID;
    }
    *out = b->stats;
    return DTRT_OK;
}

int dtrt_batch_destroy(dtrt_batch *b) {
    if (!b) return DTRT_OK;
    dt::free_batch(b);
    delete b;
    return DTRT_OK;
}

}  // extern "C"
