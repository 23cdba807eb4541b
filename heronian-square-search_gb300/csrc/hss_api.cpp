// hss_api.cpp - C ABI over the sm_103a search kernels (include/hss.h).
//
// Replaces the reference's in-process boundary: Search::prepare builds the
// factor cache (gpu_search_v42.cu:354-391), Search::run uploads it and loops
// launch / synchronise / harvest over batches of at most 512 roots
// (gpu_search_v42.cu:393-495).  Here the cache is built once per handle on all
// host threads and stays resident; each search call is one launch sequence on
// a private stream (batched: items built on the host, one persistent launch,
// one shared-prime launch; plain: one launch per <= 512 roots), timed with
// CUDA events, and its counters and hits are copied back once.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>
#include <time.h>

#include <algorithm>
#include <array>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "hss_api_status.h"
#include "hss_ctx.h"
#include "hss_kernels.h"
#include "hss_prep.h"

using namespace hss;

namespace {

constexpr uint32_t kDefaultHitCap = 4096;      // gpu_search_v42.cu:177-178
constexpr uint32_t kPlainBatch = 512;          // gpu_search_v42.cu:457
constexpr uint32_t kDefaultItemTarget = 1u << 23;
constexpr uint32_t kTileCap = 16384;           // largest m-range of one item
constexpr uint32_t kTileMin = 32;
constexpr uint32_t kBucketShift = 10;          // item ordering granularity in m
constexpr uint64_t kMergedCap = 96ull << 20;   // shared-prime queue entries
constexpr uint32_t kDescChunk = 1u << 24;       // shared-prime pairs set up per chunk (192 bytes each: 3 GB)


}  // namespace

namespace {

int fail(hss_t* h, int status, const std::string& msg) {
    if (h) h->err = msg;
    return status;
}

#define HSS_CUDA(h, call)                                                                      \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return fail(h, HSS_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

uint64_t now_ns() {
    timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (uint64_t)ts.tv_sec * 1000000000ull + (uint64_t)ts.tv_nsec;
}

template <class T>
int device_alloc(hss_t* h, T** out, size_t count) {
    void* p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    if (e != cudaSuccess) return fail(h, HSS_ERR_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    h->allocations.push_back(p);
    *out = static_cast<T*>(p);
    return HSS_OK;
}

void device_free(hss_t* h, void* p) {
    if (!p) return;
    auto it = std::find(h->allocations.begin(), h->allocations.end(), p);
    if (it != h->allocations.end()) h->allocations.erase(it);
    cudaFree(p);
}

template <class T>
int upload(hss_t* h, T** out, const T* src, size_t count) {
    int s = device_alloc(h, out, count);
    if (s) return s;
    HSS_CUDA(h, cudaMemcpy(*out, src, count * sizeof(T), cudaMemcpyHostToDevice));
    return HSS_OK;
}

uint32_t free_count(const hss_t* h, uint64_t x) { return h->seg_off[x + 1] - h->seg_off[x] - 1; }

// Upper bound on the pairs of row l that share a split prime with m in
// [l, N]: inclusion-exclusion over the distinct split primes of l.
uint64_t merged_bound(const hss_t* h, uint64_t l) {
    NumberFactors f = factor_number(h->spf.data(), l);
    if (f.count == 0) return 0;
    uint64_t n = h->limit, total = 0;
    for (uint32_t mask = 1; mask < (1u << f.count); ++mask) {
        uint64_t prod = 1;
        int bits = 0;
        bool over = false;
        for (uint32_t i = 0; i < f.count; ++i)
            if (mask & (1u << i)) {
                prod *= f.primes[i];
                ++bits;
                if (prod > n) over = true;
            }
        if (over) continue;
        uint64_t cnt = n / prod - (l - 1) / prod;
        if (bits & 1) total += cnt;
        else total -= cnt;
    }
    return total;
}

int ensure_rows(hss_t* h, size_t rows) {
    if (rows <= h->rows_cap) return HSS_OK;
    device_free(h, h->d_rows);
    h->d_rows = nullptr;
    size_t cap = std::max(rows, (size_t)1024);
    int s = device_alloc(h, &h->d_rows, cap);
    if (s) return s;
    h->rows_cap = cap;
    if (h->h_rows) cudaFreeHost(h->h_rows);
    h->h_rows = nullptr;
    HSS_CUDA(h, cudaMallocHost(&h->h_rows, cap * sizeof(RowCounts)));
    h->h_rows_cap = cap;
    return HSS_OK;
}

// Grows the shared-prime queue (entries of 16 bytes) to hold `n` pairs.
int ensure_merged(hss_t* h, uint64_t n) {
    if (n <= h->merged_cap) return HSS_OK;
    if (n >= UINT32_MAX) return fail(h, HSS_ERR_OVERFLOW, "shared-prime queue beyond 32-bit indexing");
    HSS_CUDA(h, cudaStreamSynchronize(h->stream));
    device_free(h, h->d_merged);
    h->d_merged = nullptr;
    uint64_t cap = n + n / 8;
    if (cap >= UINT32_MAX) cap = UINT32_MAX - 1;
    int s = device_alloc(h, &h->d_merged, (size_t)cap);
    if (s) return s;
    h->merged_cap = (uint32_t)cap;
    return HSS_OK;
}

// A launch group whose exact work outgrew the exact queue, or whose big
// shared-prime pairs outgrew the big-pair queue, is incomplete: the queue
// that overflowed is enlarged 4x (exact: up to 2^28 items; big pairs: up to
// 2^24 descriptors of 192 bytes) and the caller runs the whole call again.
int grow_overflowed(hss_t* h) {
    if (!h->exact_overflow && !h->big_overflow) return HSS_ERR_OVERFLOW;
    HSS_CUDA(h, cudaStreamSynchronize(h->stream));
    if (h->exact_overflow) {
        h->exact_overflow = false;
        const uint64_t cap = (uint64_t)h->exact_cap * 4;
        if (cap > (1ull << 28)) return HSS_ERR_OVERFLOW;
        device_free(h, h->d_exact);
        h->d_exact = nullptr;
        if (int s = device_alloc(h, &h->d_exact, (size_t)cap)) return s;
        h->exact_cap = (uint32_t)cap;
    }
    if (h->big_overflow) {
        h->big_overflow = false;
        const uint64_t cap = (uint64_t)h->big_cap * 4;
        if (cap > (1ull << 24)) return HSS_ERR_OVERFLOW;
        device_free(h, h->d_big);
        h->d_big = nullptr;
        if (int s = device_alloc(h, &h->d_big, (size_t)cap * kBigEntryWords)) return s;
        h->big_cap = (uint32_t)cap;
    }
    return HSS_OK;
}

// Runs `call` again after enlarging the queue that overflowed (4x per rerun;
// h->call_reruns counts the reruns).
template <class Call>
int with_exact_retry(hss_t* h, Call call) {
    for (uint32_t attempt = 0;; ++attempt) {
        h->exact_overflow = h->big_overflow = false;
        h->call_reruns = attempt;
        const int s = call();
        if (s == HSS_ERR_OVERFLOW && (h->exact_overflow || h->big_overflow) && grow_overflowed(h) == HSS_OK)
            continue;
        return s;
    }
}

int ensure_items(hss_t* h, size_t n) {
    if (n > h->items_cap) {
        device_free(h, h->d_items);
        h->d_items = nullptr;
        size_t cap = std::max(n + n / 4, (size_t)1 << 16);
        int s = device_alloc(h, &h->d_items, cap);
        if (s) return s;
        h->items_cap = cap;
    }
    if (n > h->h_items_cap) {
        if (h->h_items) cudaFreeHost(h->h_items);
        h->h_items = nullptr;
        size_t cap = std::max(n + n / 4, (size_t)1 << 16);
        HSS_CUDA(h, cudaMallocHost(&h->h_items, cap * sizeof(WorkItem)));
        h->h_items_cap = cap;
    }
    return HSS_OK;
}

// The buffers of one launch sequence (hits, control words, the shared-prime,
// big-pair, descriptor and exact-work queues, row counters), its stream and
// call events.  A handle has one set; serving gives each of its lanes another
// set over the same cache.
int alloc_launch_buffers(hss_t* h) {
    h->hit_cap = h->opts.hit_capacity ? h->opts.hit_capacity : kDefaultHitCap;
    h->merged_cap = (uint32_t)kMergedCap;
    h->big_cap = 1u << 20;
    h->desc_chunk = kDescChunk;
    h->exact_cap = h->opts.exact_capacity ? std::min<uint32_t>(h->opts.exact_capacity, 1u << 28) : 1u << 24;
    int s;
    if ((s = device_alloc(h, &h->d_hits, h->hit_cap)) || (s = device_alloc(h, &h->d_ctrl, 8)) ||
        (s = device_alloc(h, &h->d_merged, h->merged_cap)) ||
        (s = device_alloc(h, &h->d_big, (size_t)h->big_cap * kBigEntryWords)) ||
        (s = device_alloc(h, &h->d_desc, (size_t)h->desc_chunk * kBigEntryWords)) ||
        (s = device_alloc(h, &h->d_exact, h->exact_cap)) || (s = ensure_rows(h, 1024)))
        return s;
    if ((!h->stream && cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) ||
        cudaEventCreate(&h->ev0) != cudaSuccess || cudaEventCreate(&h->ev1) != cudaSuccess)
        return fail(h, HSS_ERR_CUDA, "stream or event creation failed");
    return HSS_OK;
}

LaunchBuffers buffers(const hss_t* h, size_t row_offset) {
    LaunchBuffers b;
    b.rows = h->d_rows + row_offset;
    b.hits = h->d_hits;
    b.hit_count = h->d_ctrl + 0;
    b.hit_cap = h->hit_cap;
    b.merged_queue = h->d_merged;
    b.merged_count = h->d_ctrl + 1;
    b.merged_cap = h->merged_cap;
    b.next_item = h->d_ctrl + 2;
    b.error_flags = h->d_ctrl + 3;
    b.tables = h->d_tables;
    b.row_info = h->d_row_info + row_offset;
    b.exact_queue = h->d_exact;
    b.exact_count = h->d_ctrl + 5;
    b.exact_cap = h->exact_cap;
    b.big_queue = h->d_big;
    b.big_count = h->d_ctrl + 4;
    b.big_next = h->d_ctrl + 6;
    b.big_cap = h->big_cap;
    b.pair_desc = h->d_desc;
    b.desc_chunk = h->desc_chunk;
    b.desc_next = h->d_ctrl + 7;
    return b;
}

int take_events(hss_t* h, std::array<cudaEvent_t, 3>* out) {
    for (int i = 0; i < 3; ++i) {
        if (h->events_used == h->event_pool.size()) {
            cudaEvent_t e;
            HSS_CUDA(h, cudaEventCreate(&e));
            h->event_pool.push_back(e);
        }
        (*out)[i] = h->event_pool[h->events_used++];
    }
    return HSS_OK;
}

// A row of a launch: root l and its index in the call's row counters.
struct RowRef {
    uint64_t l;
    uint32_t index;
};

// Work items of the given rows: each row's m-range [l, N] cut into ranges of
// about item_target alpha*beta evaluations (at most kTileCap roots), then
// ordered by m so that concurrently running items read the same m-side
// records from L2; the last wave is cut finer.  Returns the number of items
// and sets *alpha_cap to the largest row segment.
size_t build_items(hss_t* h, const RowRef* rows, size_t nrows, uint32_t* alpha_cap, uint32_t min_tile) {
    const uint64_t n = h->limit;
    const uint32_t target = h->opts.item_target ? h->opts.item_target : kDefaultItemTarget;
    std::vector<uint32_t> tile(nrows);
    size_t total = 0;
    uint32_t acap = 1;
    for (size_t r = 0; r < nrows; ++r) {
        uint64_t l = rows[r].l;
        uint32_t na = free_count(h, l) + 1;
        acap = std::max(acap, na);
        double per_m = (double)(h->seg_off[n + 1] - h->seg_off[l]) / (double)(n - l + 1);
        double t = (double)target / ((double)na * std::max(per_m, 1.0));
        uint32_t tm = t >= kTileCap ? kTileCap : (uint32_t)t;
        tm = std::max(min_tile, tm & ~(kTileMin - 1));
        tile[r] = tm;
        total += (n - l + 1 + tm - 1) / tm;
    }
    // the last wave of items (four per SM: two per CTA of the default shape)
    // is cut in four, so that the CTAs run out of work closer together
    const size_t tail = std::min(total, (size_t)h->sm_count * 4);
    if (ensure_items(h, total + 3 * tail)) return (size_t)-1;
    // counting sort by m-bucket of the item start
    const size_t nb = (n >> kBucketShift) + 2;
    std::vector<uint32_t> count(nb + 1, 0);
    for (size_t r = 0; r < nrows; ++r)
        for (uint64_t m = rows[r].l; m <= n; m += tile[r]) ++count[(m >> kBucketShift) + 1];
    for (size_t b = 1; b <= nb; ++b) count[b] += count[b - 1];
    for (size_t r = 0; r < nrows; ++r) {
        uint64_t l = rows[r].l;
        for (uint64_t m = l; m <= n; m += tile[r]) {
            uint64_t m1 = std::min<uint64_t>(m + tile[r], n + 1);
            h->h_items[count[m >> kBucketShift]++] =
                WorkItem{(uint32_t)l, (uint32_t)m, (uint32_t)m1, rows[r].index};
        }
    }
    std::vector<WorkItem> last(h->h_items + total - tail, h->h_items + total);
    size_t pos = total - tail;
    for (const WorkItem& it : last) {
        const uint32_t q = (it.m1 - it.m0 + 3) / 4;
        for (uint32_t s = it.m0; s < it.m1; s += q)
            h->h_items[pos++] = WorkItem{it.l, s, std::min(s + q, it.m1), it.row};
    }
    *alpha_cap = acap;
    return pos;
}

// Constants of the call's rows (row i of the call at index i).
int upload_row_info(hss_t* h, const std::vector<uint64_t>& ls) {
    if (ls.size() > h->row_info_cap) {
        HSS_CUDA(h, cudaStreamSynchronize(h->stream));
        device_free(h, h->d_row_info);
        h->d_row_info = nullptr;
        if (h->h_row_info) cudaFreeHost(h->h_row_info);
        h->h_row_info = nullptr;
        size_t cap = std::max(ls.size(), (size_t)1024);
        int s = device_alloc(h, &h->d_row_info, cap);
        if (s) return s;
        HSS_CUDA(h, cudaMallocHost(&h->h_row_info, cap * sizeof(RowInfo)));
        h->row_info_cap = cap;
    }
    HSS_CUDA(h, cudaStreamSynchronize(h->stream));
    for (size_t i = 0; i < ls.size(); ++i)
        fill_row_info(h->spf.data(), h->seg_off.data(), h->limit, ls[i], &h->h_row_info[i]);
    HSS_CUDA(h, cudaMemcpyAsync(h->d_row_info, h->h_row_info, ls.size() * sizeof(RowInfo), cudaMemcpyHostToDevice,
                                h->stream));
    h->h2d_bytes += ls.size() * sizeof(RowInfo);
    return HSS_OK;
}

[[maybe_unused]] int check_errors(hss_t* h) {
    unsigned int ctrl[4];
    HSS_CUDA(h, cudaMemcpy(ctrl, h->d_ctrl, sizeof ctrl, cudaMemcpyDeviceToHost));
    if (ctrl[3] & 1u) return fail(h, HSS_ERR_OVERFLOW, "shared-prime queue over capacity");
    if (ctrl[3] & 2u) return fail(h, HSS_ERR_OVERFLOW, "shared-prime pair exceeds the list capacity");
    return HSS_OK;
}

// Captures the stream work of `enqueue` in a CUDA graph and launches it.  The
// handle keeps one executable graph and updates it in place from each new
// capture (item count, grid and buffer sizes change between calls); when the
// update is refused, the graph is instantiated again.
template <class Enqueue>
int run_captured(hss_t* h, Enqueue enqueue) {
    HSS_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    const int s = enqueue();
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(h->stream, &g);
    if (s || ce != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        if (s) return s;
        return fail(h, HSS_ERR_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(ce));
    }
    bool updated = false;
    if (h->graph_exec) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(h->graph_exec, g, &info) == cudaSuccess) {
            updated = true;
        } else {
            cudaGetLastError();
            cudaGraphExecDestroy(h->graph_exec);
            h->graph_exec = nullptr;
        }
    }
    cudaError_t e = cudaSuccess;
    if (!updated) e = cudaGraphInstantiate(&h->graph_exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(h, HSS_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    HSS_CUDA(h, cudaGraphLaunch(h->graph_exec, h->stream));
    ++h->graph_launches;
    ++h->call_graphs;
    return HSS_OK;
}

int search_locked(hss_t* h, uint64_t first, uint64_t last, int mode, hss_counts* out, uint64_t* row_candidates,
                  hss_hit* hits, uint32_t hit_cap, uint32_t* nhits);
int search_many_locked(hss_t* h, const uint64_t* firsts, const uint64_t* lasts, uint32_t count, size_t rows,
                       hss_counts* per_interval, hss_counts* total, hss_hit* hits, uint32_t hit_cap,
                       uint32_t* nhits);

// Launches the batched sequence for a set of rows whose shared-prime pairs
// fit the queue: reset cursor/queue, items H2D, persistent kernel, shared-prime
// kernel.  Counters accumulate into d_rows[index].
int run_batched_rows(hss_t* h, const RowRef* rows, size_t nrows) {
    // the pinned item buffer may still be read by the previous group's copy
    HSS_CUDA(h, cudaStreamSynchronize(h->stream));
    uint32_t acap = 1;
    const int threads = h->opts.block_threads ? (int)h->opts.block_threads : 256;
    // every warp of a CTA claims 128 roots at a time: items span at least that
    size_t n_items = build_items(h, rows, nrows, &acap, (uint32_t)threads / 32 * 128);
    if (n_items == (size_t)-1) return HSS_ERR_MEMORY;
    if (n_items == 0) return HSS_OK;
    BatchedConfig cfg;
    cfg.threads = h->opts.block_threads ? (int)h->opts.block_threads : 256;
    cfg.min_blocks = h->opts.ctas_per_sm ? (int)h->opts.ctas_per_sm : (cfg.threads == 128 ? 4 : cfg.threads == 512 ? 1 : 2);
    cfg.alpha_cap = acap;
    size_t smem = batched_smem_bytes(cfg.threads, acap);
    int per_sm = batched_max_ctas_per_sm(cfg.threads, cfg.min_blocks, smem);
    cfg.ctas = h->sm_count * per_sm;
    LaunchBuffers b = buffers(h, 0);
    uint64_t pair_bound = 0;  // sets how many shared-prime chunks are launched
    for (size_t i = 0; i < nrows; ++i) pair_bound += merged_bound(h, rows[i].l);
    std::array<cudaEvent_t, 3> ev;
    if (int e = take_events(h, &ev)) return e;
    // the group's stream work: items H2D, queue resets, the three kernels.
    // Inside a capture the timing events become event-record nodes
    // (cudaEventRecordExternal), so they still time the graph's kernels.
    const unsigned int rec = h->opts.use_graph ? cudaEventRecordExternal : cudaEventRecordDefault;
    uint32_t merged_launches = 0;
    auto enqueue = [&]() -> int {
        HSS_CUDA(h, cudaMemcpyAsync(h->d_items, h->h_items, n_items * sizeof(WorkItem), cudaMemcpyHostToDevice,
                                    h->stream));
        HSS_CUDA(h, cudaMemsetAsync(h->d_ctrl + 1, 0, 2 * sizeof(unsigned int), h->stream));
        HSS_CUDA(h, cudaMemsetAsync(h->d_ctrl + 4, 0, 3 * sizeof(unsigned int), h->stream));
        HSS_CUDA(h, cudaEventRecordWithFlags(ev[0], h->stream, rec));
        HSS_CUDA(h, launch_batched(h->dev, h->d_items, (uint32_t)n_items, cfg, b, h->stream));
        HSS_CUDA(h, cudaEventRecordWithFlags(ev[1], h->stream, rec));
        HSS_CUDA(h, launch_merged(h->dev, pair_bound, b, h->sm_count * 4, h->stream, &merged_launches));
        HSS_CUDA(h, launch_exact(h->dev, b, h->sm_count * 4, h->stream));
        HSS_CUDA(h, cudaEventRecordWithFlags(ev[2], h->stream, rec));
        return HSS_OK;
    };
    if (h->opts.use_graph) {
        if (int e = run_captured(h, enqueue)) return e;
    } else if (int e = enqueue()) {
        return e;
    }
    h->h2d_bytes += n_items * sizeof(WorkItem);
    h->marks.push_back(ev);
    h->launches += 2 + merged_launches;  // batched, shared-prime kernels, exact
    return HSS_OK;
}

// Splits rows into groups whose shared-prime bound fits the queue.
int run_batched(hss_t* h, const std::vector<RowRef>& rows) {
    size_t start = 0;
    while (start < rows.size()) {
        uint64_t bound = 0;
        size_t end = start;
        while (end < rows.size()) {
            uint64_t b = merged_bound(h, rows[end].l);
            if (end > start && bound + b > h->merged_cap) break;
            bound += b;
            ++end;
        }
        if (bound > h->merged_cap) return fail(h, HSS_ERR_OVERFLOW, "row exceeds the shared-prime queue");
        int s = run_batched_rows(h, rows.data() + start, end - start);
        if (s) return s;
        start = end;
    }
    return HSS_OK;
}

int run_plain(hss_t* h, uint64_t first, uint64_t last) {
    for (uint64_t b = first; b <= last; b += kPlainBatch) {
        uint32_t nrows = (uint32_t)std::min<uint64_t>(kPlainBatch, last - b + 1);
        uint64_t bound = 0;
        uint32_t acap = 1;
        for (uint64_t l = b; l < b + nrows; ++l) {
            bound += merged_bound(h, l);
            acap = std::max(acap, free_count(h, l) + 1);
        }
        if (bound > h->merged_cap) {
            int g = ensure_merged(h, bound);
            if (g) return g;
        }
        HSS_CUDA(h, cudaMemsetAsync(h->d_ctrl + 1, 0, sizeof(unsigned int), h->stream));
        HSS_CUDA(h, cudaMemsetAsync(h->d_ctrl + 4, 0, 3 * sizeof(unsigned int), h->stream));
        LaunchBuffers buf = buffers(h, b - first);
        std::array<cudaEvent_t, 3> ev;
        if (int e = take_events(h, &ev)) return e;
        HSS_CUDA(h, cudaEventRecord(ev[0], h->stream));
        HSS_CUDA(h, launch_plain(h->dev, b, nrows, acap, buf, h->stream));
        HSS_CUDA(h, cudaEventRecord(ev[1], h->stream));
        uint32_t merged_launches = 0;
        HSS_CUDA(h, launch_merged(h->dev, bound, buf, h->sm_count * 4, h->stream, &merged_launches));
        HSS_CUDA(h, launch_exact(h->dev, buf, h->sm_count * 4, h->stream));
        HSS_CUDA(h, cudaEventRecord(ev[2], h->stream));
        h->marks.push_back(ev);
        h->launches += 2 + merged_launches;  // plain, shared-prime kernels, exact
    }
    return HSS_OK;
}

int begin_call(hss_t* h, size_t rows) {
    int s = ensure_rows(h, rows);
    if (s) return s;
    HSS_CUDA(h, cudaMemsetAsync(h->d_rows, 0, rows * sizeof(RowCounts), h->stream));
    HSS_CUDA(h, cudaMemsetAsync(h->d_ctrl, 0, 8 * sizeof(unsigned int), h->stream));
    HSS_CUDA(h, cudaEventRecord(h->ev0, h->stream));
    h->events_used = 0;
    h->marks.clear();
    h->launches = 0;
    h->call_graphs = 0;
    h->h2d_bytes = h->d2h_bytes = 0;
    return HSS_OK;
}

// Copies row counters and hits back; hits sorted by (l, m, n) and deduplicated.
int end_call(hss_t* h, size_t rows, double* ms, std::vector<DevHit>* hits, uint32_t* found,
             double* main_ms = nullptr, double* merged_ms = nullptr) {
    HSS_CUDA(h, cudaEventRecord(h->ev1, h->stream));
    HSS_CUDA(h, cudaMemcpyAsync(h->h_rows, h->d_rows, rows * sizeof(RowCounts), cudaMemcpyDeviceToHost,
                                h->stream));
    unsigned int ctrl[4];
    HSS_CUDA(h, cudaMemcpyAsync(ctrl, h->d_ctrl, sizeof ctrl, cudaMemcpyDeviceToHost, h->stream));
    HSS_CUDA(h, cudaStreamSynchronize(h->stream));
    float f = 0;
    HSS_CUDA(h, cudaEventElapsedTime(&f, h->ev0, h->ev1));
    *ms = f;
    double t_main = 0, t_merged = 0;
    for (auto& ev : h->marks) {
        float a = 0, b = 0;
        HSS_CUDA(h, cudaEventElapsedTime(&a, ev[0], ev[1]));
        HSS_CUDA(h, cudaEventElapsedTime(&b, ev[1], ev[2]));
        t_main += a;
        t_merged += b;
    }
    if (main_ms) *main_ms = t_main;
    if (merged_ms) *merged_ms = t_merged;
    h->d2h_bytes += rows * sizeof(RowCounts) + sizeof ctrl;
    if (ctrl[3] & 1u) return fail(h, HSS_ERR_OVERFLOW, "shared-prime queue over capacity");
    if (ctrl[3] & 2u) return fail(h, HSS_ERR_OVERFLOW, "shared-prime pair exceeds the list capacity");
    if (ctrl[3] & 12u) {
        h->exact_overflow = (ctrl[3] & 4u) != 0;
        h->big_overflow = (ctrl[3] & 8u) != 0;
        return fail(h, HSS_ERR_OVERFLOW, "exact work or big-pair queue over capacity");
    }
    if (ctrl[3] & ~15u) return fail(h, HSS_ERR_OVERFLOW, "a device index check failed (an event index out of range)");
    uint32_t nh = std::min(ctrl[0], h->hit_cap);
    hits->resize(nh);
    if (nh) HSS_CUDA(h, cudaMemcpy(hits->data(), h->d_hits, nh * sizeof(DevHit), cudaMemcpyDeviceToHost));
    h->d2h_bytes += nh * sizeof(DevHit);
    std::sort(hits->begin(), hits->end(), [](const DevHit& a, const DevHit& b) {
        if (a.l != b.l) return a.l < b.l;
        if (a.m != b.m) return a.m < b.m;
        return a.n < b.n;
    });
    hits->erase(std::unique(hits->begin(), hits->end(),
                            [](const DevHit& a, const DevHit& b) { return a.l == b.l && a.m == b.m && a.n == b.n; }),
                hits->end());
    *found = ctrl[0] > h->hit_cap ? ctrl[0] : (uint32_t)hits->size();
    return HSS_OK;
}

void add_row(hss_counts* c, const RowCounts& r) {
    c->processed += r.processed;
    c->products += r.products;
    c->candidates += r.candidates;
    c->r16 += r.r16;
    c->exact += r.exact;
    c->merged += r.merged;
    c->merged_products += r.mproducts;
    c->merged_candidates += r.mcandidates;
    c->merged_r16 += r.mr16;
}

void copy_hits(const std::vector<DevHit>& in, hss_hit* out, uint32_t cap) {
    for (size_t i = 0; i < in.size() && i < cap; ++i) {
        out[i].l = in[i].l;
        out[i].m = in[i].m;
        out[i].n = in[i].n;
        out[i].area4_lo = in[i].area4_lo;
        out[i].area4_hi = in[i].area4_hi;
        out[i].heron_ok = in[i].heron_ok;
        out[i].reserved = 0;
    }
}

}  // namespace

// ------------------------------------------------------------------ exports

extern "C" {

const char* hss_version(void) { return "hss-gb300 1.0 (sm_103a)"; }

const char* hss_strerror(int status) {
    switch (status) {
        case HSS_OK: return "ok";
        case HSS_ERR_ARGUMENT: return "invalid argument";
        case HSS_ERR_CUDA: return "CUDA error";
        case HSS_ERR_MEMORY: return "out of memory";
        case HSS_ERR_LIMIT: return "limit not supported";
        case HSS_ERR_STATE: return "checkpoint does not match requested range";
        case HSS_ERR_OVERFLOW: return "internal capacity exceeded";
        case HSS_ERR_NOT_FOUND: return "unknown request";
        case HSS_ERR_BUSY: return "request still running";
        case HSS_ERR_NO_DEVICE: return "no sm_103 CUDA device";
        default: return "unknown status";
    }
}

const char* hss_last_error(const hss_t* h) { return h ? h->err.c_str() : "null handle"; }

int hss_cache_check(uint64_t limit, int device, uint64_t* mismatches, double* host_seconds,
                    double* device_seconds) {
    if (!mismatches || limit < 1 || limit > HSS_MAX_LIMIT) return HSS_ERR_ARGUMENT;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev || cudaSetDevice(device) != cudaSuccess)
        return HSS_ERR_NO_DEVICE;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return HSS_ERR_NO_DEVICE;
    HostCache hc;
    std::string err;
    unsigned hw = std::thread::hardware_concurrency();
    int s = build_host_cache(limit, (int)(hw ? hw : 1), &hc, &err);
    if (s) return s;
    cudaStream_t st = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return HSS_ERR_CUDA;
    DeviceBuild db;
    s = build_device_cache(limit, prop.multiProcessorCount, st, &db, &err);
    cudaStreamDestroy(st);
    if (s) return s;
    uint64_t bad = 0;
    auto compare = [&](const void* dev, const void* host, size_t count, size_t elem) -> int {
        std::vector<unsigned char> copy(count * elem);
        if (count && cudaMemcpy(copy.data(), dev, count * elem, cudaMemcpyDeviceToHost) != cudaSuccess)
            return HSS_ERR_CUDA;
        const unsigned char* h = static_cast<const unsigned char*>(host);
        for (size_t i = 0; i < count; ++i)
            if (memcmp(copy.data() + i * elem, h + i * elem, elem) != 0) ++bad;
        return HSS_OK;
    };
    bad += (db.records != hc.records) + (db.pp_count != hc.pp_hot.size()) +
           (db.reference_flattened != hc.reference_flattened) + (db.reference_cached != hc.reference_cached) +
           (db.max_exponent != hc.max_exponent);
    if (!bad) {
        if ((s = compare(db.spf, hc.spf.data(), hc.spf.size(), sizeof(uint32_t))) ||
            (s = compare(db.seg_off, hc.seg_off.data(), hc.seg_off.size(), sizeof(uint32_t))) ||
            (s = compare(db.hot, hc.hot.get(), hc.records, sizeof(HotRec))) ||
            (s = compare(db.exact, hc.exact.get(), hc.records, sizeof(ExactRec))) ||
            (s = compare(db.owner, hc.owner.get(), hc.records, sizeof(uint32_t))) ||
            (s = compare(db.pp_base, hc.pp_base.data(), hc.pp_base.size(), sizeof(uint32_t))) ||
            (s = compare(db.pp_hot, hc.pp_hot.data(), hc.pp_hot.size(), sizeof(HotRec))) ||
            (s = compare(db.pp_exact, hc.pp_exact.data(), hc.pp_exact.size(), sizeof(__int128)))) {
            for (void* p : db.owned) cudaFree(p);
            return s;
        }
        bad += (db.spf_host != hc.spf) + (db.seg_off_host != hc.seg_off);
    }
    for (void* p : db.owned) cudaFree(p);
    *mismatches = bad;
    if (host_seconds) *host_seconds = hc.seconds;
    if (device_seconds) *device_seconds = db.seconds;
    return HSS_OK;
}

int hss_open(uint64_t limit, int device, const hss_opts* opts, hss_t** out) {
    if (!out) return HSS_ERR_ARGUMENT;
    *out = nullptr;
    if (limit < 1 || limit > HSS_MAX_LIMIT) return HSS_ERR_LIMIT;
    hss_t* h = new hss_t();
    if (opts) h->opts = *opts;
    h->device = device;
    h->limit = limit;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        delete h;
        return HSS_ERR_NO_DEVICE;
    }
    cudaDeviceProp prop;
    if (cudaSetDevice(device) != cudaSuccess || cudaGetDeviceProperties(&prop, device) != cudaSuccess ||
        prop.major != 10 || prop.minor != 3) {
        delete h;
        return HSS_ERR_NO_DEVICE;
    }
    h->sm_count = prop.multiProcessorCount;
    int s = HSS_OK;
    if (!h->opts.host_build) {
        // the cache built by kernels on the device (same arrays and values as the host build)
        if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete h;
            return HSS_ERR_CUDA;
        }
        DeviceBuild db;
        std::string err;
        s = build_device_cache(limit, h->sm_count, h->stream, &db, &err);
        if (s) {
            hss_close(h);
            return s;
        }
        h->allocations.insert(h->allocations.end(), db.owned.begin(), db.owned.end());
        if (db.longest > kItemRecords) {
            hss_close(h);
            return HSS_ERR_LIMIT;
        }
        h->records = db.records;
        h->ref_flattened = db.reference_flattened;
        h->ref_cached = db.reference_cached;
        h->prep_seconds = db.seconds;
        h->dev.limit = limit;
        h->dev.spf = db.spf;
        h->dev.seg_off = db.seg_off;
        h->dev.hot = db.hot;
        h->dev.exact = db.exact;
        h->dev.owner = db.owner;
        h->dev.pp_base = db.pp_base;
        h->dev.pp_hot = db.pp_hot;
        h->dev.pp_exact = db.pp_exact;
        h->dev.max_exponent = db.max_exponent;
        h->seg_off = std::move(db.seg_off_host);
        h->spf = std::move(db.spf_host);
    } else {
        HostCache hc;
        std::string err;
        unsigned hw = std::thread::hardware_concurrency();
        int threads = h->opts.prep_threads ? (int)h->opts.prep_threads : (int)(hw ? hw : 1);
        s = build_host_cache(limit, threads, &hc, &err);
        if (s) {
            delete h;
            return s;
        }
        uint32_t longest = 0;
        for (uint64_t x = 1; x <= limit; ++x) longest = std::max(longest, hc.seg_off[x + 1] - hc.seg_off[x]);
        if (longest > kItemRecords) {
            delete h;
            return HSS_ERR_LIMIT;
        }
        h->records = hc.records;
        h->ref_flattened = hc.reference_flattened;
        h->ref_cached = hc.reference_cached;
        h->prep_seconds = hc.seconds;
        uint32_t *spf, *seg, *owner, *ppb;
        HotRec *hot, *pph;
        ExactRec* ex;
        __int128* ppx;
        if ((s = upload(h, &spf, hc.spf.data(), hc.spf.size())) ||
            (s = upload(h, &seg, hc.seg_off.data(), hc.seg_off.size())) ||
            (s = upload(h, &hot, hc.hot.get(), hc.records)) || (s = upload(h, &ex, hc.exact.get(), hc.records)) ||
            (s = upload(h, &owner, hc.owner.get(), hc.records)) ||
            (s = upload(h, &ppb, hc.pp_base.data(), hc.pp_base.size())) ||
            (s = upload(h, &pph, hc.pp_hot.data(), hc.pp_hot.size())) ||
            (s = upload(h, &ppx, hc.pp_exact.data(), hc.pp_exact.size()))) {
            hss_close(h);
            return s;
        }
        h->dev.limit = limit;
        h->dev.spf = spf;
        h->dev.seg_off = seg;
        h->dev.hot = hot;
        h->dev.exact = ex;
        h->dev.owner = owner;
        h->dev.pp_base = ppb;
        h->dev.pp_hot = pph;
        h->dev.pp_exact = ppx;
        h->dev.max_exponent = hc.max_exponent;
        h->seg_off = std::move(hc.seg_off);
        h->spf = std::move(hc.spf);
    }
    std::vector<uint8_t> tables(kTableTotalBytes);
    build_residue_tables(tables.data());
    if ((s = upload(h, &h->d_tables, tables.data(), kTableTotalBytes)) || (s = alloc_launch_buffers(h))) {
        hss_close(h);
        return s;
    }
    *out = h;
    return HSS_OK;
}

int hss_serve_stop(hss_t* h);

void hss_close(hss_t* h) {
    if (!h) return;
    hss_serve_stop(h);
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (void* p : h->allocations) cudaFree(p);
    if (h->h_items) cudaFreeHost(h->h_items);
    if (h->h_rows) cudaFreeHost(h->h_rows);
    if (h->h_row_info) cudaFreeHost(h->h_row_info);
    if (h->h_ctrl) cudaFreeHost(h->h_ctrl);
    if (h->h_slots) cudaFreeHost(h->h_slots);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    for (cudaEvent_t e : h->event_pool) cudaEventDestroy(e);
    if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

int hss_int32_peak(int device, double* ops_per_second, double* ms) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return HSS_ERR_NO_DEVICE;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return HSS_ERR_CUDA;
    double v = int32_peak_ops(device, prop.multiProcessorCount, ms);
    if (ops_per_second) *ops_per_second = v;
    return v > 0 ? HSS_OK : HSS_ERR_CUDA;
}

int hss_info(const hss_t* h, uint64_t* limit, uint64_t* records, uint64_t* flattened, uint64_t* cached,
             double* prep_seconds) {
    if (!h) return HSS_ERR_ARGUMENT;
    if (limit) *limit = h->limit;
    if (records) *records = h->records;
    if (flattened) *flattened = h->ref_flattened;
    if (cached) *cached = h->ref_cached;
    if (prep_seconds) *prep_seconds = h->prep_seconds;
    return HSS_OK;
}

int hss_cache_inspect(uint64_t limit, uint64_t x, uint64_t* records, uint64_t* flattened, uint64_t* cached,
                      int64_t* re, int64_t* im, uint32_t cap, uint32_t* count) {
    if (limit < 1 || limit > HSS_MAX_LIMIT || x > limit) return HSS_ERR_ARGUMENT;
    HostCache hc;
    std::string err;
    unsigned hw = std::thread::hardware_concurrency();
    int s = build_host_cache(limit, (int)(hw ? hw : 1), &hc, &err);
    if (s) return s;
    if (records) *records = hc.records;
    if (flattened) *flattened = hc.reference_flattened;
    if (cached) *cached = hc.reference_cached;
    if (x) {
        uint32_t a = hc.seg_off[x], b = hc.seg_off[x + 1];
        if (count) *count = b - a;
        for (uint32_t i = a; i < b && i - a < cap; ++i) {
            if (re) re[i - a] = hc.exact[i].re;
            if (im) im[i - a] = hc.exact[i].im;
        }
    }
    return HSS_OK;
}

int hss_search(hss_t* h, uint64_t first, uint64_t last, int mode, hss_counts* out, uint64_t* row_candidates,
               hss_hit* hits, uint32_t hit_cap, uint32_t* nhits) {
    if (!h || !out) return HSS_ERR_ARGUMENT;
    if (first < 1 || first > last || last > h->limit)
        return fail(h, HSS_ERR_ARGUMENT, "need 1 <= first <= last <= limit");
    if (mode != HSS_MODE_PLAIN && mode != HSS_MODE_BATCHED) return fail(h, HSS_ERR_ARGUMENT, "unknown mode");
    std::lock_guard<std::mutex> lock(h->gpu_mu);
    HSS_CUDA(h, cudaSetDevice(h->device));
    return with_exact_retry(h, [&] { return search_locked(h, first, last, mode, out, row_candidates, hits, hit_cap,
                                                          nhits); });
}

}  // extern "C"

namespace {

int search_locked(hss_t* h, uint64_t first, uint64_t last, int mode, hss_counts* out, uint64_t* row_candidates,
                  hss_hit* hits, uint32_t hit_cap, uint32_t* nhits) {
    const size_t rows = (size_t)(last - first + 1);
    int s = begin_call(h, rows);
    if (s) return s;
    {
        std::vector<uint64_t> ls(rows);
        for (size_t r = 0; r < rows; ++r) ls[r] = first + r;
        if ((s = upload_row_info(h, ls))) return s;
    }
    if (mode == HSS_MODE_PLAIN) {
        s = run_plain(h, first, last);
    } else {
        std::vector<RowRef> refs(rows);
        for (size_t r = 0; r < rows; ++r) refs[r] = RowRef{first + r, (uint32_t)r};
        s = run_batched(h, refs);
    }
    if (s) return s;
    std::vector<DevHit> found;
    uint32_t nfound = 0;
    double ms = 0, main_ms = 0, merged_ms = 0;
    if ((s = end_call(h, rows, &ms, &found, &nfound, &main_ms, &merged_ms))) return s;
    memset(out, 0, sizeof *out);
    out->main_ms = main_ms;
    out->merged_ms = merged_ms;
    out->launches = h->launches;
    out->graph_launches = h->call_graphs;
    out->reruns = h->call_reruns;
    out->h2d_bytes = h->h2d_bytes;
    out->d2h_bytes = h->d2h_bytes;
    for (size_t r = 0; r < rows; ++r) {
        add_row(out, h->h_rows[r]);
        out->pairs += h->limit - (first + r) + 1;
        if (row_candidates) row_candidates[r] = h->h_rows[r].candidates;
    }
    out->hits = nfound;
    out->kernel_ms = ms;
    if (hits) copy_hits(found, hits, hit_cap);
    if (nhits) *nhits = nfound;
    return HSS_OK;
}

}  // namespace

extern "C" {

int hss_autotune(hss_t* h, uint64_t first, uint64_t last, hss_opts* best, hss_tune_trial* trials,
                 uint32_t max_trials, uint32_t* ntrials) {
    if (!h) return HSS_ERR_ARGUMENT;
    static const uint32_t kVariants[][2] = {{128, 4}, {128, 6}, {256, 2}, {256, 3}, {512, 1}};
    static const uint32_t kTargets[] = {1u << 21, 1u << 22, 1u << 23, 1u << 24, 1u << 25};
    const hss_opts saved = h->opts;
    hss_opts chosen = saved;
    float best_ms = 0;
    uint32_t n = 0;
    for (const auto& v : kVariants)
        for (uint32_t target : kTargets) {
            h->opts.block_threads = v[0];
            h->opts.ctas_per_sm = v[1];
            h->opts.item_target = target;
            hss_counts c;
            int s = hss_search(h, first, last, HSS_MODE_BATCHED, &c, nullptr, nullptr, 0, nullptr);  // warm
            if (!s) s = hss_search(h, first, last, HSS_MODE_BATCHED, &c, nullptr, nullptr, 0, nullptr);
            if (s) {
                h->opts = saved;
                return s;
            }
            float ms = (float)c.kernel_ms;
            if (trials && n < max_trials) trials[n] = hss_tune_trial{v[0], v[1], target, ms};
            ++n;
            if (best_ms == 0 || ms < best_ms) {
                best_ms = ms;
                chosen = h->opts;
            }
        }
    h->opts = chosen;
    if (best) *best = chosen;
    if (ntrials) *ntrials = n;
    return HSS_OK;
}

int hss_search_many(hss_t* h, const uint64_t* firsts, const uint64_t* lasts, uint32_t count,
                    hss_counts* per_interval, hss_counts* total, hss_hit* hits, uint32_t hit_cap,
                    uint32_t* nhits) {
    if (!h || !firsts || !lasts || count == 0) return HSS_ERR_ARGUMENT;
    size_t rows = 0;
    for (uint32_t i = 0; i < count; ++i) {
        if (firsts[i] < 1 || firsts[i] > lasts[i] || lasts[i] > h->limit)
            return fail(h, HSS_ERR_ARGUMENT, "need 1 <= first <= last <= limit for every interval");
        rows += lasts[i] - firsts[i] + 1;
    }
    if (rows > UINT32_MAX) return fail(h, HSS_ERR_ARGUMENT, "too many rows");
    std::lock_guard<std::mutex> lock(h->gpu_mu);
    HSS_CUDA(h, cudaSetDevice(h->device));
    return with_exact_retry(h, [&] {
        return search_many_locked(h, firsts, lasts, count, rows, per_interval, total, hits, hit_cap, nhits);
    });
}

}  // extern "C"

namespace {

int search_many_locked(hss_t* h, const uint64_t* firsts, const uint64_t* lasts, uint32_t count, size_t rows,
                       hss_counts* per_interval, hss_counts* total, hss_hit* hits, uint32_t hit_cap,
                       uint32_t* nhits) {
    int s = begin_call(h, rows);
    if (s) return s;
    std::vector<RowRef> refs;
    std::vector<uint64_t> ls;
    refs.reserve(rows);
    ls.reserve(rows);
    for (uint32_t i = 0; i < count; ++i)
        for (uint64_t l = firsts[i]; l <= lasts[i]; ++l) {
            refs.push_back(RowRef{l, (uint32_t)refs.size()});
            ls.push_back(l);
        }
    if ((s = upload_row_info(h, ls))) return s;
    if ((s = run_batched(h, refs))) return s;
    std::vector<DevHit> found;
    uint32_t nfound = 0;
    double ms = 0, main_ms = 0, merged_ms = 0;
    if ((s = end_call(h, rows, &ms, &found, &nfound, &main_ms, &merged_ms))) return s;
    hss_counts sum{};
    sum.main_ms = main_ms;
    sum.merged_ms = merged_ms;
    sum.launches = h->launches;
    sum.graph_launches = h->call_graphs;
    sum.reruns = h->call_reruns;
    sum.h2d_bytes = h->h2d_bytes;
    sum.d2h_bytes = h->d2h_bytes;
    size_t r = 0;
    for (uint32_t i = 0; i < count; ++i) {
        hss_counts c{};
        for (uint64_t l = firsts[i]; l <= lasts[i]; ++l, ++r) {
            add_row(&c, h->h_rows[r]);
            c.pairs += h->limit - l + 1;
        }
        for (const DevHit& hit : found)
            if (hit.l >= firsts[i] && hit.l <= lasts[i]) ++c.hits;
        if (per_interval) per_interval[i] = c;
        sum.pairs += c.pairs;
        sum.processed += c.processed;
        sum.products += c.products;
        sum.candidates += c.candidates;
        sum.r16 += c.r16;
        sum.exact += c.exact;
        sum.merged += c.merged;
        sum.merged_products += c.merged_products;
        sum.merged_candidates += c.merged_candidates;
        sum.merged_r16 += c.merged_r16;
    }
    sum.hits = nfound;
    sum.kernel_ms = ms;
    if (total) *total = sum;
    if (hits) copy_hits(found, hits, hit_cap);
    if (nhits) *nhits = nfound;
    return HSS_OK;
}

}  // namespace

// ------------------------------------------------------------------ serving
//
// Continuous admission.  Requests queue at hss_submit; a background loop
// admits them while request slots and device state space are free, and runs
// waves - a bounded slice of every admitted request - on two lanes (launch
// buffers and a stream each, over the handle's cache), so one wave runs on
// the device while the host harvests the previous one and forms the next.
// Each admitted request owns a range of row records in a device arena sized
// from free HBM at serve start: every wave ends with a kernel that writes its
// row counters there, marked done, so a request's progress and counts stay
// on the device until it completes and are read back once.  Admission waits
// when the arena has no room for a request's rows.

namespace hss {

struct Request {
    uint64_t id = 0, first = 0, last = 0;
    uint64_t next_row = 0;  // next root to schedule
    uint64_t rows_done = 0;
    uint64_t inflight = 0;  // rows in waves not yet settled
    uint32_t slot = 0;      // first record of its rows in the device state arena
    uint64_t submitted_ns = 0, admitted_ns = 0, finished_ns = 0;
    double ms_weighted = 0; // wave device time x its logical pairs in the wave
    hss_counts counts{};
    std::vector<DevHit> hits;
    int status = HSS_ERR_BUSY;
    bool admitted = false;
};

// A wave on a lane: its rows (index i of the wave) and their requests.
struct Wave {
    std::vector<RowRef> rows;
    std::vector<Request*> owner;
    bool live = false;
};

}  // namespace hss

namespace {

// A lane: a second set of launch buffers and a stream over h's cache (the
// cache arrays and residue tables are shared, not owned).
hss_t* make_lane(hss_t* h, int* status) {
    hss_t* lane = new hss_t();
    lane->device = h->device;
    lane->limit = h->limit;
    lane->opts = h->opts;
    lane->opts.use_graph = 0;
    lane->sm_count = h->sm_count;
    lane->seg_off = h->seg_off;
    lane->spf = h->spf;
    lane->dev = h->dev;
    lane->d_tables = h->d_tables;
    int s = alloc_launch_buffers(lane);
    if (!s && cudaMallocHost(&lane->h_ctrl, 8 * sizeof(unsigned int)) != cudaSuccess) s = HSS_ERR_MEMORY;
    if (s) {
        hss_close(lane);
        *status = s;
        return nullptr;
    }
    *status = HSS_OK;
    return lane;
}

int ensure_slots(hss_t* lane, size_t n) {
    if (n <= lane->slots_cap) return HSS_OK;
    device_free(lane, lane->d_slots);
    lane->d_slots = nullptr;
    if (lane->h_slots) cudaFreeHost(lane->h_slots);
    lane->h_slots = nullptr;
    const size_t cap = std::max(n, (size_t)1024);
    int s = device_alloc(lane, &lane->d_slots, cap);
    if (s) return s;
    HSS_CUDA(lane, cudaMallocHost(&lane->h_slots, cap * sizeof(uint32_t)));
    lane->slots_cap = cap;
    return HSS_OK;
}

// Enqueues a wave on its (idle) lane: row constants, the batched launch
// groups, the scatter of its row counters into the requests' device state,
// and the read-back of the control words.  Returns without waiting for the
// device.
int launch_wave(hss_t* h, hss_t* lane, const Wave& w) {
    const size_t n = w.rows.size();
    int s = begin_call(lane, n);
    if (s) return s;
    std::vector<uint64_t> ls(n);
    for (size_t i = 0; i < n; ++i) ls[i] = w.rows[i].l;
    if ((s = upload_row_info(lane, ls)) || (s = ensure_slots(lane, n))) return s;
    for (size_t i = 0; i < n; ++i) lane->h_slots[i] = w.owner[i]->slot + (uint32_t)(w.rows[i].l - w.owner[i]->first);
    HSS_CUDA(lane, cudaMemcpyAsync(lane->d_slots, lane->h_slots, n * sizeof(uint32_t), cudaMemcpyHostToDevice,
                                   lane->stream));
    if ((s = run_batched(lane, w.rows))) return s;
    HSS_CUDA(lane, launch_scatter_rows(lane->d_rows, lane->d_slots, (uint32_t)n, h->d_state, lane->stream));
    HSS_CUDA(lane, cudaEventRecord(lane->ev1, lane->stream));
    HSS_CUDA(lane, cudaMemcpyAsync(lane->h_ctrl, lane->d_ctrl, 8 * sizeof(unsigned int), cudaMemcpyDeviceToHost,
                                   lane->stream));
    return HSS_OK;
}

// Waits for a lane's wave and collects its hits and device time; a wave whose
// exact-work or big-pair queue overflowed runs again (grown queue) before it
// counts.
int finish_wave(hss_t* h, hss_t* lane, const Wave& w, std::vector<DevHit>* hits, double* ms) {
    for (uint32_t attempt = 0;; ++attempt) {
        HSS_CUDA(lane, cudaStreamSynchronize(lane->stream));
        const unsigned int* ctrl = lane->h_ctrl;
        if ((ctrl[3] & 12u) && !(ctrl[3] & 3u)) {
            lane->exact_overflow = (ctrl[3] & 4u) != 0;
            lane->big_overflow = (ctrl[3] & 8u) != 0;
            if (grow_overflowed(lane) != HSS_OK)
                return fail(lane, HSS_ERR_OVERFLOW, "exact work or big-pair queue over capacity");
            if (int s = launch_wave(h, lane, w)) return s;
            continue;
        }
        if (ctrl[3] & 1u) return fail(lane, HSS_ERR_OVERFLOW, "shared-prime queue over capacity");
        if (ctrl[3] & 2u) return fail(lane, HSS_ERR_OVERFLOW, "shared-prime pair exceeds the list capacity");
        if (ctrl[3]) return fail(lane, HSS_ERR_OVERFLOW, "a device index check failed");
        const uint32_t nh = std::min(ctrl[0], lane->hit_cap);
        hits->resize(nh);
        if (nh) HSS_CUDA(lane, cudaMemcpy(hits->data(), lane->d_hits, nh * sizeof(DevHit), cudaMemcpyDeviceToHost));
        float f = 0;
        HSS_CUDA(lane, cudaEventElapsedTime(&f, lane->ev0, lane->ev1));
        *ms = f;
        return HSS_OK;
    }
}

// Sums a completed request's row records from the device state arena into
// its counters; every row must be marked done.
int read_request_state(hss_t* h, Request* r) {
    const size_t rows = (size_t)(r->last - r->first + 1);
    std::vector<RowCounts> state(rows);
    HSS_CUDA(h, cudaMemcpy(state.data(), h->d_state + r->slot, rows * sizeof(RowCounts), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < rows; ++i) {
        if (state[i].pad != 1) return fail(h, HSS_ERR_STATE, "a request row was not recorded on the device");
        add_row(&r->counts, state[i]);
        r->counts.pairs += h->limit - (r->first + i) + 1;
    }
    r->counts.d2h_bytes += rows * sizeof(RowCounts);
    return HSS_OK;
}

// Attributes a finished wave to its requests (under serve_mu) and completes
// those whose rows are all done: counters from the device state, slot range
// released.
void settle_wave(hss_t* h, Wave& w, int status, const std::vector<DevHit>& hits, double ms,
                 std::vector<Request*>& active) {
    std::lock_guard<std::mutex> lock(h->serve_mu);
    for (size_t i = 0; i < w.rows.size(); ++i) {
        Request* r = w.owner[i];
        --r->inflight;
        if (status) {
            r->status = status;
            r->next_row = r->last + 1;  // schedule nothing more
            continue;
        }
        r->ms_weighted += ms * (double)(h->limit - w.rows[i].l + 1);
        ++r->rows_done;
    }
    for (const DevHit& hit : hits)
        if (hit.row < w.owner.size()) w.owner[hit.row]->hits.push_back(hit);
    const uint64_t t = now_ns();
    for (size_t i = 0; i < active.size();) {
        Request* r = active[i];
        const uint64_t rows = r->last - r->first + 1;
        const bool failed = r->status != HSS_ERR_BUSY;
        // a request leaves when all its rows are done, or when it failed and
        // no wave in flight still writes its state records
        if (failed ? r->inflight > 0 : r->rows_done < rows) {
            ++i;
            continue;
        }
        if (!failed) {
            const int s = read_request_state(h, r);
            r->status = s ? s : HSS_OK;
            r->counts.kernel_ms = r->ms_weighted / (double)std::max<uint64_t>(r->counts.pairs, 1);
            r->counts.hits = r->hits.size();
        }
        r->finished_ns = t;
        h->arena.release(r->slot, (uint32_t)rows);
        active[i] = active.back();
        active.pop_back();
    }
    w.rows.clear();
    w.owner.clear();
    w.live = false;
    h->serve_cv.notify_all();
}

void serve_loop(hss_t* h) {
    cudaSetDevice(h->device);
    std::vector<Request*> active;
    Wave waves[2];
    int next_lane = 0;
    for (;;) {
        Wave w;
        {
            std::unique_lock<std::mutex> lock(h->serve_mu);
            auto schedulable = [&] {
                for (Request* r : active)
                    if (r->next_row <= r->last) return true;
                return false;
            };
            h->serve_cv.wait(lock, [&] {
                return h->serve_stop || !h->pending.empty() || schedulable() || waves[0].live || waves[1].live;
            });
            if (h->serve_stop) break;
            // admission: a request slot and room for its rows in the device state arena
            while (!h->pending.empty() && active.size() < h->max_active) {
                Request* r = h->requests[h->pending.front()];
                uint32_t slot = 0;
                if (!h->arena.alloc((uint32_t)(r->last - r->first + 1), &slot)) break;
                h->pending.pop_front();
                r->slot = slot;
                r->admitted = true;
                r->admitted_ns = now_ns();
                r->next_row = r->first;
                active.push_back(r);
            }
            // The wave: the oldest admitted request with rows left takes the
            // pair budget, every younger one a single row.  Large requests
            // then finish in arrival order, as one at a time would, while
            // every newcomer advances in every wave, so short requests end
            // within a few waves instead of waiting behind the large ones.
            std::vector<Request*> order;
            for (Request* r : active)
                if (r->next_row <= r->last) order.push_back(r);
            std::sort(order.begin(), order.end(), [](const Request* x, const Request* y) { return x->id < y->id; });
            const uint64_t budget = (uint64_t)h->wave_items << 20;
            for (size_t i = 0; i < order.size(); ++i) {
                Request* r = order[i];
                const uint64_t share = i == 0 ? budget : 0;
                uint64_t taken = 0;
                while (r->next_row <= r->last && (taken == 0 || taken + (h->limit - r->next_row + 1) <= share)) {
                    taken += h->limit - r->next_row + 1;
                    w.rows.push_back(RowRef{r->next_row, (uint32_t)w.rows.size()});
                    w.owner.push_back(r);
                    ++r->next_row;
                    ++r->inflight;
                }
            }
        }
        const bool launched = !w.rows.empty();
        if (launched) {
            hss_t* lane = h->lanes[next_lane];
            waves[next_lane] = std::move(w);
            waves[next_lane].live = true;
            const int s = launch_wave(h, lane, waves[next_lane]);
            if (s) {
                cudaStreamSynchronize(lane->stream);
                settle_wave(h, waves[next_lane], s, {}, 0, active);
            }
            next_lane ^= 1;
        }
        // Lanes alternate, so waves[next_lane] is the older wave.  After a
        // launch it is harvested (the new wave keeps the device busy
        // meanwhile); with nothing new to launch, the oldest live wave is.
        int i = next_lane;
        if (!waves[i].live && !launched) i ^= 1;
        if (waves[i].live) {
            std::vector<DevHit> hits;
            double ms = 0;
            const int s = finish_wave(h, h->lanes[i], waves[i], &hits, &ms);
            settle_wave(h, waves[i], s, hits, ms, active);
        }
    }
    for (hss_t* lane : h->lanes)
        if (lane) cudaStreamSynchronize(lane->stream);
}

int request_info(hss_t* h, Request* r, hss_request_info* info, hss_hit* hits, uint32_t cap) {
    if (info) {
        info->first = r->first;
        info->last = r->last;
        info->submitted_ns = r->submitted_ns;
        info->admitted_ns = r->admitted_ns;
        info->finished_ns = r->finished_ns;
        info->counts = r->counts;
        info->nhits = (uint32_t)r->hits.size();
        info->status = r->status;
    }
    if (hits && r->status == HSS_OK) copy_hits(r->hits, hits, cap);
    (void)h;
    return r->status == HSS_ERR_BUSY ? HSS_ERR_BUSY : HSS_OK;
}

}  // namespace

extern "C" {

int hss_serve_start(hss_t* h, uint32_t max_active, uint32_t wave_mpairs) {
    if (!h) return HSS_ERR_ARGUMENT;
    std::lock_guard<std::mutex> lock(h->serve_mu);
    if (h->serving) return HSS_OK;
    HSS_CUDA(h, cudaSetDevice(h->device));
    // device state arena: opts.serve_state_kb, else 1/16 of free HBM up to 256 MiB
    size_t free_b = 0, total_b = 0;
    HSS_CUDA(h, cudaMemGetInfo(&free_b, &total_b));
    size_t bytes = h->opts.serve_state_kb ? (size_t)h->opts.serve_state_kb << 10
                                          : std::min<size_t>(free_b / 16, (size_t)256 << 20);
    const uint32_t rows = (uint32_t)std::min<size_t>(bytes / sizeof(RowCounts), UINT32_MAX);
    if (rows == 0) return fail(h, HSS_ERR_ARGUMENT, "serving state arena holds no row");
    if (int s = device_alloc(h, &h->d_state, rows)) return s;
    for (int i = 0; i < 2; ++i) {
        int s = HSS_OK;
        h->lanes[i] = make_lane(h, &s);
        if (s) {
            for (hss_t*& lane : h->lanes) {
                if (lane) hss_close(lane);
                lane = nullptr;
            }
            device_free(h, h->d_state);
            h->d_state = nullptr;
            return fail(h, s, "serving lane set-up failed");
        }
    }
    h->arena.reset(rows);
    h->max_active = max_active ? max_active : 64;
    h->wave_items = wave_mpairs ? wave_mpairs : 256;
    h->serve_stop = false;
    h->serving = true;
    h->serve_thread = std::thread(serve_loop, h);
    return HSS_OK;
}

int hss_submit(hss_t* h, uint64_t first, uint64_t last, uint64_t* request_id) {
    if (!h || !request_id) return HSS_ERR_ARGUMENT;
    if (first < 1 || first > last || last > h->limit) return fail(h, HSS_ERR_ARGUMENT, "need 1 <= first <= last <= limit");
    std::lock_guard<std::mutex> lock(h->serve_mu);
    if (!h->serving) return fail(h, HSS_ERR_ARGUMENT, "serving loop not started");
    if (last - first + 1 > h->arena.size)
        return fail(h, HSS_ERR_MEMORY, "request rows exceed the serving state arena");
    Request* r = new Request();
    r->id = h->next_id++;
    r->first = first;
    r->last = last;
    r->submitted_ns = now_ns();
    h->requests[r->id] = r;
    h->pending.push_back(r->id);
    *request_id = r->id;
    h->serve_cv.notify_all();
    return HSS_OK;
}

int hss_poll(hss_t* h, uint64_t request_id, hss_request_info* info, hss_hit* hits, uint32_t hit_cap) {
    if (!h) return HSS_ERR_ARGUMENT;
    std::lock_guard<std::mutex> lock(h->serve_mu);
    auto it = h->requests.find(request_id);
    if (it == h->requests.end()) return HSS_ERR_NOT_FOUND;
    return request_info(h, it->second, info, hits, hit_cap);
}

int hss_wait(hss_t* h, uint64_t request_id, hss_request_info* info, hss_hit* hits, uint32_t hit_cap) {
    if (!h) return HSS_ERR_ARGUMENT;
    std::unique_lock<std::mutex> lock(h->serve_mu);
    auto it = h->requests.find(request_id);
    if (it == h->requests.end()) return HSS_ERR_NOT_FOUND;
    Request* r = it->second;
    h->serve_cv.wait(lock, [&] { return r->status != HSS_ERR_BUSY || h->serve_stop; });
    return request_info(h, r, info, hits, hit_cap);
}

int hss_serve_stop(hss_t* h) {
    if (!h) return HSS_ERR_ARGUMENT;
    {
        std::lock_guard<std::mutex> lock(h->serve_mu);
        if (!h->serving) return HSS_OK;
        h->serve_stop = true;
        h->serve_cv.notify_all();
    }
    if (h->serve_thread.joinable()) h->serve_thread.join();
    std::lock_guard<std::mutex> lock(h->serve_mu);
    for (auto& kv : h->requests) delete kv.second;
    h->requests.clear();
    h->pending.clear();
    for (hss_t*& lane : h->lanes) {
        if (lane) hss_close(lane);
        lane = nullptr;
    }
    device_free(h, h->d_state);
    h->d_state = nullptr;
    h->serving = false;
    return HSS_OK;
}

}  // extern "C"
