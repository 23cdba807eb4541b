// hss_noalloc.cu - a search entry point that allocates no memory.
//
// hss_search grows its per-call buffers (row table, work items, counters,
// the shared-prime and exact-work queues, pinned staging) with cudaMalloc and
// cudaMallocHost when a call needs more than the last one.  Some callers
// cannot allow that at search time: processes whose device memory is owned by
// a pool or an embedding runtime fixed at start-up, or loops that cannot take
// the implicit synchronisation an allocation brings.  hss_search_noalloc runs
// the same batched launch sequence (persistent kernel, shared-prime kernels,
// exact kernel) with all per-call device scratch in one file-scope array of
// kNoAllocBytes that is part of the library image, and host staging in static
// buffers.  Every GPU that loads the library holds the array until the process
// exits.  The array bounds the work of one launch, not the call: a call whose
// rows have more shared-prime pairs than the array holds runs as several
// launch groups, and a group whose exact-work queue fills runs again in
// smaller pieces.
//
// Set-up: the array's name is a host-side stand-in, not a device address.
// The first call on a device, with that device current, looks the address up
// with cudaGetSymbolAddress and keeps it; that first call should come before
// any stream capture.  Calls share the array and keep the last call's
// contents; everything that must start at zero (counters, queue cursors) is
// cleared by each call.  Calls are serialised within the process; calls that
// overlap on the GPU race on the array.
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <mutex>

#include "hss_ctx.h"
#include "hss_kernels.h"
#include "hss_prep.h"

namespace {

using namespace hss;

// Limits of one call, and the layout of the scratch array.
constexpr uint32_t kNaRows = 64;          // root rows per call
constexpr uint32_t kNaItems = 8192;       // work items per call
constexpr uint32_t kNaMerged = 1u << 20;  // pairs sharing a split prime per call
constexpr uint32_t kNaBig = 1u << 13;     // of which too big for one warp
constexpr uint32_t kNaDesc = 1u << 14;    // shared-prime pairs set up per chunk
constexpr uint32_t kNaExact = 1u << 16;   // exact work items per call
constexpr uint32_t kNaHits = 4096;        // hits kept per call (as the reference, gpu_search_v42.cu:177-178)
constexpr uint32_t kNaCtrl = 8;

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kOffCtrl = 0;
constexpr size_t kOffRows = align256(kOffCtrl + kNaCtrl * sizeof(unsigned int));
constexpr size_t kOffRowInfo = align256(kOffRows + kNaRows * sizeof(RowCounts));
constexpr size_t kOffHits = align256(kOffRowInfo + kNaRows * sizeof(RowInfo));
constexpr size_t kOffItems = align256(kOffHits + kNaHits * sizeof(DevHit));
constexpr size_t kOffMerged = align256(kOffItems + kNaItems * sizeof(WorkItem));
constexpr size_t kOffBig = align256(kOffMerged + (size_t)kNaMerged * sizeof(uint4));
constexpr size_t kOffDesc = align256(kOffBig + (size_t)kNaBig * kBigEntryWords * sizeof(uint4));
constexpr size_t kOffExact = align256(kOffDesc + (size_t)kNaDesc * kBigEntryWords * sizeof(uint4));
constexpr size_t kNoAllocBytes = align256(kOffExact + kNaExact * sizeof(ExactItem));
static_assert(kNoAllocBytes <= (24u << 20), "scratch stays within 24 MiB");

static __device__ __align__(256) unsigned char g_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
unsigned char* g_scratch_ptr[kMaxDevices];  // device address of g_scratch, per device
std::mutex g_mu;                            // serialises calls (shared host and device scratch)

// Host staging (static, so the call allocates nothing).
RowInfo g_host_rows[kNaRows];
WorkItem g_host_items[kNaItems];
RowCounts g_host_counts[kNaRows];
DevHit g_host_hits[kNaHits];
unsigned int g_host_ctrl[kNaCtrl];

// Failures are reported by status code only (recording a message would
// allocate): HSS_ERR_LIMIT - the interval needs more than the scratch holds;
// HSS_ERR_OVERFLOW - a queue filled up; HSS_ERR_CUDA / HSS_ERR_NO_DEVICE.
int fail(hss_t* h, int status, const char* msg) {
    (void)h;
    (void)msg;
    return status;
}

// Address of the scratch array on the current device (looked up once).
int scratch_on(hss_t* h, unsigned char** out) {
    if (h->device < 0 || h->device >= kMaxDevices) return fail(h, HSS_ERR_NO_DEVICE, "device index beyond table");
    if (!g_scratch_ptr[h->device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess) return fail(h, HSS_ERR_CUDA, cudaGetErrorString(e));
        g_scratch_ptr[h->device] = static_cast<unsigned char*>(p);
    }
    *out = g_scratch_ptr[h->device];
    return HSS_OK;
}

// Pairs (l, m) with m in [m0, m1) that can share a split prime with l
// (inclusion-exclusion over the distinct split primes of l).
uint64_t shared_bound(const hss_t* h, uint64_t l, uint64_t m0, uint64_t m1) {
    NumberFactors f = factor_number(h->spf.data(), l);
    uint64_t total = 0;
    for (uint32_t mask = 1; mask < (1u << f.count); ++mask) {
        uint64_t prod = 1;
        int bits = 0;
        bool over = false;
        for (uint32_t i = 0; i < f.count; ++i)
            if (mask & (1u << i)) {
                prod *= f.primes[i];
                ++bits;
                if (prod > h->limit) over = true;
            }
        if (over) continue;
        const uint64_t cnt = (m1 - 1) / prod - (m0 - 1) / prod;
        total = (bits & 1) ? total + cnt : total - cnt;
    }
    return total;
}

#define NA_CUDA(call)                                                \
    do {                                                             \
        cudaError_t e_ = (call);                                     \
        if (e_ != cudaSuccess) return fail(h, HSS_ERR_CUDA, cudaGetErrorString(e_)); \
    } while (0)

// A piece of a call: row r of the call against m in [m0, m1).  A call is run
// as launch groups of pieces that fit the scratch: their shared-prime pairs
// within kNaMerged, their items within kNaItems.  A group whose exact-work or
// big-pair queue overflows is run again as smaller groups (a lone piece is
// halved by m-range), so the limits bound memory, not the interval.
struct Piece {
    uint32_t r, m0, m1;
};
constexpr uint32_t kNaPieces = 4096;  // pending pieces (a depth-first work stack)
constexpr uint32_t kNaMinSpan = 64;   // a piece is not halved below this many roots
Piece g_stack[kNaPieces];
RowCounts g_host_sum[kNaRows];

struct GroupResult {
    float ms;
    uint32_t launches;
    uint64_t h2d, d2h;
};

// Runs pieces g_stack[lo, hi) as one launch group, adding its row counters to
// g_host_sum and its hits to g_host_hits[*nh ...] (at most kNaHits kept,
// *found counts them all).  Returns HSS_ERR_OVERFLOW, with nothing added, when
// a queue of the scratch overflowed.
int run_group(hss_t* h, unsigned char* base, uint32_t rows, uint32_t lo, uint32_t hi, uint32_t alpha_cap,
              uint32_t* nh, uint64_t* found, GroupResult* res) {
    const uint32_t npieces = hi - lo;
    const uint32_t per_piece = kNaItems / npieces;
    uint32_t n_items = 0;
    uint64_t shared = 0;
    for (uint32_t i = lo; i < hi; ++i) {
        const Piece& pc = g_stack[i];
        const uint64_t l = g_host_rows[pc.r].l;
        shared += shared_bound(h, l, pc.m0, pc.m1);
        const uint64_t span = pc.m1 - pc.m0;
        const uint64_t parts = std::max<uint64_t>(1, std::min<uint64_t>(per_piece, (span + 31) / 32));
        const uint64_t tile = (span + parts - 1) / parts;
        for (uint64_t m = pc.m0; m < pc.m1; m += tile)
            g_host_items[n_items++] =
                WorkItem{(uint32_t)l, (uint32_t)m, (uint32_t)std::min<uint64_t>(m + tile, pc.m1), pc.r};
    }

    LaunchBuffers b;
    unsigned int* ctrl = reinterpret_cast<unsigned int*>(base + kOffCtrl);
    b.rows = reinterpret_cast<RowCounts*>(base + kOffRows);
    b.hits = reinterpret_cast<DevHit*>(base + kOffHits);
    b.hit_count = ctrl + 0;
    b.hit_cap = kNaHits;
    b.merged_queue = reinterpret_cast<uint4*>(base + kOffMerged);
    b.merged_count = ctrl + 1;
    b.merged_cap = kNaMerged;
    b.next_item = ctrl + 2;
    b.error_flags = ctrl + 3;
    b.big_queue = reinterpret_cast<uint4*>(base + kOffBig);
    b.big_count = ctrl + 4;
    b.big_next = ctrl + 6;
    b.big_cap = kNaBig;
    b.pair_desc = reinterpret_cast<uint4*>(base + kOffDesc);
    b.desc_chunk = kNaDesc;
    b.desc_next = ctrl + 7;
    b.exact_queue = reinterpret_cast<ExactItem*>(base + kOffExact);
    b.exact_count = ctrl + 5;
    b.exact_cap = kNaExact;
    b.tables = h->d_tables;
    b.row_info = reinterpret_cast<const RowInfo*>(base + kOffRowInfo);

    cudaStream_t st = h->stream;
    NA_CUDA(cudaMemsetAsync(base + kOffCtrl, 0, kNaCtrl * sizeof(unsigned int), st));
    NA_CUDA(cudaMemsetAsync(base + kOffRows, 0, rows * sizeof(RowCounts), st));
    NA_CUDA(cudaMemcpyAsync(base + kOffItems, g_host_items, n_items * sizeof(WorkItem), cudaMemcpyHostToDevice, st));
    BatchedConfig cfg;
    cfg.threads = h->opts.block_threads ? (int)h->opts.block_threads : 256;
    cfg.min_blocks =
        h->opts.ctas_per_sm ? (int)h->opts.ctas_per_sm : (cfg.threads == 128 ? 4 : cfg.threads == 512 ? 1 : 2);
    cfg.alpha_cap = alpha_cap;
    cfg.ctas = h->sm_count * batched_max_ctas_per_sm(cfg.threads, cfg.min_blocks,
                                                     batched_smem_bytes(cfg.threads, alpha_cap));
    NA_CUDA(cudaEventRecord(h->ev0, st));
    NA_CUDA(launch_batched(h->dev, reinterpret_cast<const WorkItem*>(base + kOffItems), n_items, cfg, b, st));
    uint32_t merged_launches = 0;
    NA_CUDA(launch_merged(h->dev, shared, b, h->sm_count * 4, st, &merged_launches));
    NA_CUDA(launch_exact(h->dev, b, h->sm_count * 4, st));
    NA_CUDA(cudaEventRecord(h->ev1, st));
    NA_CUDA(cudaMemcpyAsync(g_host_ctrl, ctrl, sizeof g_host_ctrl, cudaMemcpyDeviceToHost, st));
    NA_CUDA(cudaMemcpyAsync(g_host_counts, b.rows, rows * sizeof(RowCounts), cudaMemcpyDeviceToHost, st));
    NA_CUDA(cudaStreamSynchronize(st));
    if (g_host_ctrl[3] & ~15u) return fail(h, HSS_ERR_CUDA, "hss_search_noalloc: a device index check failed");
    if (g_host_ctrl[3]) return fail(h, HSS_ERR_OVERFLOW, "hss_search_noalloc: a scratch queue overflowed");
    const uint32_t group_hits = std::min(g_host_ctrl[0], kNaHits);
    const uint32_t room = kNaHits - *nh;
    const uint32_t take = std::min(group_hits, room);
    if (take) NA_CUDA(cudaMemcpy(g_host_hits + *nh, b.hits, take * sizeof(DevHit), cudaMemcpyDeviceToHost));
    *nh += take;
    *found += g_host_ctrl[0];
    NA_CUDA(cudaEventElapsedTime(&res->ms, h->ev0, h->ev1));
    for (uint32_t r = 0; r < rows; ++r) {
        RowCounts& a = g_host_sum[r];
        const RowCounts& c = g_host_counts[r];
        a.candidates += c.candidates;
        a.products += c.products;
        a.processed += c.processed;
        a.r16 += c.r16;
        a.exact += c.exact;
        a.merged += c.merged;
        a.mproducts += c.mproducts;
        a.mcandidates += c.mcandidates;
        a.mr16 += c.mr16;
    }
    res->launches = 2 + merged_launches;
    res->h2d = n_items * sizeof(WorkItem);
    res->d2h = sizeof g_host_ctrl + rows * sizeof(RowCounts) + take * sizeof(DevHit);
    return HSS_OK;
}

int run(hss_t* h, uint64_t first, uint64_t last, hss_counts* out, hss_hit* hits, uint32_t hit_cap,
        uint32_t* nhits) {
    const uint32_t rows = (uint32_t)(last - first + 1);
    if (rows > kNaRows) return fail(h, HSS_ERR_LIMIT, "hss_search_noalloc: more than 64 root rows");
    uint32_t alpha_cap = 1;
    for (uint32_t r = 0; r < rows; ++r)
        alpha_cap = std::max(alpha_cap, h->seg_off[first + r + 1] - h->seg_off[first + r]);
    NA_CUDA(cudaSetDevice(h->device));
    unsigned char* base = nullptr;
    if (int s = scratch_on(h, &base)) return s;

    // row constants of the whole call, uploaded once
    for (uint32_t r = 0; r < rows; ++r)
        fill_row_info(h->spf.data(), h->seg_off.data(), h->limit, first + r, &g_host_rows[r]);
    NA_CUDA(cudaMemcpyAsync(base + kOffRowInfo, g_host_rows, rows * sizeof(RowInfo), cudaMemcpyHostToDevice,
                            h->stream));
    memset(g_host_sum, 0, sizeof g_host_sum);

    // work stack: whole rows, last row at the bottom
    uint32_t top = 0;
    for (uint32_t r = rows; r-- > 0;)
        g_stack[top++] = Piece{r, (uint32_t)(first + r), (uint32_t)(h->limit + 1)};
    uint32_t max_group = kNaRows, nh = 0;
    uint64_t found = 0, h2d = rows * sizeof(RowInfo), d2h = 0;
    double ms = 0;
    uint32_t launches = 0;
    while (top) {
        // a piece whose shared-prime pairs alone exceed the queue is halved
        const Piece& t = g_stack[top - 1];
        if (shared_bound(h, g_host_rows[t.r].l, t.m0, t.m1) > kNaMerged) {
            if (top + 1 > kNaPieces || t.m1 - t.m0 < 2 * kNaMinSpan)
                return fail(h, HSS_ERR_OVERFLOW, "hss_search_noalloc: work stack full");
            const Piece p = t;
            const uint32_t mid = p.m0 + (p.m1 - p.m0) / 2;
            g_stack[top - 1] = Piece{p.r, mid, p.m1};
            g_stack[top++] = Piece{p.r, p.m0, mid};
            continue;
        }
        // the group: pieces from the top while their shared-prime pairs fit
        uint32_t lo = top;
        uint64_t bound = 0;
        while (lo > 0 && top - lo < max_group) {
            const Piece& q = g_stack[lo - 1];
            const uint64_t b = shared_bound(h, g_host_rows[q.r].l, q.m0, q.m1);
            if (b > kNaMerged || bound + b > kNaMerged) break;
            bound += b;
            --lo;
        }
        GroupResult res{};
        const int s = run_group(h, base, rows, lo, top, alpha_cap, &nh, &found, &res);
        if (s == HSS_ERR_OVERFLOW) {
            // run again smaller: half the pieces, or a lone piece halved
            if (top - lo > 1) {
                max_group = (top - lo) / 2;
                continue;
            }
            const Piece p = g_stack[lo];
            if (top + 1 > kNaPieces || p.m1 - p.m0 < 2 * kNaMinSpan)
                return fail(h, HSS_ERR_OVERFLOW, "hss_search_noalloc: a scratch queue overflowed");
            const uint32_t mid = p.m0 + (p.m1 - p.m0) / 2;
            g_stack[lo] = Piece{p.r, mid, p.m1};
            g_stack[top++] = Piece{p.r, p.m0, mid};
            continue;
        }
        if (s) return s;
        top = lo;
        ms += res.ms;
        launches += res.launches;
        h2d += res.h2d;
        d2h += res.d2h;
        max_group = std::min<uint32_t>(kNaRows, max_group * 2);
    }

    std::sort(g_host_hits, g_host_hits + nh, [](const DevHit& x, const DevHit& y) {
        if (x.l != y.l) return x.l < y.l;
        if (x.m != y.m) return x.m < y.m;
        return x.n < y.n;
    });
    const uint32_t unique = (uint32_t)(std::unique(g_host_hits, g_host_hits + nh,
                                                   [](const DevHit& x, const DevHit& y) {
                                                       return x.l == y.l && x.m == y.m && x.n == y.n;
                                                   }) -
                                       g_host_hits);
    memset(out, 0, sizeof *out);
    for (uint32_t r = 0; r < rows; ++r) {
        const RowCounts& c = g_host_sum[r];
        out->pairs += h->limit - (first + r) + 1;
        out->processed += c.processed;
        out->products += c.products;
        out->candidates += c.candidates;
        out->r16 += c.r16;
        out->exact += c.exact;
        out->merged += c.merged;
        out->merged_products += c.mproducts;
        out->merged_candidates += c.mcandidates;
        out->merged_r16 += c.mr16;
    }
    const uint64_t all = found > kNaHits ? found : unique;
    out->hits = all;
    out->kernel_ms = ms;
    out->launches = launches;
    out->graph_launches = 0;
    out->h2d_bytes = h2d;
    out->d2h_bytes = d2h;
    for (uint32_t i = 0; i < unique && i < hit_cap && hits; ++i) {
        hits[i].l = g_host_hits[i].l;
        hits[i].m = g_host_hits[i].m;
        hits[i].n = g_host_hits[i].n;
        hits[i].area4_lo = g_host_hits[i].area4_lo;
        hits[i].area4_hi = g_host_hits[i].area4_hi;
        hits[i].heron_ok = g_host_hits[i].heron_ok;
        hits[i].reserved = 0;
    }
    if (nhits) *nhits = (uint32_t)std::min<uint64_t>(all, UINT32_MAX);
    return HSS_OK;
}

}  // namespace

extern "C" int hss_search_noalloc(hss_t* h, uint64_t first, uint64_t last, hss_counts* out, hss_hit* hits,
                                  uint32_t hit_cap, uint32_t* nhits) {
    if (!h || !out) return HSS_ERR_ARGUMENT;
    if (first < 1 || first > last || last > h->limit) return HSS_ERR_ARGUMENT;
    std::lock_guard<std::mutex> process_lock(g_mu);
    std::lock_guard<std::mutex> handle_lock(h->gpu_mu);
    return run(h, first, last, out, hits, hit_cap, nhits);
}
