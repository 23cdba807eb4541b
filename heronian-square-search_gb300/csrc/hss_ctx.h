// hss_ctx.h - the handle behind hss_t, shared by the host sources.
#pragma once
#include <cuda_runtime.h>

#include <array>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "hss_api_status.h"
#include "hss_kernels.h"

namespace hss {
struct Request;

// First-fit allocator of row records in the serving state arena (host-side
// bookkeeping of device memory allocated once at serve start).
struct SlotArena {
    uint32_t size = 0;
    std::map<uint32_t, uint32_t> free;  // offset -> length of free runs

    void reset(uint32_t n) {
        size = n;
        free.clear();
        if (n) free[0] = n;
    }
    bool alloc(uint32_t n, uint32_t* off) {
        for (auto it = free.begin(); it != free.end(); ++it) {
            if (it->second < n) continue;
            *off = it->first;
            const uint32_t rest = it->second - n, at = it->first + n;
            free.erase(it);
            if (rest) free[at] = rest;
            return true;
        }
        return false;
    }
    void release(uint32_t off, uint32_t n) {
        auto next = free.lower_bound(off);
        if (next != free.end() && off + n == next->first) {
            n += next->second;
            next = free.erase(next);
        }
        if (next != free.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == off) {
                prev->second += n;
                return;
            }
        }
        free[off] = n;
    }
};
}  // namespace hss

struct hss_ctx {
    int device = 0;
    uint64_t limit = 0;
    hss_opts opts{};
    int sm_count = 0;
    std::string err;

    // host mirrors used to build work items
    std::vector<uint32_t> seg_off;
    std::vector<uint32_t> spf;
    uint64_t records = 0, ref_flattened = 0, ref_cached = 0;
    double prep_seconds = 0;

    hss::DeviceCache dev{};
    std::vector<void*> allocations;

    // launch buffers
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    hss::RowCounts* d_rows = nullptr;
    size_t rows_cap = 0;
    hss::DevHit* d_hits = nullptr;
    uint32_t hit_cap = 0;
    unsigned int* d_ctrl = nullptr;  // [0] hit_count [1] merged_count [2] next_item [3] error flags [4] big_count [5] exact_count [6] big_next [7] desc_next
    uint4* d_big = nullptr;          // shared-prime pairs too big for a warp
    uint32_t big_cap = 0;
    uint4* d_desc = nullptr;         // descriptors of one chunk of shared-prime pairs
    uint32_t desc_chunk = 0;
    hss::ExactItem* d_exact = nullptr;    // exact work queue
    uint32_t exact_cap = 0;
    bool exact_overflow = false;          // the last launch group outgrew it
    bool big_overflow = false;            // ... or outgrew the big-pair queue
    uint32_t call_reruns = 0;             // reruns of the current call after growing it
    uint4* d_merged = nullptr;
    uint32_t merged_cap = 0;
    uint8_t* d_tables = nullptr;
    hss::WorkItem* d_items = nullptr;
    size_t items_cap = 0;
    hss::WorkItem* h_items = nullptr;  // pinned
    size_t h_items_cap = 0;
    hss::RowCounts* h_rows = nullptr;  // pinned
    size_t h_rows_cap = 0;
    hss::RowInfo* d_row_info = nullptr;  // constants of the call's rows
    hss::RowInfo* h_row_info = nullptr;  // pinned
    size_t row_info_cap = 0;

    std::mutex gpu_mu;  // serialises device work on the handle

    // batched launch groups captured as a graph (opts.use_graph)
    cudaGraphExec_t graph_exec = nullptr;
    uint64_t graph_launches = 0;
    uint32_t call_graphs = 0;  // graph launches of the current call

    // per-call accounting: event triples (before main kernel, after it,
    // after the shared-prime kernels) for every launch group
    std::vector<cudaEvent_t> event_pool;
    size_t events_used = 0;
    std::vector<std::array<cudaEvent_t, 3>> marks;
    uint32_t launches = 0;
    uint64_t h2d_bytes = 0, d2h_bytes = 0;

    // serving
    std::mutex serve_mu;
    std::condition_variable serve_cv;
    std::thread serve_thread;
    bool serving = false, serve_stop = false;
    uint32_t max_active = 0, wave_items = 0;
    uint64_t next_id = 1;
    std::map<uint64_t, hss::Request*> requests;
    std::deque<uint64_t> pending;
    hss_ctx* lanes[2] = {nullptr, nullptr};  // launch lanes of the serving loop
    hss::RowCounts* d_state = nullptr;        // per-request row records (device)
    hss::SlotArena arena;                     // their allocation

    // a lane's own buffers: control words read back (pinned) and the state
    // record of each wave row (device, and its pinned staging)
    unsigned int* h_ctrl = nullptr;
    uint32_t* d_slots = nullptr;
    uint32_t* h_slots = nullptr;
    size_t slots_cap = 0;
};

