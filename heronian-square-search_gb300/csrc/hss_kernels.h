// hss_kernels.h - launch interface of the sm_103a search kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "hss_internal.h"

namespace hss {

// Residue tables the kernels stage in shared memory:
// tabA[z mod 9360] (bytes) bit0: z mod 16 in {0,1}; bit1: bit0 and z mod 9,
// 5 and 13 fourth-power residues; bit2: bit0, z mod 9 and 13 residues and
// 5 | z.  tabD (bit set from byte kModA, 32-bit words): bit z mod 45917 set
// when z is a fourth-power residue mod 17, 37 and 73.  These are necessary
// conditions for z = n^4, like the reference's mod 16, 9, 5, 625 and 7*13*17
// tables (gpu_search_v42.cu:166-170); the moduli are chosen for filtering
// power per bit (the exact test decides every hit).
constexpr uint32_t kTabDWords = (kModD + 31) / 32;
constexpr uint32_t kTableBytes = kModA + 4 * kTabDWords;
static_assert(kModA % 4 == 0, "the bit set starts on a word");
// Wide copy, after the compact one: tabA and the tabD bit set each repeated
// over two periods (indices up to 2M - 1), so the persistent kernel indexes
// them with S + d and S + M - d without reducing mod M.
constexpr uint32_t kTabD2Words = (2 * kModD + 31) / 32;
constexpr uint32_t kTable2Bytes = 2 * kModA + 4 * kTabD2Words;
constexpr uint32_t kTableTotalBytes = kTableBytes + kTable2Bytes;
static_assert(kTableBytes % 4 == 0, "the wide copy starts on a word");
void build_residue_tables(uint8_t* out /* kTableTotalBytes */);

// Constants of one root row, built on the host for every row of a launch
// (so no kernel factors l): l, l^2, l^4, N^4, residues, the odd primes of l
// as divisibility constants (m * inv <= thr exactly when p | m), and the split
// primes of l for the shared-prime path.
struct RowInfo {
    uint64_t l, l2;
    unsigned __int128 l4, n4;
    uint64_t fixed;             // prod of non-split p^(2a) of l
    uint32_t lmodA, lmodD, l2modA;  // l^4 mod kModA, kModD; l^2 mod kModA
    float l2x2f;                // 2 l^2, rounded to float
    uint32_t l3, l5, leven, nodd;          // 3 | l, 5 | l, l even, number of odd primes
    uint32_t pinv[9], pthr[9];
    uint32_t psplit;            // bit i set when odd prime i is = 1 mod 4
    uint32_t free_l, seg;       // |free(l)| and the first record of l's segment
    uint32_t nsplit;            // split primes of l (increasing) with exponents
    uint32_t sp[8], se[8];
    float l4f;                  // l^4, rounded to float
};

// Exact work queued by the search kernels for exact_kernel: kind bits 0-1
// (0: count a whole product, 1: count one orientation, 2: hit test of one
// orientation), bit 2: product alpha*conj(beta), bit 3: orientation (y, x),
// bit 4: shared-prime pair (a, b are list entries rather than cache indices).
struct ExactItem {
    uint32_t kind, a, b, l, m, row, pad0, pad1;
};

// 16-byte words of one big_queue entry.
constexpr uint32_t kBigEntryWords = 12;

// Device buffers one search call writes.
struct LaunchBuffers {
    RowCounts* rows;            // [n_rows]
    DevHit* hits;               // [hit_cap]
    unsigned int* hit_count;    // total hits found (may exceed hit_cap)
    uint32_t hit_cap;
    uint4* merged_queue;        // (l, m, row, 0) of pairs sharing a split prime
    unsigned int* merged_count; // entries appended (may exceed merged_cap)
    uint32_t merged_cap;
    unsigned int* next_item;    // work-queue cursor of the batched kernel
    unsigned int* error_flags;  // bit 0: shared-prime queue full; 1: pair lists over capacity; 2: exact queue
                                // full; 3: big-pair queue full; 8 (0x100): an event index check failed
    uint4* big_queue;           // shared-prime pairs too big for one warp's lists: kBigEntryWords
                                // words each (the pair's descriptor, written by the set-up kernel)
    unsigned int* big_count;
    unsigned int* big_next;     // cursor of the big-pair kernel over big_queue
    uint32_t big_cap;
    uint4* pair_desc;           // descriptors of one chunk of the shared-prime queue
                                // (kBigEntryWords words each), set up for the warp kernel
    uint32_t desc_chunk;        // pairs per chunk
    unsigned int* desc_next;    // cursor of the warp kernel over the chunk (blocks of 32 pairs)
    const uint8_t* tables;      // kTableTotalBytes residue tables (compact, then wide)
    const RowInfo* row_info;    // [n_rows] constants of the launch's rows
    ExactItem* exact_queue;     // rare exact work (undecided products, possible hits)
    unsigned int* exact_count;
    uint32_t exact_cap;
};

// Host-side fill of a RowInfo from the smallest-prime-factor table.
void fill_row_info(const uint32_t* spf, const uint32_t* seg_off, uint64_t limit, uint64_t l, RowInfo* out);

struct BatchedConfig {
    int threads;        // CTA size (128, 256 or 512)
    int min_blocks;     // compiled minimum CTAs per SM (register cap): 128 -> 4|6, 256 -> 2|3, 512 -> 1
    int ctas;           // persistent grid size
    uint32_t alpha_cap; // largest row segment (free set + centre) among items
};

// The batched kernel walks an item's m-range in sub-tiles of at most
// `threads` roots and kItemRecords m-side records (the compacted record list
// lives in shared memory), so one root's segment must fit kItemRecords.
constexpr uint32_t kItemRecords = 4096;
inline uint32_t tile_cap_for(int threads) { return (uint32_t)threads; }

// Shared memory the batched kernel needs for a configuration.
size_t batched_smem_bytes(int threads, uint32_t alpha_cap);

// Persistent kernel over work items (row l, m in [m0, m1)).
cudaError_t launch_batched(const DeviceCache& cache, const WorkItem* items, uint32_t n_items,
                           const BatchedConfig& cfg, const LaunchBuffers& buf, cudaStream_t stream);

// Plain kernel: rows first_l .. first_l + n_rows - 1, one block per
// (row, slice) and one thread per pair (the reference's launch shape).
cudaError_t launch_plain(const DeviceCache& cache, uint64_t first_l, uint32_t n_rows,
                         uint32_t alpha_cap, const LaunchBuffers& buf, cudaStream_t stream);

// Pairs sharing a split prime, read from buf.merged_queue (as many as the
// kernels before appended; pair_bound: an upper bound on that number, which
// sets how many chunks of buf.desc_chunk pairs are launched), then the big
// pairs they left in buf.big_queue.  *launches receives the number of
// kernels launched.
cudaError_t launch_merged(const DeviceCache& cache, uint64_t pair_bound, const LaunchBuffers& buf,
                          int ctas, cudaStream_t stream, uint32_t* launches);

// Integer-op throughput of the device measured by a probe kernel (ops/s).
double int32_peak_ops(int device, int sm_count, double* ms);

// Exact work queued by the search kernels; run after them.
cudaError_t launch_exact(const DeviceCache& cache, const LaunchBuffers& buf, int ctas, cudaStream_t stream);

// Serving: copies a wave's row counters rows[i] into the requests' device-
// resident state, state[slots[i]], marked done (RowCounts::pad = 1), so a
// request's per-row progress and counts stay on the device until it ends.
cudaError_t launch_scatter_rows(const RowCounts* rows, const uint32_t* slots, uint32_t n, RowCounts* state,
                                cudaStream_t stream);

// Occupancy helper for the persistent grid.
int batched_max_ctas_per_sm(int threads, int min_blocks, size_t smem);

}  // namespace hss
