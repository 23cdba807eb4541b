// hss_kernels.h - launch interface of the sm_103a search kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "hss_internal.h"

namespace hss {

// Sizes of the residue tables the kernels stage in shared memory:
// tab720[z mod 720] bit0: z mod 16 in {0,1}; bit1: bit0 and z mod 9 and
// z mod 5 fourth-power residues; bit2: bit0, z mod 9 residue and 5 | z.
// tab625[z mod 625]: fourth-power residue mod 625.  tab1547[z mod 1547]:
// fourth-power residue mod 7, 13 and 17 (gpu_search_v42.cu:166-170).
constexpr uint32_t kTableBytes = 720 + 625 + 1547;
void build_residue_tables(uint8_t* out /* kTableBytes */);

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
    unsigned int* error_flags;  // bit 0: shared-prime queue full; bit 1: pair lists over capacity
    uint4* big_queue;           // shared-prime pairs too big for one warp's lists
    unsigned int* big_count;
    uint32_t big_cap;
    const uint8_t* tables;      // kTableBytes residue tables
};

struct BatchedConfig {
    int threads;        // CTA size
    int ctas;           // persistent grid size
    uint32_t alpha_cap; // largest row segment (free set + centre) among items
    uint32_t tile_cap;  // largest m-range among items
};

// Shared memory the batched kernel needs for a configuration.
size_t batched_smem_bytes(uint32_t alpha_cap, uint32_t tile_cap);

// Persistent kernel over work items (row l, m in [m0, m1)).
cudaError_t launch_batched(const DeviceCache& cache, const WorkItem* items, uint32_t n_items,
                           const BatchedConfig& cfg, const LaunchBuffers& buf, cudaStream_t stream);

// Plain kernel: rows first_l .. first_l + n_rows - 1, one block per
// (row, slice) and one thread per pair (the reference's launch shape).
cudaError_t launch_plain(const DeviceCache& cache, uint64_t first_l, uint32_t n_rows,
                         uint32_t alpha_cap, const LaunchBuffers& buf, cudaStream_t stream);

// Pairs sharing a split prime, read from buf.merged_queue[0 .. count).
cudaError_t launch_merged(const DeviceCache& cache, uint32_t count, const LaunchBuffers& buf,
                          int ctas, cudaStream_t stream);

// Integer-op throughput of the device measured by a probe kernel (ops/s).
double int32_peak_ops(int device, int sm_count, double* ms);

// Occupancy helper for the persistent grid.
int batched_max_ctas_per_sm(int threads, size_t smem);

}  // namespace hss
