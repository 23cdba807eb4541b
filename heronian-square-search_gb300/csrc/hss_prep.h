// hss_prep.h - host-side construction of the factor cache for one limit N.
#pragma once
#include <stdint.h>

#include <memory>
#include <string>
#include <vector>

#include "hss_internal.h"

struct CUstream_st;  // cudaStream_t

namespace hss {

// Per-integer factor summary used on the host (and by the item builder).
struct NumberFactors {
    uint32_t primes[8];   // distinct split primes p = 1 (mod 4), increasing
    uint8_t exps[8];
    uint8_t count;
    uint64_t fixed;       // prod over p = 2 or p = 3 (mod 4) of p^(2a)
};

struct HostCache {
    uint64_t limit = 0;
    uint64_t records = 0;                 // total hot/exact records
    std::vector<uint32_t> spf;            // [N+1]
    std::vector<uint32_t> seg_off;        // [N+2]
    std::unique_ptr<HotRec[]> hot;        // [records]
    std::unique_ptr<ExactRec[]> exact;    // [records]
    std::unique_ptr<uint32_t[]> owner;    // [records]
    std::vector<uint32_t> pp_base;        // [N+1], UINT32_MAX if p is not a split prime
    std::vector<HotRec> pp_hot;           // prime-power values (hot)
    std::vector<__int128> pp_exact;       // prime-power values (re, im interleaved)
    uint32_t max_exponent = 0;
    // Sizes the reference's own preparation reports on stderr, recomputed for
    // this cache: "flattened N Gaussian values" (gpu_search_v42.cu:606) and
    // "cached N Gaussian pair values" (gpu_search_v42.cu:567).
    uint64_t reference_flattened = 0;
    uint64_t reference_cached = 0;
    double seconds = 0;
};

// Builds the cache for limit N with up to `threads` host threads.  Returns 0
// on success or a negative hss status with a message in *err.
int build_host_cache(uint64_t limit, int threads, HostCache* out, std::string* err);

// Factor summary of x from the smallest-prime-factor table.
NumberFactors factor_number(const uint32_t* spf, uint64_t x);

// The same cache built on the current device (hss_devprep.cu): device arrays
// with the host cache's layout and values, host copies of spf and seg_off.
// `owned` lists every device allocation of the result (the caller frees them).
struct DeviceBuild {
    uint64_t limit = 0;
    uint32_t* spf = nullptr;       // [N+1]
    uint32_t* seg_off = nullptr;   // [N+2]
    HotRec* hot = nullptr;         // [records]
    ExactRec* exact = nullptr;     // [records]
    uint32_t* owner = nullptr;     // [records]
    uint32_t* pp_base = nullptr;   // [N+1]
    HotRec* pp_hot = nullptr;      // [pp_count]
    __int128* pp_exact = nullptr;  // [2 pp_count]
    uint64_t records = 0, pp_count = 0;
    uint32_t max_exponent = 0, longest = 0;  // longest: the largest segment
    uint64_t reference_flattened = 0, reference_cached = 0;
    std::vector<uint32_t> spf_host, seg_off_host;
    std::vector<void*> owned;
    double seconds = 0;
};

// Builds the cache for limit N on the current device, on `stream`, with grids
// of sm_count * 8 CTAs.  Returns 0 or a negative hss status with *err set.
int build_device_cache(uint64_t limit, int sm_count, CUstream_st* stream, DeviceBuild* out, std::string* err);

}  // namespace hss
