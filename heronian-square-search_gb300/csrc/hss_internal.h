// hss_internal.h - layouts shared by the host precompute and the sm_103a kernels.
//
// The search enumerates, for every root pair (l, m), the Gaussian integers
// z = x + iy of norm (2 l^2 m^2)^2 built from the factorisation of 2 l^2 m^2,
// one per conjugate pair, and tests both orientations (D, 4A) = (x, y), (y, x)
// (reference: src/gpu_search_v42.cu:158-345, src/search_v18.cpp:329-479).
//
// Factor cache.  For every integer x <= N the cache holds a "segment": the
// free set of x (one representative of each conjugate pair of the Gaussian
// divisor products fixed(x) * prod_p pi_p^r conj(pi_p)^(4e-r) of norm x^4,
// chosen as the vectors whose first non-central exponent index r_i is below
// its centre 2e_i) followed by the central value (x^2, 0).  A pair (l, m) with
// no common split prime has the product set free(l) x raw(m) + {l^2} x
// (free(m) + {m^2}) (reference: gpu_search_v42.cu:273-290), and since
// raw(m) = free(m) + conj(free(m)) + {m^2} every (alpha, beta) pair of the two
// segments yields alpha*beta, plus alpha*conj(beta) when neither is central.
//
// Each cached value is stored twice: an exact record (two int64 coordinates,
// |coord| <= x^2 < 2^47 for x <= 10^7) used only by the rare exact path, and a
// 16-byte "hot" record read by the filter loop: both coordinates as float and
// both coordinates' residues modulo 9360 and 45917 packed in one word.
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define HSS_HD __host__ __device__
#else
#define HSS_HD
#endif

namespace hss {

// Residue moduli packed in a hot record word: bits 0-13 mod 9360 (field A,
// = 16*9*5*13: the area mod 8*3*9*5, the mod-16 counter and the first
// fourth-power filter, z mod 16, 9, 5 and 13) and bits 14-29 mod 45917
// (field D, = 17*37*73: the second fourth-power filter).  Bit 31 of the
// real-part word marks the central value.  Both fields are evaluated for every
// counted candidate in the filter loop; fourth powers fill about a quarter of
// the classes of each prime = 1 mod 4, and on the candidates of a reference
// batch the D field passes 3.4 % of those that pass A, so only they become
// events.  Each field's products stay in 32 bits (2 M^2 < 2^32).
constexpr uint32_t kModA = 9360;
constexpr uint32_t kModD = 45917;
constexpr uint32_t kShiftD = 14;
constexpr uint32_t kMaskA = 0x3FFFu, kMaskD = 0xFFFFu;
constexpr uint32_t kResMask = kMaskA | (kMaskD << kShiftD);  // both fields of a word
constexpr uint32_t kResOne = 1u | (1u << kShiftD);           // residues of 1
constexpr uint32_t kCentralBit = 0x80000000u;
static_assert(kModA <= kMaskA + 1 && kModD <= kMaskD + 1, "fields hold their moduli");
static_assert(2ull * kModA * kModA < (1ull << 32) && 2ull * kModD * kModD < (1ull << 32),
              "two products of a field fit 32 bits");

struct HotRec {
    float re, im;
    uint32_t rre, rim;  // packed residues of re (bit 31: central) and im
};
static_assert(sizeof(HotRec) == 16, "hot record is 16 bytes");

struct ExactRec {
    int64_t re, im;
};

// Residue of a signed 128-bit value modulo m (result in [0, m)).
HSS_HD inline uint32_t mod_i128(__int128 v, uint32_t m) {
    bool neg = v < 0;
    unsigned __int128 a = neg ? (unsigned __int128)(-(v + 1)) + 1 : (unsigned __int128)v;
    uint64_t hi = (uint64_t)(a >> 64), lo = (uint64_t)a;
    uint64_t s = (uint64_t)((((unsigned __int128)1) << 64) % m);
    uint32_t r = (uint32_t)(((hi % m) * s + lo % m) % m);
    return neg && r ? m - r : r;
}

HSS_HD inline uint32_t pack_residues(__int128 v) {
    return mod_i128(v, kModA) | (mod_i128(v, kModD) << kShiftD);
}

// Float nearest-ish to a signed 128-bit value: relative error below 3*2^-24
// (hi and lo halves converted separately, then added; no cancellation because
// both halves are taken from the magnitude).
HSS_HD inline float i128_to_float(__int128 v) {
    bool neg = v < 0;
    unsigned __int128 a = neg ? (unsigned __int128)(-(v + 1)) + 1 : (unsigned __int128)v;
    float f = (float)(uint64_t)(a >> 64) * 18446744073709551616.0f + (float)(uint64_t)a;
    return neg ? -f : f;
}

// One unit of batched work: root row l against roots m in [m0, m1).
struct WorkItem {
    uint32_t l, m0, m1, row;  // row = index of l within the launch's row list
};

// Per-row device counters (all cumulative within one launch).
struct RowCounts {
    unsigned long long candidates;  // reference counter (test_d entries)
    unsigned long long products;    // Gaussian products tested (P)
    unsigned long long processed;   // pairs that reach the enumeration (Q)
    unsigned long long r16;         // candidates whose z passes mod 16 (R)
    unsigned long long exact;       // products resolved on the exact path
    unsigned long long merged;      // pairs that share a split prime
    unsigned long long mproducts;   // products of those pairs (shared-prime kernels)
    unsigned long long mcandidates;
    unsigned long long mr16;
    unsigned long long pad;
};

// A hit as produced on the device: roots and the signed 4A of the
// orientation that produced it, plus the 256-bit Heron recheck verdict.
struct DevHit {
    uint64_t l, m, n;
    uint64_t area4_lo;
    int64_t area4_hi;
    uint32_t heron_ok;
    uint32_t row;  // index of the hit's root row among the launch's rows
};
static_assert(sizeof(DevHit) == 48, "hit record is 48 bytes");

// Device-resident factor cache for one limit N (all pointers are device
// pointers; host mirrors of seg_off / spf are kept by the owner).
struct DeviceCache {
    uint64_t limit;
    const uint32_t* spf;        // smallest prime factor, [N+1]
    const uint32_t* seg_off;    // segment start of x, [N+2]; seg of x = [seg_off[x], seg_off[x+1])
    const HotRec* hot;          // [records]
    const ExactRec* exact;      // [records]
    const uint32_t* owner;      // owning x of each record, [records]
    const uint32_t* pp_base;    // prime-power table base of split prime p, [N+1]
    const HotRec* pp_hot;       // prime-power values, hot form
    const __int128* pp_exact;   // prime-power values, exact (re, im) pairs
    uint32_t max_exponent;      // largest exponent covered by the prime-power table
};

// Offset of exponent e's 4e+1 values within prime p's block:
// sum_{a<e} (4a+1) = 2e^2 - e - 1.
HSS_HD inline uint32_t pp_exponent_offset(uint32_t e) { return 2 * e * e - e - 1; }

}  // namespace hss
