// hss_kernels.cu - sm_103a kernels of the square-sided Heronian triangle search.
//
// What is computed (reference semantics, src/gpu_search_v42.cu:158-345 and
// src/search_v18.cpp:329-479): for root rows l and every m in [l, N] that is
// not skipped (both even; a prime p = 3 mod 4 dividing both; no split prime in
// either), every Gaussian integer z = x + iy of norm (2 l^2 m^2)^2 built from
// the split primes of l and m (one per conjugate pair) is a "product".  Each
// product has two orientations (D, 4A) = (x, y) and (y, x); an orientation
// whose 4A is nonzero, = 0 mod 8 and = 0 mod 3 (mod 9 when 3 | lm, mod 5 when
// 5 divides neither) counts one candidate for each sign of D inside the
// window [l^4 + m^4 - N^4, l^4]; a candidate is a hit when z = l^4 + m^4 - D
// is a fourth power n^4 with m <= n <= N, gcd(l, m, n) = 1 and 5 | lmn.
//
// How it is computed here.  The reference multiplies every product out in
// 128-bit arithmetic.  These kernels decide almost every product from
//   * residues of the product's coordinates mod 720, 625 and 1547, formed from
//     per-value residues (exact, 32-bit integer multiplies), and
//   * float approximations of the coordinates with a proven error bound
//     (|z| = 2 l^2 m^2 is known per pair, so every coordinate error is below
//     eps = 2 l^2 m^2 * 2^-20),
// and send a product to the exact 128-bit path only when a window decision is
// within eps of a boundary, or when its z survives every residue filter (a
// possible hit).  Candidate counts are therefore exact, and every hit is
// confirmed exactly and rechecked in 256-bit arithmetic.
//
// Work shapes.  batched_kernel is persistent: CTAs pull (row l, m-range)
// items from a global cursor; the m-side values of the range are read once,
// coalesced, and each thread multiplies its value against the row's whole
// segment held in shared memory (a uniform loop: no per-pair divergence).
// plain_kernel keeps the reference's shape (a block per (row, slice), one
// thread per pair).  merged_kernel handles the pairs that share a split prime
// (gpu_search_v42.cu:318-341), one CTA per pair.
#include <cuda_runtime.h>
#include <math.h>

#include "hss_kernels.h"

namespace hss {
namespace {

using u128 = unsigned __int128;
using i128 = __int128;

constexpr uint32_t kSqA = kModA * kModA;
constexpr uint32_t kSqB = kModB * kModB;
constexpr uint32_t kSqC = kModC * kModC;
constexpr uint32_t kTabA = 0, kTabB = 720, kTabC = 720 + 625;
constexpr uint32_t kSlices = 8;           // plain kernel: blocks per row
constexpr uint32_t kPlainThreads = 128;   // plain kernel: threads per block
constexpr uint32_t kMergedThreads = 128;   // big shared-prime pairs: one CTA per pair
constexpr uint32_t kMergedListCap = 2048;  // alpha + beta entries of one big pair
constexpr uint32_t kWarpPairThreads = 256; // shared-prime pairs: one warp per pair
constexpr uint32_t kWarpPairWarps = kWarpPairThreads / 32;
constexpr uint32_t kWarpListCap = 192;     // alpha + beta entries of one warp's pair
constexpr uint32_t kMaxTerms = 16;

// Window and filter constants of one pair (l, m).
struct PairCtx {
    float lo1, hi1, lo1o, hi1o;  // z = S - t counted iff t in [lo1, hi1]; not iff t < lo1o or t > hi1o
    float hi2, hi2o;             // z = S + t counted iff t <= hi2; not iff t > hi2o
    float eps;                   // bound on |float - exact| of a product coordinate
    uint32_t sres;               // S = l^4 + m^4 mod 720 | mod 625 << 10 | mod 1547 << 20 | flag5 << 31
    uint32_t dinv;               // inverse of D mod 2^32 (0: pair not on this path)
    uint32_t dthr;               // floor((2^32 - 1) / (8 D))
};

// Constants of one root row.
struct RowConst {
    uint64_t l, l2;
    u128 l4, n4;
    uint32_t lmodA, lmodB, lmodC;   // l^4 mod 720, 625, 1547
    uint32_t l2modA;                // l^2 mod 720
    uint32_t l3, l5, leven;
    uint32_t nprimes;               // odd primes of l
    uint32_t pinv[9], pthr[9], psplit[9];
    uint32_t free_l;                // |free(l)|
};

struct Acc {
    uint32_t cand, r16, prod, exact, processed, merged;
};

// ------------------------------------------------------------ arithmetic

__host__ __device__ inline float u128_to_float(u128 a) {
    return (float)(uint64_t)(a >> 64) * 18446744073709551616.0f + (float)(uint64_t)a;
}

__host__ __device__ inline uint32_t mod_u128_small(u128 v, uint32_t m) {
    uint64_t s = (uint64_t)((((u128)1) << 64) % m);
    return (uint32_t)((((uint64_t)(v >> 64) % m) * s + (uint64_t)v % m) % m);
}

__device__ inline uint64_t gcd64(uint64_t a, uint64_t b) {
    while (b) {
        uint64_t r = a % b;
        a = b;
        b = r;
    }
    return a;
}

// Multiplicative inverse of an odd number mod 2^32 (Newton iteration).
__host__ __device__ inline uint32_t inverse_odd(uint32_t d) {
    uint32_t x = d;  // correct to 3 bits
    for (int i = 0; i < 4; ++i) x *= 2u - d * x;
    return x;
}

__device__ inline bool divides(uint32_t inv, uint32_t thr, uint32_t m) { return m * inv <= thr; }

// n = 0 mod 8D for n < 2^29, via one multiply and a rotate: n * D^-1 mod 2^32
// rotated right by 3 is at most floor((2^32-1)/(8D)) exactly when 8D | n.
__device__ __forceinline__ bool area_gate(uint32_t n, uint32_t dinv, uint32_t dthr) {
    uint32_t h = n * dinv;
    return __funnelshift_r(h, h, 3) <= dthr;
}

// ----------------------------------------------------------- 256-bit check

// Heron recheck (the reference's CPU does it on the host, search_v18.cpp:
// 481-501): the four Heron factors of sides l^2, m^2, n^2 are positive and
// their product equals (4A)^2, compared in 256-bit arithmetic.
__device__ void mul256(const uint64_t a[4], const uint64_t b[4], uint64_t out[4]) {
    uint64_t acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = 0; i < 4; ++i) {
        uint64_t carry = 0;
        for (int j = 0; j < 4; ++j) {
            u128 cur = (u128)a[i] * b[j] + acc[i + j] + carry;
            acc[i + j] = (uint64_t)cur;
            carry = (uint64_t)(cur >> 64);
        }
        for (int k = i + 4; carry && k < 8; ++k) {
            u128 cur = (u128)acc[k] + carry;
            acc[k] = (uint64_t)cur;
            carry = (uint64_t)(cur >> 64);
        }
    }
    for (int i = 0; i < 4; ++i) out[i] = acc[i];
}

__device__ uint32_t heron_ok(uint64_t l, uint64_t m, uint64_t n, i128 area4) {
    u128 x = (u128)l * l, y = (u128)m * m, z = (u128)n * n;
    i128 f[4] = {(i128)(x + y + z), -(i128)x + (i128)y + (i128)z, (i128)x - (i128)y + (i128)z,
                 (i128)x + (i128)y - (i128)z};
    if (f[0] <= 0 || f[1] <= 0 || f[2] <= 0 || f[3] <= 0 || area4 % 4 != 0) return 0;
    uint64_t h[4] = {(uint64_t)f[0], (uint64_t)((u128)f[0] >> 64), 0, 0};
    for (int i = 1; i < 4; ++i) {
        uint64_t t[4] = {(uint64_t)f[i], (uint64_t)((u128)f[i] >> 64), 0, 0};
        mul256(h, t, h);
    }
    u128 a = (u128)(area4 < 0 ? -area4 : area4);
    uint64_t e[4] = {(uint64_t)a, (uint64_t)(a >> 64), 0, 0};
    uint64_t sq[4];
    mul256(e, e, sq);
    for (int i = 0; i < 4; ++i)
        if (sq[i] != h[i]) return 0;
    return 1;
}

// ------------------------------------------------------------- exact path

struct ExactPair {
    uint64_t l, m, n;
    uint32_t row;
    u128 l4, m4, n4;
    i128 lower, upper;
    uint32_t flags;
};

__device__ ExactPair exact_pair(uint64_t l, uint64_t m, uint64_t n, uint32_t row) {
    ExactPair p;
    p.row = row;
    p.l = l;
    p.m = m;
    p.n = n;
    p.l4 = (u128)(l * l) * (l * l);
    p.m4 = (u128)(m * m) * (m * m);
    p.n4 = (u128)(n * n) * (n * n);
    p.lower = (i128)p.l4 + (i128)p.m4 - (i128)p.n4;
    p.upper = (i128)p.l4;
    p.flags = ((l % 3 == 0 || m % 3 == 0) ? 1u : 0u) | ((l % 5 != 0 && m % 5 != 0) ? 2u : 0u);
    return p;
}

// The candidate test of one signed D (gpu_search_v42.cu:158-179): counted on
// entry; then z = l^4 + m^4 - D is tested exactly.
__device__ void exact_test_d(const ExactPair& p, i128 d, i128 area4, uint32_t& cand, uint32_t& r16,
                             const uint8_t* tab, const LaunchBuffers& buf) {
    ++cand;
    i128 sz = (i128)p.l4 + (i128)p.m4 - d;
    if (sz < 0 || (u128)sz < p.m4 || (u128)sz > p.n4) return;
    u128 z = (u128)sz;
    uint32_t low = (uint32_t)z & 15u;
    if (low > 1) return;
    ++r16;
    // necessary conditions for z = n^4 (with 5 | n when 5 divides neither l
    // nor m): z mod 720 (16, 9, 5), mod 625 and mod 7*13*17, from the tables
    uint32_t rA = mod_u128_small(z, kModA), rB = mod_u128_small(z, kModB);
    if (!(tab[kTabA + rA] & ((p.flags & 2u) ? 4u : 2u))) return;
    if ((p.flags & 2u) ? rB != 0 : !tab[kTabB + rB]) return;
    if (!tab[kTabC + mod_u128_small(z, kModC)]) return;
    double zd = (double)(uint64_t)(z >> 64) * 18446744073709551616.0 + (double)(uint64_t)z;
    uint64_t root = (uint64_t)sqrt(sqrt(zd));
    while (root > 0 && (u128)root * root * root * root > z) --root;
    while ((u128)(root + 1) * (root + 1) * (root + 1) * (root + 1) <= z) ++root;
    if ((u128)root * root * root * root != z) return;
    if (gcd64(gcd64(p.l, p.m), root) != 1) return;
    if ((p.l % 5 && p.m % 5 && root % 5) || root < p.m || root > p.n) return;
    unsigned int idx = atomicAdd(buf.hit_count, 1u);
    if (idx < buf.hit_cap) {
        DevHit h;
        h.l = p.l;
        h.m = p.m;
        h.n = root;
        h.area4_lo = (uint64_t)area4;
        h.area4_hi = (int64_t)(area4 >> 64);
        h.heron_ok = heron_ok(p.l, p.m, root, area4);
        h.row = p.row;
        buf.hits[idx] = h;
    }
}

// One orientation (gpu_search_v42.cu:181-194).
__device__ void exact_test_pair(const ExactPair& p, i128 d, i128 area4, uint32_t& cand, uint32_t& r16,
                                const uint8_t* tab, const LaunchBuffers& buf) {
    if (area4 == 0 || ((uint64_t)area4 & 7) != 0) return;
    bool pos = d >= p.lower && d <= p.upper;
    bool neg = -d >= p.lower && -d <= p.upper;
    if (!pos && !neg) return;
    u128 a = (u128)(area4 < 0 ? -area4 : area4);
    if (mod_u128_small(a, 3) != 0) return;
    if ((p.flags & 1u) && mod_u128_small(a, 9) != 0) return;
    if ((p.flags & 2u) && mod_u128_small(a, 5) != 0) return;
    if (pos) exact_test_d(p, d, area4, cand, r16, tab, buf);
    if (neg && d != 0) exact_test_d(p, -d, area4, cand, r16, tab, buf);
}

// Both orientations of the product x + iy (gpu_search_v42.cu:196-200).
__device__ void exact_product(const ExactPair& p, i128 x, i128 y, uint32_t& cand, uint32_t& r16,
                              const uint8_t* tab, const LaunchBuffers& buf) {
    exact_test_pair(p, x, y, cand, r16, tab, buf);
    if (x != y && x != -y) exact_test_pair(p, y, x, cand, r16, tab, buf);
}

// Resolves the products flagged by eval_pair: status bit k (k = 0: a*b,
// k = 1: a*conj(b)) means "undecided: count exactly", bit 2+k means "possible
// hit: test exactly, counts already taken".
__device__ __noinline__ void resolve_exact(uint32_t st, i128 ar, i128 ai, i128 br, i128 bi, uint64_t l, uint64_t m,
                              uint64_t n, uint32_t row, const uint8_t* tab, Acc& acc, const LaunchBuffers& buf) {
    ExactPair p = exact_pair(l, m, n, row);
    for (int k = 0; k < 2; ++k) {
        if (!(st & ((1u | 4u) << k))) continue;
        i128 bim = k ? -bi : bi;
        i128 x = ar * br - ai * bim, y = ar * bim + ai * br;
        uint32_t c = 0, r = 0;
        exact_product(p, x, y, c, r, tab, buf);
        if (st & (1u << k)) {
            acc.cand += c;
            acc.r16 += r;
            acc.exact += 1;
        }
    }
}

// --------------------------------------------------------------- fast path

// Deeper residue filters mod 625 and 1547 for a counted orientation whose z
// passed the mod-720 table; true when some counted sign survives.
__device__ __forceinline__ bool deep_filters(uint32_t arw, uint32_t aiw, uint32_t brw, uint32_t biw,
                                             int k, int o, bool neg, bool c1, bool c2, uint32_t sres,
                                             bool flag5, const uint8_t* tab) {
    uint32_t ar = (arw >> 10) & 1023u, ai = (aiw >> 10) & 1023u, br = (brw >> 10) & 1023u,
             bi = (biw >> 10) & 1023u;
    uint32_t q1 = ar * br, q2 = ai * bi, q3 = ar * bi, q4 = ai * br;
    uint32_t x = k ? q1 + q2 : q1 + kSqB - q2;
    uint32_t y = k ? q4 + kSqB - q3 : q3 + q4;
    uint32_t dB = (o ? y : x) % kModB;
    uint32_t tB = neg ? (dB ? kModB - dB : 0u) : dB;
    uint32_t sB = (sres >> 10) & 1023u;
    uint32_t zB1 = sB >= tB ? sB - tB : sB + kModB - tB;
    uint32_t zB2 = sB + tB >= kModB ? sB + tB - kModB : sB + tB;
    bool okB1 = flag5 ? zB1 == 0 : tab[kTabB + zB1] != 0;
    bool okB2 = flag5 ? zB2 == 0 : tab[kTabB + zB2] != 0;
    c1 = c1 && okB1;
    c2 = c2 && okB2;
    if (!(c1 || c2)) return false;
    ar = (arw >> 20) & 2047u;
    ai = (aiw >> 20) & 2047u;
    br = (brw >> 20) & 2047u;
    bi = (biw >> 20) & 2047u;
    q1 = ar * br;
    q2 = ai * bi;
    q3 = ar * bi;
    q4 = ai * br;
    x = k ? q1 + q2 : q1 + kSqC - q2;
    y = k ? q4 + kSqC - q3 : q3 + q4;
    uint32_t dC = (o ? y : x) % kModC;
    uint32_t tC = neg ? (dC ? kModC - dC : 0u) : dC;
    uint32_t sC = (sres >> 20) & 2047u;
    uint32_t zC1 = sC >= tC ? sC - tC : sC + kModC - tC;
    uint32_t zC2 = sC + tC >= kModC ? sC + tC - kModC : sC + tC;
    return (c1 && tab[kTabC + zC1]) || (c2 && tab[kTabC + zC2]);
}

// One product x + iy (float xf, yf; mod-720 residues xa, ya as unreduced
// sums).  Adds its candidates to acc when every decision is certain and
// returns 0, 1 (undecided) or 4 (possible hit), shifted by k by the caller.
__device__ __forceinline__ uint32_t eval_product(float xf, float yf, uint32_t xa, uint32_t ya, int k,
                                                 uint32_t arw, uint32_t aiw, uint32_t brw,
                                                 uint32_t biw, const PairCtx& c, const uint8_t* tab,
                                                 Acc& acc) {
    uint32_t cnt = 0, r = 0, status = 0;
    const bool flag5 = (c.sres >> 31) != 0;
    const uint32_t sA = c.sres & 1023u;
#pragma unroll
    for (int o = 0; o < 2; ++o) {
        uint32_t ares = o ? xa : ya;
        if (!area_gate(ares, c.dinv, c.dthr)) continue;
        float df = o ? yf : xf;
        float t = fabsf(df);
        bool in1 = (t >= c.lo1) & (t <= c.hi1);
        bool in2 = t <= c.hi2;
        bool und = (!in1 & (t >= c.lo1o) & (t <= c.hi1o)) | (!in2 & (t <= c.hi2o)) | (t < c.eps);
        if (und) {
            status |= 1u;
            continue;
        }
        if (!(in1 | in2)) continue;
        cnt += (uint32_t)in1 + (uint32_t)in2;
        bool neg = df < 0.f;
        uint32_t dA = (o ? ya : xa) % kModA;
        uint32_t tA = neg ? (dA ? kModA - dA : 0u) : dA;
        uint32_t z1 = sA >= tA ? sA - tA : sA + kModA - tA;
        uint32_t z2 = sA + tA >= kModA ? sA + tA - kModA : sA + tA;
        uint32_t m1 = in1 ? tab[kTabA + z1] : 0u;
        uint32_t m2 = in2 ? tab[kTabA + z2] : 0u;
        r += (m1 & 1u) + (m2 & 1u);
        uint32_t sel = flag5 ? 4u : 2u;
        if ((m1 | m2) & sel) {
            if (deep_filters(arw, aiw, brw, biw, k, o, neg, (m1 & sel) != 0, (m2 & sel) != 0, c.sres,
                             flag5, tab))
                status |= 4u;
        }
    }
    if (status & 1u) return 1u;
    acc.cand += cnt;
    acc.r16 += r;
    return status;
}

// One (alpha, beta) value pair: products alpha*beta and, when neither value
// is central, alpha*conj(beta).  Returns the exact-path status bits.
__device__ __forceinline__ uint32_t eval_pair(const HotRec& a, const HotRec& b, bool two,
                                              const PairCtx& c, const uint8_t* tab, Acc& acc) {
    uint32_t ar = a.rre & 1023u, ai = a.rim & 1023u, br = b.rre & 1023u, bi = b.rim & 1023u;
    uint32_t p1 = ar * br, p2 = ai * bi, p3 = ar * bi, p4 = ai * br;
    float f1 = a.re * b.re, f2 = a.im * b.im, f3 = a.re * b.im, f4 = a.im * b.re;
    uint32_t st = eval_product(f1 - f2, f3 + f4, p1 + kSqA - p2, p3 + p4, 0, a.rre, a.rim, b.rre, b.rim,
                               c, tab, acc);
    if (two) {
        uint32_t s2 = eval_product(f1 + f2, f4 - f3, p1 + p2, p4 + kSqA - p3, 1, a.rre, a.rim, b.rre,
                                   b.rim, c, tab, acc);
        st |= s2 << 1;
    }
    return st;
}

// ------------------------------------------------------------ pair set-up

__device__ __noinline__ void row_setup(const DeviceCache& cache, uint64_t l, RowConst& R) {
    uint64_t n = cache.limit;
    R.l = l;
    R.l2 = l * l;
    R.l4 = (u128)R.l2 * R.l2;
    R.n4 = (u128)(n * n) * (n * n);
    R.lmodA = mod_u128_small(R.l4, kModA);
    R.lmodB = mod_u128_small(R.l4, kModB);
    R.lmodC = mod_u128_small(R.l4, kModC);
    R.l2modA = (uint32_t)(R.l2 % kModA);
    R.l3 = l % 3 == 0;
    R.l5 = l % 5 == 0;
    R.leven = (l & 1) == 0;
    R.free_l = cache.seg_off[l + 1] - cache.seg_off[l] - 1;
    uint32_t np = 0;
    uint64_t x = l;
    while (x > 1) {
        uint32_t p = cache.spf[x];
        do x /= p;
        while (x % p == 0);
        if (p == 2) continue;
        R.pinv[np] = inverse_odd(p);
        R.pthr[np] = 0xFFFFFFFFu / p;
        R.psplit[np] = (p & 3u) == 1u;
        ++np;
    }
    R.nprimes = np;
}

enum PairKind : uint32_t { kSkip = 0, kCached = 1, kMerged = 2 };

// Skip rules of gpu_search_v42.cu:305-316 (and search_v18.cpp:336-339, 362):
// both even; an inert prime of l dividing m; neither has a split prime.
// A split prime of l dividing m sends the pair to the shared-prime path.
__device__ __forceinline__ uint32_t classify(const RowConst& R, const DeviceCache& cache, uint32_t m,
                                             uint32_t free_m) {
    if (R.leven && (m & 1u) == 0) return kSkip;
    bool shared_split = false;
    for (uint32_t i = 0; i < R.nprimes; ++i) {
        if (divides(R.pinv[i], R.pthr[i], m)) {
            if (!R.psplit[i]) return kSkip;
            shared_split = true;
        }
    }
    if (R.free_l == 0 && free_m == 0) return kSkip;
    return shared_split ? kMerged : kCached;
}

__device__ __forceinline__ uint32_t pow4_mod(uint32_t x, uint32_t m) {
    uint32_t s = x * x % m;
    return s * s % m;
}

// Window and filter constants for pair (l, m); also the analytic count of
// the all-central product (2 l^2 m^2, 0), whose only orientation with a
// nonzero area is D = 0, 4A = 2 l^2 m^2 (counted when the window contains 0;
// z = l^4 + m^4 is never a fourth power).
__device__ __noinline__ PairCtx make_ctx(const RowConst& R, uint64_t m, uint32_t& cc_cand, uint32_t& cc_r16) {
    uint64_t m2 = m * m;
    u128 m4 = (u128)m2 * m2;
    i128 w = (i128)R.l4 + (i128)m4 - (i128)R.n4;
    u128 twoL = (u128)(2 * R.l2) * m2;
    float E = u128_to_float(twoL) * 0x1p-20f;
    float T2 = u128_to_float(R.l4);
    float e2 = E + T2 * 0x1p-22f;
    float wf = i128_to_float(w);
    float ew = E + fabsf(wf) * 0x1p-21f;
    PairCtx c;
    c.hi1 = T2 - e2;
    c.hi1o = T2 + e2;
    if (w >= 0) {
        c.lo1 = wf + ew;
        c.lo1o = wf - ew;
        c.hi2 = -INFINITY;
        c.hi2o = -INFINITY;
    } else {
        c.lo1 = -1.f;   // non-central products have |D| >= 1 > 0 = max(w, 0)
        c.lo1o = -2.f;
        c.hi2 = -wf - ew;
        c.hi2o = -wf + ew;
    }
    c.eps = E;
    bool f3 = R.l3 || m % 3 == 0;
    bool f5 = !R.l5 && m % 5 != 0;
    uint32_t D = 3u * (f3 ? 3u : 1u) * (f5 ? 5u : 1u);
    c.dinv = inverse_odd(D);
    c.dthr = 0xFFFFFFFFu / (8u * D);
    uint32_t mA = (uint32_t)(m % kModA), mB = (uint32_t)(m % kModB), mC = (uint32_t)(m % kModC);
    uint32_t sA = (R.lmodA + pow4_mod(mA, kModA)) % kModA;
    uint32_t sB = (R.lmodB + pow4_mod(mB, kModB)) % kModB;
    uint32_t sC = (R.lmodC + pow4_mod(mC, kModC)) % kModC;
    c.sres = sA | (sB << 10) | (sC << 20) | (f5 ? 0x80000000u : 0u);
    // all-central product: 4A = 2 l^2 m^2 must be = 0 mod 8D and w <= 0
    uint32_t areaA = 2u * (R.l2modA * (uint32_t)(m2 % kModA) % kModA);
    bool cc = area_gate(areaA, c.dinv, c.dthr) && w <= 0;
    cc_cand = cc ? 1u : 0u;
    cc_r16 = (cc && (sA & 15u) <= 1u) ? 1u : 0u;
    return c;
}

__device__ __forceinline__ HotRec scale2(HotRec h) {
    HotRec s;
    s.re = 2.f * h.re;
    s.im = 2.f * h.im;
    uint32_t ra = h.rre & 1023u, rb = (h.rre >> 10) & 1023u, rc = (h.rre >> 20) & 2047u;
    ra = 2 * ra >= kModA ? 2 * ra - kModA : 2 * ra;
    rb = 2 * rb >= kModB ? 2 * rb - kModB : 2 * rb;
    rc = 2 * rc >= kModC ? 2 * rc - kModC : 2 * rc;
    s.rre = ra | (rb << 10) | (rc << 20) | (h.rre & kCentralBit);
    ra = h.rim & 1023u;
    rb = (h.rim >> 10) & 1023u;
    rc = (h.rim >> 20) & 2047u;
    ra = 2 * ra >= kModA ? 2 * ra - kModA : 2 * ra;
    rb = 2 * rb >= kModB ? 2 * rb - kModB : 2 * rb;
    rc = 2 * rc >= kModC ? 2 * rc - kModC : 2 * rc;
    s.rim = ra | (rb << 10) | (rc << 20);
    return s;
}

__device__ __forceinline__ void push_merged(const LaunchBuffers& buf, uint32_t l, uint32_t m, uint32_t row) {
    unsigned int idx = atomicAdd(buf.merged_count, 1u);
    if (idx < buf.merged_cap)
        buf.merged_queue[idx] = make_uint4(l, m, row, 0u);
    else
        atomicOr(buf.error_flags, 1u);
}

// Warp-level reduction of the per-thread counters into a row's counters;
// `shared_prime` also books them as work of the shared-prime kernels.
__device__ __forceinline__ void flush_acc(Acc& acc, RowCounts* rc, bool shared_prime = false) {
    uint32_t v[6] = {acc.cand, acc.r16, acc.prod, acc.exact, acc.processed, acc.merged};
#pragma unroll
    for (int i = 0; i < 6; ++i) v[i] = __reduce_add_sync(0xFFFFFFFFu, v[i]);
    if ((threadIdx.x & 31) == 0) {
        if (v[0]) atomicAdd(&rc->candidates, (unsigned long long)v[0]);
        if (v[1]) atomicAdd(&rc->r16, (unsigned long long)v[1]);
        if (v[2]) atomicAdd(&rc->products, (unsigned long long)v[2]);
        if (v[3]) atomicAdd(&rc->exact, (unsigned long long)v[3]);
        if (v[4]) atomicAdd(&rc->processed, (unsigned long long)v[4]);
        if (v[5]) atomicAdd(&rc->merged, (unsigned long long)v[5]);
        if (shared_prime) {
            if (v[0]) atomicAdd(&rc->mcandidates, (unsigned long long)v[0]);
            if (v[1]) atomicAdd(&rc->mr16, (unsigned long long)v[1]);
            if (v[2]) atomicAdd(&rc->mproducts, (unsigned long long)v[2]);
        }
    }
    acc = Acc{0, 0, 0, 0, 0, 0};
}

// Products of one m-side record against the row's segment in shared memory.
__device__ __forceinline__ void record_loop(const HotRec* s_alpha, uint32_t na, const HotRec& b,
                                            const PairCtx& c, const uint8_t* tab, const DeviceCache& cache,
                                            uint32_t a0, uint32_t j, uint64_t l, uint64_t m, uint32_t row,
                                            Acc& acc, const LaunchBuffers& buf) {
    const bool cb = (b.rre & kCentralBit) != 0;
    for (uint32_t k = 0; k < na; ++k) {
        HotRec a = s_alpha[k];
        const bool ca = (a.rre & kCentralBit) != 0;
        if (ca & cb) continue;
        const bool two = !(ca | cb);
        acc.prod += two ? 2u : 1u;
        uint32_t st = eval_pair(a, b, two, c, tab, acc);
        if (st) {
            ExactRec ea = cache.exact[a0 + k], eb = cache.exact[j];
            resolve_exact(st, 2 * (i128)ea.re, 2 * (i128)ea.im, (i128)eb.re, (i128)eb.im, l, m, cache.limit,
                          row, tab, acc, buf);
        }
    }
}

// ------------------------------------------------------------ batched kernel

template <int NT>
__global__ void __launch_bounds__(NT, 512 / NT) batched_kernel(const DeviceCache cache, const WorkItem* __restrict__ items,
                                                     uint32_t n_items, uint32_t alpha_cap, uint32_t tile_cap,
                                                     const LaunchBuffers buf) {
    extern __shared__ __align__(16) unsigned char smem[];
    HotRec* s_alpha = reinterpret_cast<HotRec*>(smem);
    PairCtx* s_ctx = reinterpret_cast<PairCtx*>(s_alpha + alpha_cap);
    uint8_t* s_tab = reinterpret_cast<uint8_t*>(s_ctx + tile_cap);
    __shared__ RowConst s_row;
    __shared__ uint32_t s_item;

    for (uint32_t i = threadIdx.x; i < kTableBytes; i += NT) s_tab[i] = buf.tables[i];
    Acc acc{0, 0, 0, 0, 0, 0};
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(buf.next_item, 1u);
        __syncthreads();
        const uint32_t it = s_item;
        if (it >= n_items) break;
        const WorkItem w = items[it];
        if (threadIdx.x == 0) row_setup(cache, w.l, s_row);
        __syncthreads();
        const uint32_t a0 = cache.seg_off[w.l];
        const uint32_t na = cache.seg_off[w.l + 1] - a0;
        for (uint32_t i = threadIdx.x; i < na; i += NT) s_alpha[i] = scale2(cache.hot[a0 + i]);
        const uint32_t nm = w.m1 - w.m0;
        for (uint32_t i = threadIdx.x; i < nm; i += NT) {
            const uint32_t m = w.m0 + i;
            const uint32_t free_m = cache.seg_off[m + 1] - cache.seg_off[m] - 1;
            const uint32_t kind = classify(s_row, cache, m, free_m);
            PairCtx c;
            c.dinv = 0;
            if (kind == kCached) {
                uint32_t cc_c, cc_r;
                c = make_ctx(s_row, m, cc_c, cc_r);
                acc.processed += 1;
                acc.prod += 1;
                acc.cand += cc_c;
                acc.r16 += cc_r;
            } else if (kind == kMerged) {
                acc.processed += 1;
                acc.merged += 1;
                push_merged(buf, w.l, m, w.row);
            }
            s_ctx[i] = c;
        }
        __syncthreads();
        // Rounds of NT records: every lane runs the same alpha iteration at the
        // same time (lanes without a record on this path are predicated off),
        // so lanes never drift into different phases of the alpha loop.
        const uint32_t r0 = cache.seg_off[w.m0], r1 = cache.seg_off[w.m1];
        for (uint32_t base = r0; base < r1; base += NT) {
            const uint32_t j = base + threadIdx.x;
            uint32_t m = 0;
            PairCtx c;
            c.dinv = 0;
            HotRec b{0.f, 0.f, 0u, 0u};
            if (j < r1) {
                m = cache.owner[j];
                c = s_ctx[m - w.m0];
                b = cache.hot[j];
            }
            const bool live = c.dinv != 0;
            const bool cb = (b.rre & kCentralBit) != 0;
            for (uint32_t k = 0; k < na; ++k) {
                const HotRec a = s_alpha[k];
                const bool ca = (a.rre & kCentralBit) != 0;
                if (live && !(ca & cb)) {
                    const bool two = !(ca | cb);
                    acc.prod += two ? 2u : 1u;
                    uint32_t st = eval_pair(a, b, two, c, s_tab, acc);
                    if (st) {
                        ExactRec ea = cache.exact[a0 + k], eb = cache.exact[j];
                        resolve_exact(st, 2 * (__int128)ea.re, 2 * (__int128)ea.im, (__int128)eb.re,
                                      (__int128)eb.im, w.l, m, cache.limit, w.row, s_tab, acc, buf);
                    }
                }
            }
        }
        flush_acc(acc, &buf.rows[w.row]);
    }
}

// -------------------------------------------------------------- plain kernel

__global__ void __launch_bounds__(kPlainThreads, 4) plain_kernel(const DeviceCache cache, uint64_t first_l,
                                                              uint32_t alpha_cap, const LaunchBuffers buf) {
    extern __shared__ __align__(16) unsigned char smem[];
    HotRec* s_alpha = reinterpret_cast<HotRec*>(smem);
    uint8_t* s_tab = reinterpret_cast<uint8_t*>(s_alpha + alpha_cap);
    __shared__ RowConst s_row;
    const uint32_t row = blockIdx.x / kSlices, slice = blockIdx.x % kSlices;
    const uint64_t l = first_l + row;
    for (uint32_t i = threadIdx.x; i < kTableBytes; i += kPlainThreads) s_tab[i] = buf.tables[i];
    if (threadIdx.x == 0) row_setup(cache, l, s_row);
    const uint32_t a0 = cache.seg_off[l];
    const uint32_t na = cache.seg_off[l + 1] - a0;
    for (uint32_t i = threadIdx.x; i < na; i += kPlainThreads) s_alpha[i] = scale2(cache.hot[a0 + i]);
    __syncthreads();
    Acc acc{0, 0, 0, 0, 0, 0};
    const uint64_t n = cache.limit;
    for (uint64_t m = l + slice * kPlainThreads + threadIdx.x; m <= n; m += kSlices * kPlainThreads) {
        const uint32_t s0 = cache.seg_off[m], s1 = cache.seg_off[m + 1];
        const uint32_t kind = classify(s_row, cache, (uint32_t)m, s1 - s0 - 1);
        if (kind == kSkip) continue;
        acc.processed += 1;
        if (kind == kMerged) {
            acc.merged += 1;
            push_merged(buf, (uint32_t)l, (uint32_t)m, row);
            continue;
        }
        uint32_t cc_c, cc_r;
        const PairCtx c = make_ctx(s_row, m, cc_c, cc_r);
        acc.prod += 1;
        acc.cand += cc_c;
        acc.r16 += cc_r;
        for (uint32_t j = s0; j < s1; ++j) {
            const HotRec b = cache.hot[j];
            record_loop(s_alpha, na, b, c, s_tab, cache, a0, j, l, m, row, acc, buf);
        }
    }
    flush_acc(acc, &buf.rows[row]);
}

// ------------------------------------------------------------- merged kernel

// Terms of a pair that shares split primes: merged exponents e = a + b
// (gpu_search_v42.cu:318-338), split in two groups whose products form the
// two lists; each list is the group's free set plus its central value.
struct Group {
    uint32_t count;
    uint32_t p[kMaxTerms], e[kMaxTerms];
    uint32_t base[kMaxTerms];   // index of the term's first value in the prime-power table
    uint32_t block[kMaxTerms];  // number of free vectors whose first non-central index is i
    uint32_t suffix[kMaxTerms]; // prod_{j>i} (4 e_j + 1)
    uint32_t free_count;
    i128 scale;                 // real factor folded into every value of the group
};

struct MergedShared {
    Group g[2];
    PairCtx ctx;
    uint64_t l, m;
    uint32_t row, ok, cc_cand, cc_r16;
};

__device__ void group_finish(Group& g) {
    uint32_t total = 0;
    for (int i = (int)g.count - 1, suffix = 1; i >= 0; --i) {
        g.suffix[i] = (uint32_t)suffix;
        g.block[i] = 2 * g.e[i] * (uint32_t)suffix;
        suffix *= 4 * (int)g.e[i] + 1;
    }
    for (uint32_t i = 0; i < g.count; ++i) total += g.block[i];
    g.free_count = total;
}

// Exact value of list entry k of group g (k == free_count: central value).
__device__ void group_value(const DeviceCache& cache, const Group& g, uint32_t k, i128& re, i128& im) {
    i128 xr = g.scale, xi = 0;
    uint32_t i = 0;
    if (k < g.free_count) {
        while (k >= g.block[i]) {
            k -= g.block[i];
            ++i;
        }
    } else {
        i = g.count;
    }
    for (uint32_t j = 0; j < i; ++j) {  // central values of the leading terms: p^(2e), real
        xr *= cache.pp_exact[2 * (g.base[j] + 2 * g.e[j])];
    }
    if (i < g.count) {
        uint32_t r = k / g.suffix[i];
        uint32_t rem = k - r * g.suffix[i];
        uint32_t digits[kMaxTerms];
        for (uint32_t j = g.count - 1; j > i; --j) {
            uint32_t s = 4 * g.e[j] + 1;
            digits[j] = rem % s;
            rem /= s;
        }
        digits[i] = r;
        for (uint32_t j = i; j < g.count; ++j) {
            i128 vr = cache.pp_exact[2 * (g.base[j] + digits[j])];
            i128 vi = cache.pp_exact[2 * (g.base[j] + digits[j]) + 1];
            i128 nr = xr * vr - xi * vi, ni = xr * vi + xi * vr;
            xr = nr;
            xi = ni;
        }
    }
    re = xr;
    im = xi;
}

__device__ HotRec hot_of(i128 re, i128 im, bool central) {
    HotRec h;
    h.re = i128_to_float(re);
    h.im = i128_to_float(im);
    h.rre = pack_residues(re) | (central ? kCentralBit : 0u);
    h.rim = pack_residues(im);
    return h;
}

__device__ void merged_setup(const DeviceCache& cache, uint4 q, MergedShared& S, uint32_t list_cap) {
    uint64_t l = q.x, m = q.y;
    S.l = l;
    S.m = m;
    S.row = q.z;
    S.ok = 1;
    // factor l and m (split primes with exponents, and the fixed parts)
    uint32_t lp[9], le[9], mp[9], me[9], nl = 0, nm = 0;
    i128 fixed = 2;
    for (int side = 0; side < 2; ++side) {
        uint64_t x = side ? m : l;
        uint32_t* P = side ? mp : lp;
        uint32_t* E = side ? me : le;
        uint32_t& cnt = side ? nm : nl;
        while (x > 1) {
            uint32_t p = cache.spf[x], a = 0;
            do {
                x /= p;
                ++a;
            } while (x % p == 0);
            if ((p & 3u) == 1u) {
                P[cnt] = p;
                E[cnt] = a;
                ++cnt;
            } else {
                for (uint32_t t = 0; t < 2 * a; ++t) fixed *= p;
            }
        }
    }
    uint32_t tp[kMaxTerms], te[kMaxTerms], count = 0;
    uint32_t i = 0, j = 0;
    while (i < nl || j < nm) {
        if (j == nm || (i < nl && lp[i] < mp[j])) {
            tp[count] = lp[i];
            te[count++] = le[i++];
        } else if (i == nl || mp[j] < lp[i]) {
            tp[count] = mp[j];
            te[count++] = me[j++];
        } else {
            tp[count] = lp[i];
            te[count++] = le[i++] + me[j++];
        }
    }
    // greedy split by list size: largest terms first, each to the smaller group
    uint32_t order[kMaxTerms];
    for (uint32_t t = 0; t < count; ++t) order[t] = t;
    for (uint32_t a = 1; a < count; ++a)
        for (uint32_t b = a; b > 0 && te[order[b]] > te[order[b - 1]]; --b) {
            uint32_t tmp = order[b];
            order[b] = order[b - 1];
            order[b - 1] = tmp;
        }
    uint64_t w[2] = {1, 1};
    S.g[0].count = S.g[1].count = 0;
    for (uint32_t t = 0; t < count; ++t) {
        uint32_t idx = order[t];
        int side = w[0] <= w[1] ? 0 : 1;
        Group& g = S.g[side];
        g.p[g.count] = tp[idx];
        g.e[g.count] = te[idx];
        g.base[g.count] = cache.pp_base[tp[idx]] + pp_exponent_offset(te[idx]);
        ++g.count;
        w[side] *= 4 * te[idx] + 1;
        if (te[idx] > cache.max_exponent) S.ok = 0;
    }
    group_finish(S.g[0]);
    group_finish(S.g[1]);
    S.g[0].scale = fixed;
    S.g[1].scale = 1;
    if (S.g[0].free_count + S.g[1].free_count + 2 > list_cap) S.ok = 2;  // too big for this path
}

__global__ void __launch_bounds__(kMergedThreads, 4) merged_big_kernel(const DeviceCache cache, const LaunchBuffers buf) {
    __shared__ MergedShared S;
    __shared__ __align__(16) HotRec s_list[kMergedListCap];
    __shared__ uint8_t s_tab[kTableBytes];
    __shared__ RowConst s_row;
    for (uint32_t i = threadIdx.x; i < kTableBytes; i += kMergedThreads) s_tab[i] = buf.tables[i];
    const uint32_t count = min(*buf.big_count, buf.big_cap);
    for (uint32_t q = blockIdx.x; q < count; q += gridDim.x) {
        __syncthreads();
        if (threadIdx.x == 0) {
            uint4 e = buf.big_queue[q];
            merged_setup(cache, e, S, kMergedListCap);
            row_setup(cache, e.x, s_row);
            uint32_t cc_c, cc_r;
            S.ctx = make_ctx(s_row, e.y, cc_c, cc_r);
            S.cc_cand = cc_c;
            S.cc_r16 = cc_r;
            if (S.ok != 1) atomicOr(buf.error_flags, 2u);
        }
        __syncthreads();
        if (S.ok != 1) continue;
        const uint32_t na = S.g[0].free_count + 1, nb = S.g[1].free_count + 1;
        HotRec* s_a = s_list;
        HotRec* s_b = s_list + na;
        for (uint32_t k = threadIdx.x; k < na + nb; k += kMergedThreads) {
            int side = k < na ? 0 : 1;
            uint32_t idx = side ? k - na : k;
            i128 re, im;
            group_value(cache, S.g[side], idx, re, im);
            s_list[k] = hot_of(re, im, idx == S.g[side].free_count);
        }
        __syncthreads();
        Acc acc{0, 0, 0, 0, 0, 0};
        if (threadIdx.x == 0) {
            acc.prod += 1;
            acc.cand += S.cc_cand;
            acc.r16 += S.cc_r16;
        }
        const uint32_t total = na * nb;
        const float rcp = 1.0f / (float)nb;
        for (uint32_t k = threadIdx.x; k < total; k += kMergedThreads) {
            uint32_t ka = (uint32_t)((float)k * rcp);
            int32_t kb = (int32_t)(k - ka * nb);
            while (kb < 0) {
                --ka;
                kb += (int32_t)nb;
            }
            while (kb >= (int32_t)nb) {
                ++ka;
                kb -= (int32_t)nb;
            }
            const HotRec a = s_a[ka], b = s_b[kb];
            const bool ca = (a.rre & kCentralBit) != 0, cb = (b.rre & kCentralBit) != 0;
            if (ca & cb) continue;
            const bool two = !(ca | cb);
            acc.prod += two ? 2u : 1u;
            uint32_t st = eval_pair(a, b, two, S.ctx, s_tab, acc);
            if (st) {
                i128 ar, ai, br, bi;
                group_value(cache, S.g[0], ka, ar, ai);
                group_value(cache, S.g[1], (uint32_t)kb, br, bi);
                resolve_exact(st, ar, ai, br, bi, S.l, S.m, cache.limit, S.row, s_tab, acc, buf);
            }
        }
        flush_acc(acc, &buf.rows[S.row], true);
    }
}

// Shared-prime pairs, one warp per pair: lane 0 factors the pair and splits
// its terms, the lanes build both lists in the warp's shared slice, then all
// (alpha, beta) combinations are evaluated in lockstep rounds of 32.  Pairs
// whose lists exceed the slice go to the big-pair queue (one CTA per pair).
__global__ void __launch_bounds__(kWarpPairThreads, 2) merged_kernel(const DeviceCache cache, const LaunchBuffers buf) {
    __shared__ MergedShared S[kWarpPairWarps];
    __shared__ RowConst R[kWarpPairWarps];
    __shared__ __align__(16) HotRec s_list[kWarpPairWarps][kWarpListCap];
    __shared__ uint8_t s_tab[kTableBytes];
    for (uint32_t i = threadIdx.x; i < kTableBytes; i += kWarpPairThreads) s_tab[i] = buf.tables[i];
    __syncthreads();
    const uint32_t warp = threadIdx.x / 32, lane = threadIdx.x & 31;
    MergedShared& P = S[warp];
    HotRec* list = s_list[warp];
    const uint32_t count = min(*buf.merged_count, buf.merged_cap);
    const uint32_t stride = gridDim.x * kWarpPairWarps;
    for (uint32_t q = blockIdx.x * kWarpPairWarps + warp; q < count; q += stride) {
        __syncwarp();
        if (lane == 0) {
            uint4 e = buf.merged_queue[q];
            merged_setup(cache, e, P, kWarpListCap);
            if (P.ok == 1) {
                row_setup(cache, e.x, R[warp]);
                uint32_t cc_c, cc_r;
                P.ctx = make_ctx(R[warp], e.y, cc_c, cc_r);
                P.cc_cand = cc_c;
                P.cc_r16 = cc_r;
            } else if (P.ok == 2) {
                unsigned int idx = atomicAdd(buf.big_count, 1u);
                if (idx < buf.big_cap)
                    buf.big_queue[idx] = e;
                else
                    atomicOr(buf.error_flags, 2u);
            } else {
                atomicOr(buf.error_flags, 2u);
            }
        }
        __syncwarp();
        if (P.ok != 1) continue;
        const uint32_t na = P.g[0].free_count + 1, nb = P.g[1].free_count + 1;
        for (uint32_t k = lane; k < na + nb; k += 32) {
            int side = k < na ? 0 : 1;
            uint32_t idx = side ? k - na : k;
            __int128 re, im;
            group_value(cache, P.g[side], idx, re, im);
            list[k] = hot_of(re, im, idx == P.g[side].free_count);
        }
        __syncwarp();
        Acc acc{0, 0, 0, 0, 0, 0};
        if (lane == 0) {
            acc.prod += 1;
            acc.cand += P.cc_cand;
            acc.r16 += P.cc_r16;
        }
        const PairCtx c = P.ctx;
        const uint32_t total = na * nb;
        const float rcp = 1.0f / (float)nb;
        for (uint32_t base = 0; base < total; base += 32) {
            const uint32_t k = base + lane;
            uint32_t ka = (uint32_t)((float)k * rcp);
            int32_t kb = (int32_t)k - (int32_t)(ka * nb);
            while (kb < 0) {
                --ka;
                kb += (int32_t)nb;
            }
            while (kb >= (int32_t)nb) {
                ++ka;
                kb -= (int32_t)nb;
            }
            if (k < total) {
                const HotRec a = list[ka], b = list[na + kb];
                const bool ca = (a.rre & kCentralBit) != 0, cb = (b.rre & kCentralBit) != 0;
                if (!(ca & cb)) {
                    const bool two = !(ca | cb);
                    acc.prod += two ? 2u : 1u;
                    uint32_t st = eval_pair(a, b, two, c, s_tab, acc);
                    if (st) {
                        __int128 ar, ai, br, bi;
                        group_value(cache, P.g[0], ka, ar, ai);
                        group_value(cache, P.g[1], (uint32_t)kb, br, bi);
                        resolve_exact(st, ar, ai, br, bi, P.l, P.m, cache.limit, P.row, s_tab, acc, buf);
                    }
                }
            }
        }
        flush_acc(acc, &buf.rows[P.row], true);
    }
}

// INT32 throughput probe: 8 independent chains per thread, each step one
// IMAD and one LOP3 (the multiply and logic pipes the search loop uses),
// i.e. 16 integer instructions per unrolled step; the result is stored so
// nothing is eliminated.
__global__ void __launch_bounds__(256) int_peak_kernel(uint32_t iters, uint32_t seed, uint32_t* out) {
    uint32_t a[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = threadIdx.x * (i + 3) + blockIdx.x + seed;
    for (uint32_t it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            a[i] = a[i] * 0x9E3779B1u + (uint32_t)i;
            a[i] = (a[i] ^ (a[i] >> 7)) & 0x7FFFFFFFu;
        }
    }
    uint32_t r = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) r ^= a[i];
    if (r == seed) out[0] = r;
}

}  // namespace

double int32_peak_ops(int device, int sm_count, double* ms_out) {
    cudaSetDevice(device);
    uint32_t* out = nullptr;
    if (cudaMalloc(&out, sizeof(uint32_t)) != cudaSuccess) return 0;
    const int blocks = sm_count * 8, threads = 256;
    const uint32_t iters = 1u << 14;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int_peak_kernel<<<blocks, threads>>>(64, 1, out);  // warm-up
    cudaEventRecord(e0);
    int_peak_kernel<<<blocks, threads>>>(iters, 1, out);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (ms_out) *ms_out = ms;
    // per unrolled step: 8 IMAD + 8 shift-xor-and (SHF/LOP3 pairs count as 2)
    double ops = (double)blocks * threads * iters * 8.0 * 3.0;
    return ms > 0 ? ops / (ms * 1e-3) : 0;
}

// ------------------------------------------------------------------ host side

void build_residue_tables(uint8_t* out) {
    auto is4 = [](uint32_t r, uint32_t m) {
        for (uint64_t x = 0; x < m; ++x)
            if (x * x % m * x % m * x % m == r) return true;
        return false;
    };
    for (uint32_t z = 0; z < 720; ++z) {
        bool m16 = (z & 15u) <= 1u;
        bool m9 = is4(z % 9, 9);
        bool m5 = is4(z % 5, 5);
        out[kTabA + z] = (uint8_t)((m16 ? 1u : 0u) | ((m16 && m9 && m5) ? 2u : 0u) |
                                   ((m16 && m9 && z % 5 == 0) ? 4u : 0u));
    }
    for (uint32_t z = 0; z < 625; ++z) out[kTabB + z] = is4(z, 625) ? 1 : 0;
    for (uint32_t z = 0; z < 1547; ++z)
        out[kTabC + z] = (is4(z % 7, 7) && is4(z % 13, 13) && is4(z % 17, 17)) ? 1 : 0;
}

size_t batched_smem_bytes(uint32_t alpha_cap, uint32_t tile_cap) {
    return (size_t)alpha_cap * sizeof(HotRec) + (size_t)tile_cap * sizeof(PairCtx) + kTableBytes;
}

static const void* batched_fn(int threads) {
    switch (threads) {
        case 128: return (const void*)batched_kernel<128>;
        case 512: return (const void*)batched_kernel<512>;
        default: return (const void*)batched_kernel<256>;
    }
}

int batched_max_ctas_per_sm(int threads, size_t smem) {
    const void* fn = batched_fn(threads);
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, threads, smem) != cudaSuccess) return 1;
    return n > 0 ? n : 1;
}

cudaError_t launch_batched(const DeviceCache& cache, const WorkItem* items, uint32_t n_items,
                           const BatchedConfig& cfg, const LaunchBuffers& buf, cudaStream_t stream) {
    size_t smem = batched_smem_bytes(cfg.alpha_cap, cfg.tile_cap);
    const void* fn = batched_fn(cfg.threads);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    switch (cfg.threads) {
        case 128:
            batched_kernel<128><<<cfg.ctas, 128, smem, stream>>>(cache, items, n_items, cfg.alpha_cap, cfg.tile_cap, buf);
            break;
        case 512:
            batched_kernel<512><<<cfg.ctas, 512, smem, stream>>>(cache, items, n_items, cfg.alpha_cap, cfg.tile_cap, buf);
            break;
        default:
            batched_kernel<256><<<cfg.ctas, 256, smem, stream>>>(cache, items, n_items, cfg.alpha_cap, cfg.tile_cap, buf);
            break;
    }
    return cudaGetLastError();
}

cudaError_t launch_plain(const DeviceCache& cache, uint64_t first_l, uint32_t n_rows, uint32_t alpha_cap,
                         const LaunchBuffers& buf, cudaStream_t stream) {
    size_t smem = (size_t)alpha_cap * sizeof(HotRec) + kTableBytes;
    cudaError_t e = cudaFuncSetAttribute((const void*)plain_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    plain_kernel<<<n_rows * kSlices, kPlainThreads, smem, stream>>>(cache, first_l, alpha_cap, buf);
    return cudaGetLastError();
}

cudaError_t launch_merged(const DeviceCache& cache, uint32_t count, const LaunchBuffers& buf, int ctas,
                          cudaStream_t stream) {
    (void)count;
    merged_kernel<<<ctas, kWarpPairThreads, 0, stream>>>(cache, buf);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    merged_big_kernel<<<ctas, kMergedThreads, 0, stream>>>(cache, buf);
    return cudaGetLastError();
}

}  // namespace hss
