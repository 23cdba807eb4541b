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
//   * residues of the product's coordinates mod 9360 and 45917, formed from
//     per-value residues with 32-bit multiplies (exact), and
//   * float coordinates with a proven error bound: |z| = 2 l^2 m^2 is known per
//     pair, so every coordinate's float error is below eps = 2 l^2 m^2 2^-20,
// and only go to exact 128-bit arithmetic when a decision is within eps of a
// window boundary, or when z passes every residue filter and a fourth root n
// inside z's float bounds matches z modulo 9360 * 45917 (a possible hit).
// Counts are therefore exact and every hit is confirmed exactly and rechecked
// in 256-bit arithmetic.
//
// The hot loop is branch-free per (alpha, beta) value pair and tests both
// residue fields of every counted candidate.  Work that only a few lanes need
// (the fourth-root filter of candidates that passed both fields, undecided
// products, products whose both orientations pass the area test) is written
// to a per-warp queue of events and processed 32 at a time, outside the hot
// loop; the root filter's windows are then scanned by the whole warp.
//
// Work shapes.  batched_kernel is persistent: CTAs pull (row l, m-range)
// items from a global cursor; per item the row's values are staged in shared
// memory, and each warp walks the m-side records of 128 roots (read from the
// cache, coalesced) in lockstep rounds against them.  plain_kernel keeps the reference's shape
// (a block per (row, slice), one thread per pair).  The pairs that share a
// split prime (gpu_search_v42.cu:318-341) are set up by merged_setup_kernel (a
// thread per pair, in chunks of the queue) and run by merged_kernel (a warp
// per pair) or, when their lists exceed a warp's slice, merged_big_kernel (a
// CTA per pair).
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include "hss_kernels.h"

namespace hss {
namespace {

using u128 = unsigned __int128;
using i128 = __int128;

constexpr uint32_t kSqA = kModA * kModA;
constexpr uint32_t kSqD = kModD * kModD;
constexpr uint32_t kTabA = 0, kTabD = kModA;  // byte offsets: field-A bytes, then the field-D bit set
constexpr uint32_t kTabD2 = 2 * kModA;        // field-D bit set in the wide copy
constexpr uint32_t kSlices = 8;            // plain kernel: blocks per row
constexpr uint32_t kPlainThreads = 128;    // plain kernel: threads per block
constexpr uint32_t kMergedThreads = 128;   // big shared-prime pairs: one CTA per pair
constexpr uint32_t kMergedListCap = 1536;  // alpha + beta entries of one big pair
constexpr uint32_t kWarpListCap = 160;     // alpha + beta entries of one warp's pair
constexpr uint32_t kMaxTerms = 16;
constexpr uint32_t kQueue = 64;            // events per warp queue
constexpr uint32_t kFull = 0xFFFFFFFFu;

// Window and filter constants of one pair (l, m).
struct PairCtx {
    float lo1, hi1, lo1o, hi1o;  // z = S - t counted iff t in [lo1, hi1]; maybe iff t in [lo1o, hi1o]
    float hi2, hi2o;             // z = S + t counted iff t <= hi2; maybe iff t <= hi2o
    float eps;                   // bound on |float - exact| of a product coordinate
    float sf;                    // S = l^4 + m^4 as float
    uint32_t sres;               // S mod kModA | S mod kModD << 14 | flag5 << 31
    uint32_t dinv;               // inverse of D mod 2^32 (0: pair not on this path)
    uint32_t dthr;               // floor((2^32 - 1) / (8 D))
    uint32_t m;
};

// Row-side value in shared memory: coordinates as float and their packed
// residues (fields A and D; bit 31 of ra: central value).
struct AlphaHot {
    float re, im;
    uint32_t ra, ia;
};

struct Acc {
    uint32_t cand, r16, prod, exact, processed, merged;
};

// Event flags per product p (bits 4p .. 4p+3).
constexpr uint32_t kEvU = 1;   // undecided: count the whole product exactly
constexpr uint32_t kEvDx = 2;  // orientation (x, y) counted, z passed fields A and D: root filter
constexpr uint32_t kEvDy = 4;  // the same for orientation (y, x)
constexpr uint32_t kEvB = 8;   // non-dual pair with both orientations gated: (y, x) still to do

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
__host__ __device__ constexpr uint32_t inverse_odd(uint32_t d) {
    uint32_t x = d;  // correct to 3 bits
    for (int i = 0; i < 4; ++i) x *= 2u - d * x;
    return x;
}

__device__ __forceinline__ bool divides(uint32_t inv, uint32_t thr, uint32_t m) { return m * inv <= thr; }

// 8D | n via one multiply and a rotate: n * D^-1 mod 2^32 rotated right by 3
// is at most floor((2^32-1)/(8D)) exactly when 8D divides n.
__device__ __forceinline__ bool area_gate(uint32_t n, uint32_t dinv, uint32_t dthr) {
    uint32_t h = n * dinv;
    return __funnelshift_r(h, h, 3) <= dthr;
}

__host__ __device__ __forceinline__ uint32_t pow4_mod(uint32_t x, uint32_t m) {
    uint32_t s = x * x % m;
    return s * s % m;
}

// Index checks of the event paths: an index outside its buffer is recorded
// (kErrIndex in the launch's error word, which the host reports as an
// error) and the access is skipped.
constexpr unsigned int kErrIndex = 0x100u;

__device__ __forceinline__ bool index_ok(uint32_t i, uint32_t n, unsigned int* err) {
    if (i < n) return true;
    atomicOr(err, kErrIndex);
    return false;
}

__device__ __forceinline__ uint32_t tab_at(const uint8_t* tab, uint32_t base, uint32_t i, uint32_t n,
                                           unsigned int* err) {
    return index_ok(i, n, err) ? tab[base + i] : 0u;
}

// Bit z of a field-D bit set: z is a fourth-power residue mod 17, 37 and 73.
__device__ __forceinline__ uint32_t tab_d(const uint32_t* bits, uint32_t z) { return (bits[z >> 5] >> (z & 31u)) & 1u; }

__device__ __forceinline__ const uint32_t* tab_d_bits(const uint8_t* tab, uint32_t offset) {
    return reinterpret_cast<const uint32_t*>(tab + offset);
}

__device__ __forceinline__ uint32_t tab_d_at(const uint32_t* bits, uint32_t z, unsigned int* err) {
    return index_ok(z, kModD, err) ? tab_d(bits, z) : 0u;
}

// ----------------------------------------------------------- 256-bit check

// Heron recheck (done on the host by the reference's CPU search,
// search_v18.cpp:481-501): the four Heron factors of sides l^2, m^2, n^2 are
// positive and their product equals (4A)^2, compared in 256-bit arithmetic.
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
// entry; then z = l^4 + m^4 - D is tested exactly.  The residue tables hold
// necessary conditions for z = n^4 (with 5 | n when 5 divides neither l nor
// m); the fourth root itself is found and checked in 128-bit arithmetic.
__device__ void exact_test_d(const ExactPair& p, i128 d, i128 area4, uint32_t& cand, uint32_t& r16,
                             const uint8_t* tab, const LaunchBuffers& buf) {
    ++cand;
    i128 sz = (i128)p.l4 + (i128)p.m4 - d;
    if (sz < 0 || (u128)sz < p.m4 || (u128)sz > p.n4) return;
    u128 z = (u128)sz;
    if (((uint32_t)z & 15u) > 1u) return;
    ++r16;
    if (!(tab[kTabA + mod_u128_small(z, kModA)] & ((p.flags & 2u) ? 4u : 2u))) return;
    if (!tab_d(tab_d_bits(tab, kTabD), mod_u128_small(z, kModD))) return;
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

// Exact evaluation of the product (ar + i ai) * (br + i bi), or of
// (ar + i ai) * conj(br + i bi) when conj_b, for the orientations in `omask`
// (bit 0: (D, 4A) = (x, y); bit 1: (y, x), taken only when x != +-y as in
// gpu_search_v42.cu:196-200).  Hits are recorded; counts are returned.
__device__ __noinline__ void exact_eval(i128 ar, i128 ai, i128 br, i128 bi, bool conj_b, uint32_t omask,
                                        uint64_t l, uint64_t m, uint64_t n, uint32_t row, const uint8_t* tab,
                                        const LaunchBuffers& buf, uint32_t* cand, uint32_t* r16) {
    ExactPair p = exact_pair(l, m, n, row);
    i128 bim = conj_b ? -bi : bi;
    i128 x = ar * br - ai * bim, y = ar * bim + ai * br;
    uint32_t c = 0, r = 0;
    if (omask & 1u) exact_test_pair(p, x, y, c, r, tab, buf);
    if ((omask & 2u) && x != y && x != -y) exact_test_pair(p, y, x, c, r, tab, buf);
    *cand = c;
    *r16 = r;
}

// ------------------------------------------------------------ fast path

struct Window {
    bool in1, in2, und;
};

// Window decision for t = |D| from its float value: counted terms (z = S - t
// and z = S + t) and whether any boundary is within the error bound.
__device__ __forceinline__ Window window(float t, const PairCtx& c) {
    Window w;
    w.in1 = (t >= c.lo1) & (t <= c.hi1);
    w.in2 = t <= c.hi2;
    bool maybe1 = (t >= c.lo1o) & (t <= c.hi1o);
    bool maybe2 = t <= c.hi2o;
    // a counted term also needs the sign of D, certain once t > eps
    w.und = (maybe1 & !w.in1) | (maybe2 & !w.in2) | ((w.in1 | w.in2) & (t < c.eps));
    return w;
}

__device__ __forceinline__ uint32_t add_mod(uint32_t a, uint32_t b, uint32_t m) {
    uint32_t s = a + b;
    return s >= m ? s - m : s;
}

__device__ __forceinline__ uint32_t sub_mod(uint32_t a, uint32_t b, uint32_t m) {
    return a >= b ? a - b : a + m - b;
}

// Hot evaluation of one (alpha, beta) value pair: products p = 0 (alpha*beta)
// and, when neither value is central, p = 1 (alpha*conj(beta)).  Counts the
// candidates and mod-16 survivors it can decide; returns event flags for the
// rest (0 for nearly all pairs).
//
// Which orientations can pass the area test is a property of the pair: when
// l*m is even and 3 and 5 both divide l*m, both coordinates of every product
// are = 0 mod 8*9 (the powers of 1+i and of 3 in 2 l^2 m^2 divide both) and
// no mod-5 condition applies, so both orientations pass (DUAL).  Otherwise at
// most one does: for odd l*m only the coordinate with the higher power of 2 is
// = 0 mod 8; if 3 (or 5) does not divide 2 l^2 m^2 it divides at most one leg
// of the triple (x, y, 2 l^2 m^2).  The non-dual path evaluates the one gated
// orientation and raises kEvB if both ever pass, so it stays exact regardless.
// MODE 0: non-dual pair, 1: dual pair, 2: either (dual_rt), one code copy for
// kernels whose lanes meet both kinds and whose instruction cache is tight.
// WIDE: `tab` is the wide copy (tables over two periods), so z residues are
// indexed as S + d and S + M - d without a reduction; otherwise the compact one.
// 32-bit multiply-add d = a b + c (mod 2^32), kept as one fused instruction so
// that the residue coordinates go to the multiply-add pipe, not the integer ALU.
__device__ __forceinline__ uint32_t imad(uint32_t a, uint32_t b, uint32_t c) {
    uint32_t d;
    asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}

// FUSED: coordinates by multiply-adds with the negated beta residues (worth it
// where beta is fixed across the loop, so the negation is hoisted out of it).
template <int MODE, bool WIDE = false, bool FUSED = false>
__device__ __forceinline__ uint32_t eval_fast(const AlphaHot& a, float br, float bi, uint32_t brw, uint32_t biw,
                                              bool cb, const PairCtx& c, const uint8_t* tab, Acc& acc,
                                              bool dual_rt = false) {
    const uint32_t* tabd = tab_d_bits(tab, WIDE ? kTabD2 : kTabD);
    const bool dual = MODE == 2 ? dual_rt : MODE == 1;
    const bool ca = (a.ra >> 31) != 0;
    const uint32_t ar = a.ra & kMaskA, ai = a.ia & kMaskA, bra = brw & kMaskA, bia = biw & kMaskA;
    const uint32_t ad = (a.ra >> kShiftD) & kMaskD, adi = (a.ia >> kShiftD) & kMaskD;
    const uint32_t bd = (brw >> kShiftD) & kMaskD, bdi = (biw >> kShiftD) & kMaskD;
    // coordinates of alpha beta (p = 0) and alpha conj(beta) (p = 1) in each
    // field, all in [0, 2 M^2): X0 = ar br - ai bi + M^2, Y0 = ar bi + ai br,
    // X1 = ar br + ai bi, Y1 = ai br - ar bi + M^2 (nbi = -bi mod 2^32)
    uint32_t XA[2], YA[2], XDs[2], YDs[2];
    if (FUSED) {
        const uint32_t nbia = 0u - bia, nbdi = 0u - bdi;
        XA[0] = imad(ar, bra, imad(ai, nbia, kSqA));
        XA[1] = imad(ar, bra, ai * bia);
        YA[0] = imad(ar, bia, ai * bra);
        YA[1] = imad(ai, bra, imad(ar, nbia, kSqA));
        XDs[0] = imad(ad, bd, imad(adi, nbdi, kSqD));
        XDs[1] = imad(ad, bd, adi * bdi);
        YDs[0] = imad(ad, bdi, adi * bd);
        YDs[1] = imad(adi, bd, imad(ad, nbdi, kSqD));
    } else {
        const uint32_t p1 = ar * bra, p2 = ai * bia, p3 = ar * bia, p4 = ai * bra;
        const uint32_t q1 = ad * bd, q2 = adi * bdi, q3 = ad * bdi, q4 = adi * bd;
        XA[0] = p1 + kSqA - p2;
        XA[1] = p1 + p2;
        YA[0] = p3 + p4;
        YA[1] = p4 + kSqA - p3;
        XDs[0] = q1 + kSqD - q2;
        XDs[1] = q1 + q2;
        YDs[0] = q3 + q4;
        YDs[1] = q4 + kSqD - q3;
    }
    const float f1 = a.re * br, f2 = a.im * bi, f3 = a.re * bi, f4 = a.im * br;
    const uint32_t sA = c.sres & kMaskA, sD = (c.sres >> kShiftD) & kMaskD;
    const uint32_t sel = (c.sres >> 31) ? 4u : 2u;
    uint32_t flags = 0, cnt = 0, r16 = 0;
#pragma unroll
    for (int p = 0; p < 2; ++p) {
        const bool valid = p == 0 ? !(ca & cb) : !(ca | cb);
        const uint32_t X = XA[p], Y = YA[p], XD = XDs[p], YD = YDs[p];
        const float xf = p ? f1 + f2 : f1 - f2;
        const float yf = p ? f4 - f3 : f3 + f4;
        const bool gx = valid & area_gate(Y, c.dinv, c.dthr);  // (D, 4A) = (x, y)
        const bool gy = valid & area_gate(X, c.dinv, c.dthr);  // (D, 4A) = (y, x)
        uint32_t f = 0, pc = 0, pr = 0;
        bool und = false;
#pragma unroll
        for (int o = 0; o < (MODE == 0 ? 1 : 2); ++o) {
            if (MODE == 2 && o == 1 && !dual) break;
            // dual: o = 0 is (x, y), o = 1 is (y, x); otherwise the gated one
            const bool g = dual ? (o ? gy : gx) : (gx | gy);
            const bool oy = dual ? (o == 1) : !gx;
            const float d = oy ? yf : xf;
            const uint32_t dres = oy ? Y : X;
            const Window w = window(fabsf(d), c);
            und |= g & w.und;
            const bool ok = g & !w.und;
            // z = S - t and S + t for t = |d|: S -+ d, swapped when d < 0.
            // Wide tables: t mod M is taken once (M - (d mod M) when d < 0,
            // which is M for a multiple of M, still inside two periods) and
            // both indices come from multiply-adds, off the integer ALU.
            const bool neg = d < 0.f;
            const uint32_t dA = dres % kModA;
            uint32_t z1, z2;
            if (WIDE) {
                const uint32_t tA = neg ? kModA - dA : dA;
                z1 = imad(tA, 0xFFFFFFFFu, sA + kModA);
                z2 = imad(tA, 1u, sA);
            } else {
                const uint32_t uA = sub_mod(sA, dA, kModA), vA = add_mod(sA, dA, kModA);
                z1 = neg ? vA : uA;
                z2 = neg ? uA : vA;
            }
            const uint32_t m1 = (ok & w.in1) ? tab[kTabA + z1] : 0u;
            const uint32_t m2 = (ok & w.in2) ? tab[kTabA + z2] : 0u;
            pc += ok ? (uint32_t)w.in1 + (uint32_t)w.in2 : 0u;
            pr += (m1 & 1u) + (m2 & 1u);
            // field D of the terms that passed field A
            const uint32_t dD = (oy ? YD : XD) % kModD;
            uint32_t y1, y2;
            if (WIDE) {
                const uint32_t tD = neg ? kModD - dD : dD;
                y1 = imad(tD, 0xFFFFFFFFu, sD + kModD);
                y2 = imad(tD, 1u, sD);
            } else {
                const uint32_t uD = sub_mod(sD, dD, kModD), vD = add_mod(sD, dD, kModD);
                y1 = neg ? vD : uD;
                y2 = neg ? uD : vD;
            }
            const uint32_t e1 = (m1 & sel) ? tab_d(tabd, y1) : 0u;
            const uint32_t e2 = (m2 & sel) ? tab_d(tabd, y2) : 0u;
            f |= (e1 | e2) ? (oy ? kEvDy : kEvDx) : 0u;
        }
        if (!dual) f |= (gx & gy) ? kEvB : 0u;
        // an undecided product is counted whole on the exact path instead
        cnt += und ? 0u : pc;
        r16 += und ? 0u : pr;
        flags |= (und ? kEvU : f) << (4 * p);
    }
    acc.cand += cnt;
    acc.r16 += r16;
    return flags;
}

// Gaussian products of a pair whose two sides have na and nb values (each
// list or segment ending with its central value): two per combination of
// non-central values (alpha beta and alpha conj(beta)), one when exactly one
// value is central, and the all-central product, 2 na nb - na - nb + 1.
__device__ __forceinline__ uint32_t pair_products(uint32_t na, uint32_t nb) { return 2 * na * nb - na - nb + 1; }

// A possible hit needs some n in [m, N] with n^4 = z.  From z's float bounds
// (|error| below sf 2^-22 + eps + |z| 2^-22) take the window of n with n^4
// inside them, and keep the candidate only if some n of the window has
// n^4 = z mod 9360 and 45917.  The float fourth root sqrtf(sqrtf(x)) is
// within 1.5 * 2^-24 relative of x^(1/4) (two correctly rounded square
// roots), so scaling by 1 -+ 2^-22 (and rounding once more) keeps the bounds
// on the safe side; 2 units are added on top.  Float and 32-bit integers only.
__device__ __forceinline__ void root_window(float zf, const PairCtx& c, uint32_t n_limit, uint32_t& nlo,
                                            uint32_t& nhi) {
    const float ez = c.sf * 0x1p-22f + c.eps + fabsf(zf) * 0x1p-22f;
    const float lo = fmaxf(zf - ez, 0.f), hi = zf + ez;
    const float rlo = sqrtf(sqrtf(lo)) * (1.f - 0x1p-22f), rhi = sqrtf(sqrtf(hi)) * (1.f + 0x1p-22f);
    const uint32_t m = c.m & 0x7FFFFFFFu;
    const uint32_t flo = __float2uint_rd(rlo), fhi = __float2uint_ru(rhi);
    nlo = flo > m + 2 ? flo - 2 : m;
    nhi = fhi + 2 < n_limit ? fhi + 2 : n_limit;
}

__device__ __forceinline__ bool root_match(uint32_t n, uint32_t zres) {
    return pow4_mod(n % kModA, kModA) == (zres & kMaskA) &&
           pow4_mod(n % kModD, kModD) == ((zres >> kShiftD) & kMaskD);
}

// First n >= nlo with the parity of z (n^4 = z mod 2 forces n = z mod 2;
// bit 0 of zres is z mod 2, as 2 divides 9360): only every second n of a
// window can be a root.
__device__ __forceinline__ uint32_t root_first(uint32_t nlo, uint32_t zres) { return nlo + ((nlo ^ zres) & 1u); }

// One thread scans the window (paths without a warp queue).
__device__ bool root_scan(uint32_t nlo, uint32_t nhi, uint32_t zres) {
    for (uint32_t n = root_first(nlo, zres); n <= nhi; n += 2)
        if (root_match(n, zres)) return true;
    return false;
}

// A root-filter request left by an event for its warp: the window and packed
// residues of one counted term, and the orientation (tag = 2p + o) whose
// exact hit test it gates.  The warp scans the requests of all its lanes
// together: their candidate roots (every second n of each window) are laid
// end to end and taken 32 at a time, one per lane, instead of one lane
// walking a window while the others wait.
struct RootReq {
    uint32_t nlo, nhi, zres, tag;
};
constexpr uint32_t kReqPerLane = 2;  // per event; further terms are scanned by the lane itself

// Number of candidate roots of a request.
__device__ __forceinline__ uint32_t root_count(const RootReq& rq) {
    const uint32_t n0 = root_first(rq.nlo, rq.zres);
    return n0 <= rq.nhi ? (rq.nhi - n0) / 2 + 1 : 0u;
}

// Scans the requests wreq[lane * kReqPerLane + r], r < cnt (cnt per lane,
// at most kReqPerLane); returns, per lane, the tags of its requests whose
// window holds an n with n^4 = z in both residue fields.  All 32 lanes call it.
__device__ __forceinline__ uint32_t root_scan_requests(const RootReq* wreq, uint32_t cnt, uint32_t lane) {
    uint32_t num0 = 0, mine = 0;
#pragma unroll
    for (uint32_t r = 0; r < kReqPerLane; ++r) {
        const uint32_t c = r < cnt ? root_count(wreq[lane * kReqPerLane + r]) : 0u;
        if (r == 0) num0 = c;
        mine += c;
    }
    uint32_t incl = mine;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t t = __shfl_up_sync(kFull, incl, d);
        if (lane >= (uint32_t)d) incl += t;
    }
    const uint32_t total = __shfl_sync(kFull, incl, 31), excl = incl - mine;
    uint32_t passed = 0;
    for (uint32_t base = 0; base < total; base += 32) {
        const uint32_t s = base + lane;
        // owning lane of candidate s: the first lane whose inclusive sum exceeds s
        uint32_t owner = 0;
#pragma unroll
        for (uint32_t step = 16; step >= 1; step >>= 1) {
            const uint32_t v = __shfl_sync(kFull, incl, owner + step - 1);
            if (v <= s) owner += step;
        }
        owner &= 31u;
        uint32_t off = s - __shfl_sync(kFull, excl, owner);
        const uint32_t n0 = __shfl_sync(kFull, num0, owner);
        const uint32_t r = off < n0 ? 0u : 1u;
        off -= r ? n0 : 0u;
        bool match = false;
        uint32_t tag = 0;
        if (s < total) {
            const RootReq rq = wreq[owner * kReqPerLane + r];
            tag = rq.tag;
            match = root_match(root_first(rq.nlo, rq.zres) + 2u * off, rq.zres);
        }
        uint32_t mm = __ballot_sync(kFull, match);
        while (mm) {  // rare: a possible root
            const uint32_t src = __ffs(mm) - 1;
            mm &= mm - 1;
            const uint32_t o = __shfl_sync(kFull, owner, src), t = __shfl_sync(kFull, tag, src);
            if (lane == o) passed |= 1u << t;
        }
    }
    return passed;
}

// Exact coordinates for the rare exact path.
struct ExactValues {
    __int128 ar, ai, br, bi;
};

__device__ __forceinline__ uint32_t pair_m(const PairCtx& c) { return c.m & 0x7FFFFFFFu; }
__device__ __forceinline__ bool pair_dual(const PairCtx& c) { return (c.m >> 31) != 0; }

// Exact work raised by an event, done later by exact_kernel: count a whole
// product, count one orientation, or test one orientation for a hit.
constexpr uint32_t kExCount = 0, kExOrient = 1, kExHit = 2;

// Appends one exact work item (a, b: exact-value indices; for shared-prime
// pairs, list entries) to the global exact queue.
__device__ __forceinline__ void push_exact(const LaunchBuffers& buf, uint32_t kind, uint32_t a, uint32_t b, uint32_t l,
                                           uint32_t m, uint32_t row, bool shared_prime) {
    unsigned int idx = atomicAdd(buf.exact_count, 1u);
    if (idx < buf.exact_cap)
        buf.exact_queue[idx] = ExactItem{kind | (shared_prime ? 16u : 0u), a, b, l, m, row, 0u, 0u};
    else
        atomicOr(buf.error_flags, 4u);
}

// Where an event's exact work goes: the exact-value indices (a, b) of its two
// values, the pair and its row, and whether the values are shared-prime
// list entries.  Passed by value, so no pointer to a caller's locals crosses
// an out-of-line call.
struct EventSink {
    const LaunchBuffers* buf;
    uint32_t a, b, l, m, row, shared_prime;
    const uint32_t* tabd;  // field-D bit set of the kernel's shared-memory table copy
};

__device__ __forceinline__ void sink_push(const EventSink& s, uint32_t kind) {
    push_exact(*s.buf, kind, s.a, s.b, s.l, s.m, s.row, s.shared_prime != 0);
}

// One counted orientation o of product p (p = 1: alpha * conj(beta)) through
// the residue filters.  The coordinate D of the orientation is u + v, u - v
// or v - u with u, v = (ar br, ai bi) for o = 0 and (ar bi, ai br) for o = 1;
// both residue fields are computed branch-free in p and o, so lanes holding
// different orientations run one instruction stream.  Counted terms whose z
// passes the field-A and field-D tables go to the root filter: left as
// requests in `slots` while there is room, else scanned here; returns true
// when such a scan found a possible root.
// `tab` may be the compact or the wide table copy (field A's first period is
// the same in both); `tabd` is that copy's field-D bit set.
__device__ __forceinline__ bool deep_unit(uint32_t p, uint32_t o, const AlphaHot& a, const HotRec& b,
                                          const PairCtx& c, uint32_t n_limit, const uint8_t* tab, RootReq* slots,
                                          uint32_t& nreq, unsigned int* err, const uint32_t* tabd) {
    const bool plus = o != p;
    const float fu = o ? a.re * b.im : a.re * b.re;
    const float fv = o ? a.im * b.re : a.im * b.im;
    const float d = plus ? fu + fv : (o ? fv - fu : fu - fv);
    const float t = fabsf(d);
    const bool neg = d < 0.f;
    // D mod M from the packed residues of one field, signed by d
    auto field = [&](uint32_t shift, uint32_t mask, uint32_t M) {
        const uint32_t wa = (a.ra >> shift) & mask, wai = (a.ia >> shift) & mask;
        const uint32_t wb = (b.rre >> shift) & mask, wbi = (b.rim >> shift) & mask;
        const uint32_t u = o ? wa * wbi : wa * wb, v = o ? wai * wb : wai * wbi;
        const uint32_t r = (plus ? u + v : (o ? v + M * M - u : u + M * M - v)) % M;
        return neg ? (r ? M - r : 0u) : r;
    };
    const uint32_t tA = field(0u, kMaskA, kModA), tD = field(kShiftD, kMaskD, kModD);
    const Window w = window(t, c);
    const uint32_t sA = c.sres & kMaskA, sD = (c.sres >> kShiftD) & kMaskD;
    const uint32_t sel = (c.sres >> 31) ? 4u : 2u;
    bool hit = false;
#pragma unroll
    for (int term = 0; term < 2; ++term) {
        if (!(term ? w.in2 : w.in1)) continue;
        const uint32_t zA = term ? add_mod(sA, tA, kModA) : sub_mod(sA, tA, kModA);
        if (!(tab_at(tab, kTabA, zA, kModA, err) & sel)) continue;
        const uint32_t zD = term ? add_mod(sD, tD, kModD) : sub_mod(sD, tD, kModD);
        if (!tab_d_at(tabd, zD, err)) continue;
        uint32_t nlo, nhi;
        root_window(term ? c.sf + t : c.sf - t, c, n_limit, nlo, nhi);
        const uint32_t zres = zA | (zD << kShiftD);
        if (slots && nreq < kReqPerLane)
            slots[nreq++] = RootReq{nlo, nhi, zres, 2u * p + o};
        else if (!hit && root_scan(nlo, nhi, zres))
            hit = true;
    }
    return hit;
}

// Work of one event (one lane) that holds an undecided product or a
// non-dual product whose both orientations passed, in float and 32-bit
// integer arithmetic only: an undecided product is queued for exact
// counting; the (y, x) orientation of the second kind is decided and counted
// (or queued for exact counting when undecided); every counted orientation
// that is marked, or that was just counted, goes through deep_unit, and
// possible hits are queued for the exact test (kind | p << 2 | o << 3).
//
// With `slots` (warp-queue paths) the root filter of up to kReqPerLane terms
// is left to the warp as requests; orientations that the lane itself found
// possible are returned instead of being queued, so that the caller queues
// each orientation once.  Returns (candidates, mod-16 survivors, requests
// left, possible orientations as bits 2p + o).
__device__ __noinline__ uint4 general_event(uint32_t flags, AlphaHot a, HotRec b, PairCtx c, uint32_t n_limit,
                                            const uint8_t* tab, EventSink sink, RootReq* slots) {
    uint32_t cand = 0, r16 = 0, nreq = 0, passed = 0;
    const uint32_t ar = a.ra & kMaskA, ai = a.ia & kMaskA;
    const uint32_t bra = b.rre & kMaskA, bia = b.rim & kMaskA;
    const uint32_t p1 = ar * bra, p2 = ai * bia, p3 = ar * bia, p4 = ai * bra;
    const float f1 = a.re * b.re, f2 = a.im * b.im, f3 = a.re * b.im, f4 = a.im * b.re;
    const uint32_t sA = c.sres & kMaskA;
    unsigned int* err = sink.buf->error_flags;
    for (uint32_t p = 0; p < 2; ++p) {
        const uint32_t f = (flags >> (4 * p)) & 15u;
        if (!f) continue;
        if (f & kEvU) {
            sink_push(sink, kExCount | p << 2);
            continue;
        }
        const uint32_t X = p ? p1 + p2 : p1 + kSqA - p2;
        const uint32_t Y = p ? p4 + kSqA - p3 : p3 + p4;
        const float xf = p ? f1 + f2 : f1 - f2;
        const float yf = p ? f4 - f3 : f3 + f4;
        for (uint32_t o = 0; o < 2; ++o) {
            const bool full = o == 1 && (f & kEvB);
            const bool deep = (f & (o ? kEvDy : kEvDx)) != 0;
            if (!full && !deep) continue;
            if (full) {
                const float d = o ? yf : xf;
                const Window w = window(fabsf(d), c);
                if (w.und) {
                    sink_push(sink, kExOrient | p << 2 | o << 3);
                    continue;
                }
                cand += (uint32_t)w.in1 + (uint32_t)w.in2;
                const uint32_t dA = (o ? Y : X) % kModA;
                const uint32_t tA = d < 0.f ? (dA ? kModA - dA : 0u) : dA;
                if (w.in1) r16 += tab_at(tab, kTabA, sub_mod(sA, tA, kModA), kModA, err) & 1u;
                if (w.in2) r16 += tab_at(tab, kTabA, add_mod(sA, tA, kModA), kModA, err) & 1u;
            }
            if (deep_unit(p, o, a, b, c, n_limit, tab, slots, nreq, err, sink.tabd)) {
                if (slots)
                    passed |= 1u << (2 * p + o);
                else
                    sink_push(sink, kExHit | p << 2 | o << 3);
            }
        }
    }
    return make_uint4(cand, r16, nreq, passed);
}

// Work of one event: events with an undecided product or a non-dual product
// whose both orientations passed take the general path; the others are a set
// of deep units (one bit per counted orientation whose z passed fields A and
// D).  Returns (candidates, mod-16 survivors, requests left, possible
// orientations) as general_event does.
__device__ __forceinline__ uint4 process_event(uint32_t flags, const AlphaHot& a, const HotRec& b, const PairCtx& c,
                                               uint32_t n_limit, const uint8_t* tab, const EventSink& sink,
                                               RootReq* slots) {
    if (flags & ((kEvU | kEvB) * 0x11u)) return general_event(flags, a, b, c, n_limit, tab, sink, slots);
    uint32_t units = ((flags & kEvDx) ? 1u : 0u) | ((flags & kEvDy) ? 2u : 0u) |
                     ((flags & (kEvDx << 4)) ? 4u : 0u) | ((flags & (kEvDy << 4)) ? 8u : 0u);
    uint32_t nreq = 0, passed = 0;
    while (units) {
        const uint32_t u = __ffs(units) - 1;
        units &= units - 1;
        if (deep_unit(u >> 1, u & 1u, a, b, c, n_limit, tab, slots, nreq, sink.buf->error_flags,
                      sink.tabd)) {
            if (slots)
                passed |= 1u << u;
            else
                sink_push(sink, kExHit | (u >> 1) << 2 | (u & 1u) << 3);
        }
    }
    return make_uint4(0u, 0u, nreq, passed);
}

// Event handler of the cached path: record j against the row value whose
// exact value is at index ka; counts come back by value (x: candidates, y:
// mod-16 survivors).  Out of line, so that the hot loops stay small in the
// instruction cache; it has no 128-bit code, so the call costs few registers.
// With `slots`, x also carries the root requests left (bits 16-19) and the
// orientations already found possible (bits 20-23).
__device__ __noinline__ uint2 cached_event(uint32_t flags, AlphaHot a, HotRec b, PairCtx c, uint32_t ka, uint32_t j,
                                              uint32_t l, uint32_t row, const uint8_t* tab, uint32_t tabd_ofs, uint32_t limit,
                                              const LaunchBuffers* buf, RootReq* slots = nullptr) {
    const EventSink sink{buf, ka, j, l, pair_m(c), row, 0u, tab_d_bits(tab, tabd_ofs)};
    const uint4 r = process_event(flags, a, b, c, limit, tab, sink, slots);
    return make_uint2(r.x | (r.z << 16) | (r.w << 20), r.y);
}

// Queues the exact hit test of each orientation in `tags` (bit 2p + o).
__device__ __noinline__ void push_hits(const LaunchBuffers* buf, uint32_t tags, uint32_t a, uint32_t b, uint32_t l,
                                       uint32_t m, uint32_t row, bool shared_prime) {
    for (uint32_t t = 0; t < 4; ++t)
        if ((tags >> t) & 1u) push_exact(*buf, kExHit | (t >> 1) << 2 | (t & 1u) << 3, a, b, l, m, row, shared_prime);
}

__device__ __forceinline__ void add_event(Acc& acc, uint2 r) {
    acc.cand += r.x;
    acc.r16 += r.y;
}

// ------------------------------------------------------------ pair set-up

enum PairKind : uint32_t { kSkip = 0, kCached = 1, kMerged = 2 };

// Skip rules of gpu_search_v42.cu:305-316 (and search_v18.cpp:336-339, 362):
// both even; an inert prime of l dividing m; neither has a split prime.
// A split prime of l dividing m sends the pair to the shared-prime path.
__device__ __forceinline__ uint32_t classify(const RowInfo& R, uint32_t m, uint32_t free_m) {
    if (R.leven && (m & 1u) == 0) return kSkip;
    bool shared_split = false;
    for (uint32_t i = 0; i < R.nodd; ++i) {
        if (divides(R.pinv[i], R.pthr[i], m)) {
            if (!((R.psplit >> i) & 1u)) return kSkip;
            shared_split = true;
        }
    }
    if (R.free_l == 0 && free_m == 0) return kSkip;
    return shared_split ? kMerged : kCached;
}

// Window and filter constants for pair (l, m); also the analytic count of
// the all-central product (2 l^2 m^2, 0), whose only orientation with a
// nonzero area is D = 0, 4A = 2 l^2 m^2 (counted when the window contains 0;
// z = l^4 + m^4 is never a fourth power).
// eps_scale: 2^-20 for values read from the cache (float coordinates within
// 2^-24 relative, products within 4.9 * 2^-24 of |z|); for shared-prime lists
// multiplied out in float, (12 + 8 K) 2^-24 for a pair whose two groups hold
// K terms (see shared_prime_eps_scale).
__device__ PairCtx make_ctx(const RowInfo& R, uint64_t m, uint32_t& cc_cand, uint32_t& cc_r16,
                           float eps_scale = 0x1p-20f) {
    const uint32_t m32 = (uint32_t)m;  // m <= 3e7
    const uint64_t m2 = (uint64_t)m32 * m32;
    const u128 m4 = (u128)m2 * m2;
    const i128 w = (i128)R.l4 + (i128)m4 - (i128)R.n4;
    // |z| = 2 l^2 m^2 in float from three roundings: within 2^-22 of the
    // exact value, far inside the factor-2 margin of every eps_scale
    const float mf = (float)m32;
    float E = R.l2x2f * (mf * mf) * eps_scale;
    float T2 = R.l4f;
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
        c.lo1 = -1.f;  // non-central products have |D| >= 1 > 0 = max(w, 0)
        c.lo1o = -2.f;
        c.hi2 = -wf - ew;
        c.hi2o = -wf + ew;
    }
    c.eps = E;
    c.sf = u128_to_float(R.l4 + m4);
    bool f3 = R.l3 || m32 % 3 == 0;
    bool f5 = !R.l5 && m32 % 5 != 0;
    // both orientations pass the area test for every product exactly when
    // l*m is even and 3 and 5 both divide l*m (see eval_fast)
    const bool dual = (R.leven || (m & 1) == 0) && f3 && !f5;
    c.m = m32 | (dual ? 0x80000000u : 0u);
    // the area divisor D = 3 (f3 ? 3 : 1) (f5 ? 5 : 1): its inverse and gate
    // threshold floor((2^32 - 1) / (8 D)) are compile-time constants
    constexpr uint32_t kInv3 = inverse_odd(3), kInv9 = inverse_odd(9), kInv15 = inverse_odd(15),
                       kInv45 = inverse_odd(45);
    c.dinv = f3 ? (f5 ? kInv45 : kInv9) : (f5 ? kInv15 : kInv3);
    c.dthr = f3 ? (f5 ? 0xFFFFFFFFu / 360u : 0xFFFFFFFFu / 72u) : (f5 ? 0xFFFFFFFFu / 120u : 0xFFFFFFFFu / 24u);
    const uint32_t mA = m32 % kModA, mD = m32 % kModD;
    uint32_t sA = (R.lmodA + pow4_mod(mA, kModA)) % kModA;
    uint32_t sD = (R.lmodD + pow4_mod(mD, kModD)) % kModD;
    c.sres = sA | (sD << kShiftD) | (f5 ? 0x80000000u : 0u);
    uint32_t areaA = 2u * (R.l2modA * (mA * mA % kModA) % kModA);
    bool cc = area_gate(areaA, c.dinv, c.dthr) && w <= 0;
    cc_cand = cc ? 1u : 0u;
    cc_r16 = (cc && (sA & 15u) <= 1u) ? 1u : 0u;
    return c;
}

// Row value alpha scaled by 2 (the factor 2 of 2 l^2 m^2; the reference
// doubles the product instead, gpu_search_v42.cu:223-225).
__device__ __forceinline__ void scale2(const HotRec& h, AlphaHot& a) {
    a.re = 2.f * h.re;
    a.im = 2.f * h.im;
    uint32_t w[2] = {h.rre, h.rim};
    uint32_t out[2];
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        uint32_t ra = w[i] & kMaskA, rd = (w[i] >> kShiftD) & kMaskD;
        ra = 2 * ra >= kModA ? 2 * ra - kModA : 2 * ra;
        rd = 2 * rd >= kModD ? 2 * rd - kModD : 2 * rd;
        out[i] = ra | (rd << kShiftD);
    }
    a.ra = out[0] | (h.rre & kCentralBit);
    a.ia = out[1];
}

__device__ __forceinline__ void push_merged(const LaunchBuffers& buf, uint32_t l, uint32_t m, uint32_t row) {
    unsigned int idx = atomicAdd(buf.merged_count, 1u);
    if (idx < buf.merged_cap)
        buf.merged_queue[idx] = make_uint4(l, m, row, 0u);
    else
        atomicOr(buf.error_flags, 1u);
}

// Per-lane flush of the counters into a row's counters (64-bit atomics): for
// kernels whose threads each cover so much of a row that a warp's 32-bit sum
// could pass 2^32.
__device__ __forceinline__ void flush_acc_lanes(Acc& acc, RowCounts* rc) {
    if (acc.cand) atomicAdd(&rc->candidates, (unsigned long long)acc.cand);
    if (acc.r16) atomicAdd(&rc->r16, (unsigned long long)acc.r16);
    if (acc.prod) atomicAdd(&rc->products, (unsigned long long)acc.prod);
    if (acc.exact) atomicAdd(&rc->exact, (unsigned long long)acc.exact);
    if (acc.processed) atomicAdd(&rc->processed, (unsigned long long)acc.processed);
    if (acc.merged) atomicAdd(&rc->merged, (unsigned long long)acc.merged);
    acc = Acc{0, 0, 0, 0, 0, 0};
}

// Warp-level reduction of the per-thread counters into a row's counters;
// `shared_prime` also books them as work of the shared-prime kernels.
__device__ __forceinline__ void flush_acc(Acc& acc, RowCounts* rc, bool shared_prime = false) {
    uint32_t v[6] = {acc.cand, acc.r16, acc.prod, acc.exact, acc.processed, acc.merged};
#pragma unroll
    for (int i = 0; i < 6; ++i) v[i] = __reduce_add_sync(kFull, v[i]);
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

__device__ __forceinline__ uint64_t make_event(uint32_t v, uint32_t k, uint32_t flags) {
    return (uint64_t)v | ((uint64_t)k << 16) | ((uint64_t)flags << 40);
}

// Appends the lanes' events to the warp's queue (ballot-aggregated); returns
// true when the queue holds at least 32 events.  All 32 lanes must call it.
template <class Ev>
__device__ __forceinline__ bool queue_push(Ev* q, uint32_t& count, bool has, Ev ev) {
    const uint32_t mask = __ballot_sync(kFull, has);
    if (!mask) return false;
    const uint32_t lane = threadIdx.x & 31;
    if (has) q[count + __popc(mask & ((1u << lane) - 1u))] = ev;
    count += __popc(mask);
    return count >= 32;
}

// Processes the first `n` events of a warp queue, one per lane, then moves
// the rest to the front.  handle(ev, slots) returns the event's root requests
// left in `slots` (bits 0-3) and the orientations it found possible itself
// (bits 4-7); the warp then scans every request together, and hit(ev, tags)
// queues the exact hit test of each possible orientation of the lane's event.
// All 32 lanes must call it.
template <class Ev, class Handler, class HitFn>
__device__ __forceinline__ void drain(Ev* q, uint32_t& count, uint32_t n, RootReq* wreq, unsigned int* err,
                                      Handler handle, HitFn hit) {
    __syncwarp();
    const uint32_t lane = threadIdx.x & 31;
    Ev ev = 0;
    uint32_t info = 0;
    if (lane < n) {
        ev = q[lane];
        info = handle(ev, wreq + lane * kReqPerLane);
    }
    __syncwarp();
    uint32_t nreq = info & 15u;
    uint32_t passed = (info >> 4) & 15u;
    if (nreq > kReqPerLane) {
        atomicOr(err, kErrIndex);
        nreq = kReqPerLane;
    }
    __syncwarp();
    if (__any_sync(kFull, nreq != 0)) passed |= root_scan_requests(wreq, nreq, lane);
    if (passed) hit(ev, passed);
    __syncwarp();
    const uint32_t rest = count - n;
    if (lane < rest) q[lane] = q[n + lane];
    __syncwarp();
    count = rest;
}

// ------------------------------------------------------------ batched kernel

// Persistent batched kernel.  CTAs pull items (row l, m-range); the row's
// segment (scaled by 2) is staged in shared memory once per item.  Warps then
// work on their own: each claims 128 roots m at a time (4 per lane),
// classifies them, keeps the pair constants in its shared slice, and walks the
// valid m-side records in rounds of 32 - lane i of round r takes record
// 32r + i of the concatenated segments, found with a shuffle search over the
// lanes' prefix sums - running the row's values in lockstep.  Pairs of the
// dual kind (both orientations live) go in a second pass of their own.
// Events are drained 32 at a time; those left when a claim ends move to the
// warp's carry slots, and the item's end drains the rest.
struct BatchedShared {
    uint32_t item;
    uint32_t next_m;
};

constexpr uint32_t kRootsPerLane = 4;  // a warp claims 128 roots at a time
constexpr uint32_t kChunk = 32 * kRootsPerLane;
constexpr uint32_t kCarry = 32;        // pair-constant slots of events left over from earlier claims

__device__ __forceinline__ uint64_t batched_event_word(uint32_t j, uint32_t slot, uint32_t k, uint32_t flags) {
    return (uint64_t)j | ((uint64_t)slot << 32) | ((uint64_t)k << 40) | ((uint64_t)flags << 53);
}

// One pass over the records of the warp's 128 roots (the dual or the
// non-dual ones): lane i holds roots slot = 32u + i (u < 4) with cnt[u]
// records starting at s0[u].  Record r of the pass (lane-major order, so
// consecutive records are consecutive in memory) is found by a binary search
// over the lanes' inclusive prefix sums, then within the owner lane.
template <bool DUAL, bool FLUSH = false>
__device__ __forceinline__ void batched_pass(const AlphaHot* s_alpha, uint32_t na,
                                             const PairCtx* wctx, const uint32_t (&cnt)[kRootsPerLane],
                                             const uint32_t (&s0)[kRootsPerLane], uint32_t lane,
                                             const DeviceCache& cache, const uint8_t* s_tab, uint32_t a0, uint64_t l,
                                             uint32_t row, const LaunchBuffers& buf, uint64_t* q, uint32_t& qn,
                                             RootReq* wreq, Acc& acc) {
    uint32_t mine = 0;
#pragma unroll
    for (uint32_t u = 0; u < kRootsPerLane; ++u) mine += cnt[u];
    uint32_t incl = mine;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t t = __shfl_up_sync(kFull, incl, d);
        if (lane >= (uint32_t)d) incl += t;
    }
    const uint32_t total = __shfl_sync(kFull, incl, 31);
    if (!FLUSH && total == 0) return;
    const uint32_t excl = incl - mine;
    auto handle = [&](uint64_t ev, RootReq* slots) -> uint32_t {
        const uint32_t j = (uint32_t)ev, slot = (uint32_t)(ev >> 32) & 0xFFu, k = (uint32_t)(ev >> 40) & 0x1FFFu;
        if (!index_ok(k, na, buf.error_flags) || !index_ok(slot, kChunk + kCarry, buf.error_flags)) return 0u;
        const uint2 r = cached_event((uint32_t)(ev >> 53), s_alpha[k], cache.hot[j], wctx[slot], a0 + k, j,
                                     (uint32_t)l, row, s_tab, kTabD2, (uint32_t)cache.limit, &buf, slots);
        acc.cand += r.x & 0xFFFFu;
        acc.r16 += r.y;
        return r.x >> 16;
    };
    auto hit = [&](uint64_t ev, uint32_t tags) {
        const uint32_t j = (uint32_t)ev, slot = (uint32_t)(ev >> 32) & 0xFFu, k = (uint32_t)(ev >> 40) & 0x1FFFu;
        push_hits(&buf, tags, a0 + k, j, (uint32_t)l, pair_m(wctx[slot]), row, false);
    };
    if constexpr (FLUSH) {
        // the item's last events (the row values are replaced next)
        while (qn) drain(q, qn, qn < 32 ? qn : 32, wreq, buf.error_flags, handle, hit);
        return;
    } else {
        for (uint32_t base = 0; base < total; base += 32) {
            const uint32_t r = base + lane;
            uint32_t owner = 0;
#pragma unroll
            for (uint32_t step = 16; step >= 1; step >>= 1) {
                const uint32_t v = __shfl_sync(kFull, incl, owner + step - 1);
                if (v <= r) owner += step;
            }
            owner &= 31u;
            uint32_t off = r - __shfl_sync(kFull, excl, owner);
            uint32_t slot = owner, j = 0;
#pragma unroll
            for (uint32_t u = 0; u < kRootsPerLane; ++u) {
                const uint32_t cu = __shfl_sync(kFull, cnt[u], owner);
                const uint32_t su = __shfl_sync(kFull, s0[u], owner);
                if (off < cu && slot == owner) {
                    slot = 32 * u + owner + 1024u;  // mark found
                    j = su + off;
                }
                if (slot == owner) off -= cu;
            }
            slot = (slot - 1024u) & 127u;
            const bool live = r < total;
            const PairCtx c = wctx[slot];
            const HotRec b = live ? cache.hot[j] : HotRec{0.f, 0.f, kCentralBit, 0u};
            const bool cb = (b.rre & kCentralBit) != 0;
            for (uint32_t k = 0; k < na; ++k) {
                const AlphaHot a = s_alpha[k];
                uint32_t flags = 0;
                if (live) flags = eval_fast<DUAL ? 1 : 0, true, true>(a, b.re, b.im, b.rre, b.rim, cb, c, s_tab, acc);
                if (queue_push(q, qn, flags != 0, batched_event_word(j, slot, k, flags)))
                    drain(q, qn, 32, wreq, buf.error_flags, handle, hit);
            }
        }
    }
}

// Events still queued when a warp's claim ends keep their pair constants in
// the warp's carry slots (kChunk + lane), so that they wait for the drains of
// the next claim, whose constants replace slots 0 .. kChunk - 1.  Every read
// precedes every write: a carried event may be carried again.
__device__ __forceinline__ void carry_events(uint64_t* q, uint32_t qn, PairCtx* wctx, uint32_t lane) {
    __syncwarp();
    uint64_t ev = 0;
    PairCtx c;
    if (lane < qn) {
        ev = q[lane];
        c = wctx[(uint32_t)(ev >> 32) & 0xFFu];
    }
    __syncwarp();
    if (lane < qn) {
        wctx[kChunk + lane] = c;
        q[lane] = (ev & ~(0xFFull << 32)) | ((uint64_t)(kChunk + lane) << 32);
    }
    __syncwarp();
}

template <int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) batched_kernel(const DeviceCache cache, const WorkItem* __restrict__ items,
                                                           uint32_t n_items, uint32_t alpha_cap,
                                                           const LaunchBuffers buf) {
    constexpr uint32_t kWarps = NT / 32;
    extern __shared__ __align__(16) unsigned char smem[];
    AlphaHot* s_alpha = reinterpret_cast<AlphaHot*>(smem);
    PairCtx* s_wctx = reinterpret_cast<PairCtx*>(s_alpha + alpha_cap);
    uint64_t* s_queue = reinterpret_cast<uint64_t*>(s_wctx + kWarps * (kChunk + kCarry));
    RootReq* s_req = reinterpret_cast<RootReq*>(s_queue + kWarps * kQueue);
    uint8_t* s_tab = reinterpret_cast<uint8_t*>(s_req + kWarps * 32 * kReqPerLane);
    __shared__ BatchedShared S;

    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid / 32;
    uint64_t* q = s_queue + warp * kQueue;
    PairCtx* wctx = s_wctx + warp * (kChunk + kCarry);
    RootReq* wreq = s_req + warp * 32 * kReqPerLane;
    uint32_t qn = 0;
    for (uint32_t i = tid; i < kTable2Bytes; i += NT) s_tab[i] = buf.tables[kTableBytes + i];
    Acc acc{0, 0, 0, 0, 0, 0};
    for (;;) {
        __syncthreads();
        if (tid == 0) {
            S.item = atomicAdd(buf.next_item, 1u);
            S.next_m = 0;
        }
        __syncthreads();
        const uint32_t it = S.item;
        if (it >= n_items) break;
        const WorkItem w = items[it];
        const RowInfo& R = buf.row_info[w.row];
        const uint32_t a0 = R.seg, na = R.free_l + 1;
        for (uint32_t i = tid; i < na; i += NT) scale2(cache.hot[a0 + i], s_alpha[i]);
        __syncthreads();
        const uint32_t nm = w.m1 - w.m0;
        for (;;) {
            uint32_t c0 = 0;
            if (lane == 0) c0 = atomicAdd(&S.next_m, kChunk);
            c0 = __shfl_sync(kFull, c0, 0);
            if (c0 >= nm) break;
            uint32_t cnt_single[kRootsPerLane], cnt_dual[kRootsPerLane], s0[kRootsPerLane];
            bool any_dual = false;
#pragma unroll
            for (uint32_t u = 0; u < kRootsPerLane; ++u) {
                cnt_single[u] = cnt_dual[u] = s0[u] = 0;
                if (c0 + 32 * u + lane >= nm) continue;
                const uint32_t m = w.m0 + c0 + 32 * u + lane;
                const uint32_t seg0 = cache.seg_off[m], seg1 = cache.seg_off[m + 1];
                const uint32_t kind = classify(R, m, seg1 - seg0 - 1);
                if (kind == kCached) {
                    uint32_t cc_c, cc_r;
                    const PairCtx c = make_ctx(R, m, cc_c, cc_r);
                    wctx[32 * u + lane] = c;
                    s0[u] = seg0;
                    if (pair_dual(c)) {
                        cnt_dual[u] = seg1 - seg0;
                        any_dual = true;
                    } else {
                        cnt_single[u] = seg1 - seg0;
                    }
                    acc.processed += 1;
                    acc.prod += pair_products(na, seg1 - seg0);
                    acc.cand += cc_c;
                    acc.r16 += cc_r;
                } else if (kind == kMerged) {
                    acc.processed += 1;
                    acc.merged += 1;
                    push_merged(buf, w.l, m, w.row);
                }
            }
            __syncwarp();
            batched_pass<false>(s_alpha, na, wctx, cnt_single, s0, lane, cache, s_tab, a0, w.l, w.row, buf,
                                q, qn, wreq, acc);
            if (__any_sync(kFull, any_dual))
                batched_pass<true>(s_alpha, na, wctx, cnt_dual, s0, lane, cache, s_tab, a0, w.l, w.row, buf, q,
                                   qn, wreq, acc);
            carry_events(q, qn, wctx, lane);
        }
        {
            const uint32_t none[kRootsPerLane] = {};
            batched_pass<false, true>(s_alpha, na, wctx, none, none, lane, cache, s_tab, a0, w.l, w.row, buf, q, qn,
                                      wreq, acc);
        }
        flush_acc(acc, &buf.rows[w.row]);
    }
}

// -------------------------------------------------------------- plain kernel

// One block per (row, slice) and one thread per pair, as the reference
// (gpu_search_v42.cu:298-304); events are handled by the lane that raised them.
__global__ void __launch_bounds__(kPlainThreads, 4) plain_kernel(const DeviceCache cache, uint32_t alpha_cap,
                                                                 const LaunchBuffers buf) {
    extern __shared__ __align__(16) unsigned char smem[];
    AlphaHot* s_alpha = reinterpret_cast<AlphaHot*>(smem);
    uint8_t* s_tab = reinterpret_cast<uint8_t*>(s_alpha + alpha_cap);
    const uint32_t row = blockIdx.x / kSlices, slice = blockIdx.x % kSlices;
    const RowInfo& R = buf.row_info[row];
    const uint64_t l = R.l;
    for (uint32_t i = threadIdx.x; i < kTableBytes; i += kPlainThreads) s_tab[i] = buf.tables[i];
    const uint32_t a0 = R.seg, na = R.free_l + 1;
    for (uint32_t i = threadIdx.x; i < na; i += kPlainThreads) scale2(cache.hot[a0 + i], s_alpha[i]);
    __syncthreads();
    Acc acc{0, 0, 0, 0, 0, 0};
    const uint64_t n = cache.limit;
    for (uint64_t m = l + slice * kPlainThreads + threadIdx.x; m <= n; m += kSlices * kPlainThreads) {
        const uint32_t s0 = cache.seg_off[m], s1 = cache.seg_off[m + 1];
        const uint32_t kind = classify(R, (uint32_t)m, s1 - s0 - 1);
        if (kind == kSkip) continue;
        acc.processed += 1;
        if (kind == kMerged) {
            acc.merged += 1;
            push_merged(buf, (uint32_t)l, (uint32_t)m, row);
            continue;
        }
        uint32_t cc_c, cc_r;
        const PairCtx c = make_ctx(R, m, cc_c, cc_r);
        acc.prod += pair_products(na, s1 - s0);
        acc.cand += cc_c;
        acc.r16 += cc_r;
        for (uint32_t j = s0; j < s1; ++j) {
            const HotRec b = cache.hot[j];
            const bool cb = (b.rre & kCentralBit) != 0;
            for (uint32_t k = 0; k < na; ++k) {
                const uint32_t flags =
                    pair_dual(c) ? eval_fast<1>(s_alpha[k], b.re, b.im, b.rre, b.rim, cb, c, s_tab, acc)
                                 : eval_fast<0>(s_alpha[k], b.re, b.im, b.rre, b.rim, cb, c, s_tab, acc);
                if (flags)
                    add_event(acc, cached_event(flags, s_alpha[k], b, c, a0 + k, j, (uint32_t)l, row, s_tab, kTabD,
                                                (uint32_t)n, &buf));
            }
        }
    }
    flush_acc_lanes(acc, &buf.rows[row]);
}

// ------------------------------------------------------------- merged kernels

// Terms of a pair that shares split primes: merged exponents e = a + b
// (gpu_search_v42.cu:318-338), split in two groups whose products form the
// two lists; each list is the group's free set plus its central value.
struct Group {
    uint32_t count;
    uint32_t e[kMaxTerms];
    uint32_t base[kMaxTerms];   // index of the term's first value in the prime-power table
    uint32_t block[kMaxTerms];  // number of free vectors whose first non-central index is i
    uint32_t suffix[kMaxTerms]; // prod_{j>i} (4 e_j + 1)
    uint32_t free_count;
    i128 scale;                 // real factor folded into every value of the group
    float scale_f;              // the same as float and packed residues
    uint32_t scale_res;
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
    for (uint32_t j = 0; j < i; ++j) xr *= cache.pp_exact[2 * (g.base[j] + 2 * g.e[j])];
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

// Complex product of packed residues (fields A and D).
__device__ __forceinline__ void res_mul(uint32_t ar, uint32_t ai, uint32_t br, uint32_t bi, uint32_t& xr,
                                        uint32_t& xi) {
    uint32_t outr = 0, outi = 0;
#pragma unroll
    for (int f = 0; f < 2; ++f) {
        const uint32_t shift = f == 0 ? 0u : kShiftD;
        const uint32_t mask = f == 0 ? kMaskA : kMaskD;
        const uint32_t M = f == 0 ? kModA : kModD;
        const uint32_t a0 = (ar >> shift) & mask, a1 = (ai >> shift) & mask;
        const uint32_t b0 = (br >> shift) & mask, b1 = (bi >> shift) & mask;
        outr |= ((a0 * b0 + M * M - a1 * b1) % M) << shift;
        outi |= ((a0 * b1 + a1 * b0) % M) << shift;
    }
    xr = outr;
    xi = outi;
}

// One event of a shared-prime pair: list entries ka (alpha side) and kb.
__device__ __noinline__ uint2 merged_event(uint32_t flags, AlphaHot a, AlphaHot bh, PairCtx c, uint32_t ka,
                                              uint32_t kb, uint32_t l, uint32_t row, const uint8_t* tab,
                                              uint32_t tabd_ofs, uint32_t limit, const LaunchBuffers* buf,
                                              RootReq* slots = nullptr) {
    const HotRec b{bh.re, bh.im, bh.ra, bh.ia};
    const EventSink sink{buf, ka, kb, l, pair_m(c), row, 1u, tab_d_bits(tab, tabd_ofs)};
    const uint4 r = process_event(flags, a, b, c, limit, tab, sink, slots);
    return make_uint2(r.x | (r.z << 16) | (r.w << 20), r.y);
}

// The merged terms of pair (l, m): the split primes of l and of m, with the
// exponents added where both have the prime, and the term order that splits
// them into two groups (decreasing exponent, stable); fixed gets
// 2 fixed(l) fixed(m), the real factor of every value.  Returns the count.
__device__ uint32_t merged_terms(const DeviceCache& cache, const RowInfo& R, uint64_t m, uint32_t (&tp)[kMaxTerms],
                                 uint32_t (&te)[kMaxTerms], uint32_t (&order)[kMaxTerms], i128& fixed) {
    uint32_t mp[9], me[9], nm = 0;
    fixed = (i128)2 * (i128)R.fixed;
    uint32_t x = (uint32_t)m;  // m <= 3e7: 32-bit divisions
    while (x > 1) {
        uint32_t p = cache.spf[x], a = 0;
        do {
            x /= p;
            ++a;
        } while (x % p == 0);
        if ((p & 3u) == 1u) {
            mp[nm] = p;
            me[nm++] = a;
        } else {
            for (uint32_t t = 0; t < 2 * a; ++t) fixed *= p;
        }
    }
    uint32_t count = 0;
    uint32_t i = 0, j = 0;
    while (i < R.nsplit || j < nm) {
        if (j == nm || (i < R.nsplit && R.sp[i] < mp[j])) {
            tp[count] = R.sp[i];
            te[count++] = R.se[i++];
        } else if (i == R.nsplit || mp[j] < R.sp[i]) {
            tp[count] = mp[j];
            te[count++] = me[j++];
        } else {
            tp[count] = R.sp[i];
            te[count++] = R.se[i++] + me[j++];
        }
    }
    for (uint32_t t = 0; t < count; ++t) order[t] = t;
    for (uint32_t a = 1; a < count; ++a)
        for (uint32_t b = a; b > 0 && te[order[b]] > te[order[b - 1]]; --b) {
            uint32_t tmp = order[b];
            order[b] = order[b - 1];
            order[b - 1] = tmp;
        }
    return count;
}

// Splits the merged terms of (l, m) into two groups (largest terms first,
// each to the group with the smaller product of sizes), with the block and
// suffix tables of the exact path's decode.  ok = 1: fits list_cap; 2: too
// big for it; 0: an exponent beyond the prime-power table.
__device__ void merged_setup(const DeviceCache& cache, const RowInfo& R, uint4 q, MergedShared& S,
                             uint32_t list_cap) {
    S.l = q.x;
    S.m = q.y;
    S.row = q.z;
    S.ok = 1;
    uint32_t tp[kMaxTerms], te[kMaxTerms], order[kMaxTerms];
    i128 fixed;
    const uint32_t count = merged_terms(cache, R, q.y, tp, te, order, fixed);
    uint64_t wsz[2] = {1, 1};
    S.g[0].count = S.g[1].count = 0;
    for (uint32_t t = 0; t < count; ++t) {
        uint32_t idx = order[t];
        int side = wsz[0] <= wsz[1] ? 0 : 1;
        Group& g = S.g[side];
        g.e[g.count] = te[idx];
        g.base[g.count] = cache.pp_base[tp[idx]] + pp_exponent_offset(te[idx]);
        ++g.count;
        wsz[side] *= 4 * te[idx] + 1;
        if (te[idx] > cache.max_exponent) S.ok = 0;
    }
    group_finish(S.g[0]);
    group_finish(S.g[1]);
    S.g[0].scale = fixed;
    S.g[1].scale = 1;
    S.g[0].scale_f = i128_to_float(fixed);
    S.g[0].scale_res = pack_residues(fixed);
    S.g[1].scale_f = 1.f;
    S.g[1].scale_res = kResOne;
    if (S.ok == 1 && S.g[0].free_count + S.g[1].free_count + 2 > list_cap) S.ok = 2;
}

// Compact description of a shared-prime pair for the warp kernel: its two
// term groups (prime-power table index and exponent of each term), the list
// sizes, the float/residue form of the group-0 scale 2 fixed(l) fixed(m), and
// the pair constants.  state: 0 none, 1 fits a warp slice, 2 big, 3 unusable.
constexpr uint32_t kDescTerms = 10;  // l, m <= 3e7 have at most 5 split primes each
struct __align__(16) PairDesc {
    PairCtx ctx;
    uint32_t base[2][kDescTerms];
    uint32_t free_count[2];
    float scale_f;
    uint32_t scale_res;
    uint32_t l, m, row;
    uint8_t count[2];
    uint8_t e[2][kDescTerms];
    uint8_t state;
    uint8_t cc;  // bit 0: the all-central product is a candidate; bit 1: it passes mod 16
};
static_assert(sizeof(PairDesc) <= kBigEntryWords * 16 && sizeof(PairDesc) % 16 == 0,
              "a descriptor fits one big-queue entry");

// Error bound of a shared-prime pair's float products, relative to |z|, with
// u = 2^-24.  A float complex product x v (with or without fused multiply-
// adds) is within 2 sqrt(2) u |x| |v| of the product of its float inputs, as
// |x_re v_re| + |x_im v_im| <= |x| |v| for each component; an input with
// relative error e_x adds e_x |x| |v|.  A list value is the group's scale
// (within 3 u: an i128 rounded to float) times one prime-power value per term
// of the group (each within u, correctly rounded), so it is within
// 3 u + 3.83 k u for k terms; the filter loop's product alpha beta adds the
// two values' errors and 2.83 u.  For K = k0 + k1 terms that is at most
// (5.83 + 3.83 K) u; the bound used, (12 + 8 K) u, keeps a factor 2 (and is
// never looser than the 2^-16 once used for every pair, as K <= 20).  Every
// window decision and root window of the pair is taken against it.
__device__ __forceinline__ float shared_prime_eps_scale(uint32_t K) { return (float)(12 + 8 * K) * 0x1p-24f; }

// The descriptor of a shared-prime pair: the groups of merged_setup written
// straight into it (a group of value count w has (w - 1) / 2 free values,
// the sum of its blocks), without the block and suffix tables that only the
// exact path's decode needs.
__device__ void pair_desc_setup(const DeviceCache& cache, const RowInfo& R, uint4 q, PairDesc& D, uint32_t cap) {
    uint32_t tp[kMaxTerms], te[kMaxTerms], order[kMaxTerms];
    i128 fixed;
    const uint32_t count = merged_terms(cache, R, q.y, tp, te, order, fixed);
    D.l = q.x;
    D.m = q.y;
    D.row = q.z;
    uint64_t wsz[2] = {1, 1};
    uint32_t n[2] = {0, 0};
    bool ok = true;
    for (uint32_t t = 0; t < count; ++t) {
        const uint32_t idx = order[t];
        const int side = wsz[0] <= wsz[1] ? 0 : 1;
        if (n[side] < kDescTerms) {
            D.base[side][n[side]] = cache.pp_base[tp[idx]] + pp_exponent_offset(te[idx]);
            D.e[side][n[side]] = (uint8_t)te[idx];
        } else {
            ok = false;  // more terms than a descriptor holds
        }
        ++n[side];
        wsz[side] *= 4 * te[idx] + 1;
        if (te[idx] > cache.max_exponent) ok = false;
    }
    const uint32_t free0 = (uint32_t)((wsz[0] - 1) / 2), free1 = (uint32_t)((wsz[1] - 1) / 2);
    D.state = !ok ? 3 : (free0 + free1 + 2 > cap ? 2 : 1);
    if (D.state == 3) return;
    D.count[0] = (uint8_t)n[0];
    D.count[1] = (uint8_t)n[1];
    D.free_count[0] = free0;
    D.free_count[1] = free1;
    D.scale_f = i128_to_float(fixed);
    D.scale_res = pack_residues(fixed);
    uint32_t cc_c, cc_r;
    D.ctx = make_ctx(R, q.y, cc_c, cc_r, shared_prime_eps_scale(count));
    D.cc = (uint8_t)(cc_c | (cc_r << 1));
}

// Entry k of side g of a described pair, in float and residues (the decode
// of group_value, with the block sizes recomputed from the exponents).
__device__ void desc_value_hot(const DeviceCache& cache, const PairDesc& D, int g, uint32_t k, AlphaHot& out) {
    const uint32_t count = D.count[g];
    float xr = g == 0 ? D.scale_f : 1.f, xi = 0.f;
    uint32_t rr = g == 0 ? D.scale_res : kResOne, ri = 0u;
    auto mul = [&](const HotRec& v) {
        const float nr = xr * v.re - xi * v.im, ni = xr * v.im + xi * v.re;
        uint32_t yr, yi;
        res_mul(rr, ri, v.rre & kResMask, v.rim, yr, yi);
        xr = nr;
        xi = ni;
        rr = yr;
        ri = yi;
    };
    const bool central = k >= D.free_count[g];
    if (count <= 3) {
        // sides of up to three terms (every side of a warp-sized pair),
        // decoded directly into one digit per term (s_j = 4 e_j + 1, the
        // central digit 2 e_j).  One term: entry k is scale v_0[k], k = 2 e_0
        // being the central value.  Two terms: block 0 holds
        // scale v_0[k / s_1] v_1[k mod s_1] for k < 2 e_0 s_1, then
        // scale v_0[2 e_0] v_1[k - 2 e_0 s_1] up to the central value.  Three
        // terms: the same with the last two digits in mixed radix (s_1, s_2)
        // in block 0, then block 1 (digits 2 e_0, r, d_2), then the last
        // term's digits after 2 e_0, 2 e_1.
        if (count == 1) {
            mul(cache.pp_hot[D.base[g][0] + k]);
        } else if (count == 2) {
            const uint32_t two_e0 = 2u * D.e[g][0];
            const uint32_t s1 = 4u * D.e[g][1] + 1u, block0 = two_e0 * s1;
            const uint32_t r = k < block0 ? k / s1 : two_e0;
            mul(cache.pp_hot[D.base[g][0] + r]);
            mul(cache.pp_hot[D.base[g][1] + (k < block0 ? k - r * s1 : k - block0)]);
        } else if (count == 3) {
            const uint32_t two_e0 = 2u * D.e[g][0], two_e1 = 2u * D.e[g][1];
            const uint32_t s1 = 2u * two_e1 + 1u, s2 = 4u * D.e[g][2] + 1u;
            const uint32_t block0 = two_e0 * s1 * s2, block1 = two_e1 * s2;
            uint32_t d0 = two_e0, d1 = two_e1, d2;
            if (k < block0) {
                const uint32_t q = k / s2;
                d2 = k - q * s2;
                d0 = q / s1;
                d1 = q - d0 * s1;
            } else if (k < block0 + block1) {
                const uint32_t k1 = k - block0;
                d1 = k1 / s2;
                d2 = k1 - d1 * s2;
            } else {
                d2 = k - block0 - block1;
            }
            mul(cache.pp_hot[D.base[g][0] + d0]);
            mul(cache.pp_hot[D.base[g][1] + d1]);
            mul(cache.pp_hot[D.base[g][2] + d2]);
        }
        out.re = xr;
        out.im = xi;
        out.ra = rr | (central ? kCentralBit : 0u);
        out.ia = ri;
        return;
    }
    uint32_t suffix[kDescTerms];
    for (int i = (int)count - 1, acc = 1; i >= 0; --i) {
        suffix[i] = (uint32_t)acc;
        acc *= 4 * (int)D.e[g][i] + 1;
    }
    uint32_t i = 0;
    if (!central) {
        while (k >= 2u * D.e[g][i] * suffix[i]) {
            k -= 2u * D.e[g][i] * suffix[i];
            ++i;
        }
    } else {
        i = count;
    }
    for (uint32_t j = 0; j < i; ++j) mul(cache.pp_hot[D.base[g][j] + 2u * D.e[g][j]]);
    if (i < count) {
        const uint32_t r = k / suffix[i];
        uint32_t rem = k - r * suffix[i];
        mul(cache.pp_hot[D.base[g][i] + r]);
        for (uint32_t j = i + 1; j < count; ++j) {
            const uint32_t below = suffix[j];
            const uint32_t digit = rem / below;
            rem -= digit * below;
            mul(cache.pp_hot[D.base[g][j] + digit]);
        }
    }
    out.re = xr;
    out.im = xi;
    out.ra = rr | (central ? kCentralBit : 0u);
    out.ia = ri;
}

// Shared-prime pair set-up, one thread per pair of one chunk of the queue
// (entries chunk0 .. chunk0 + desc_chunk - 1): factors m, splits the pair's
// terms and computes its constants into the pair's descriptor slot.  Pairs
// whose lists exceed a warp's slice also go to the big-pair queue (one CTA
// per pair).  Kept apart from the warp kernel, whose filter loop then has the
// instruction cache to itself.
__global__ void __launch_bounds__(128) merged_setup_kernel(const DeviceCache cache, const LaunchBuffers buf,
                                                         uint32_t chunk0) {
    const uint32_t count = min(*buf.merged_count, buf.merged_cap);
    if (chunk0 >= count) return;
    const uint32_t n = min(count - chunk0, buf.desc_chunk);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint4 e = buf.merged_queue[chunk0 + i];
        PairDesc D;
        pair_desc_setup(cache, buf.row_info[e.z], e, D, kWarpListCap);
        const uint4* src = reinterpret_cast<const uint4*>(&D);
        if (D.state == 2) {
            unsigned int idx = atomicAdd(buf.big_count, 1u);
            if (idx < buf.big_cap) {
                uint4* dst = buf.big_queue + (size_t)idx * kBigEntryWords;
                for (uint32_t w = 0; w < sizeof(PairDesc) / 16; ++w) dst[w] = src[w];
            } else {
                atomicOr(buf.error_flags, 8u);  // the big-pair queue is full: the host grows it and reruns
            }
        } else if (D.state == 3) {
            atomicOr(buf.error_flags, 2u);
        }
        uint4* dst = buf.pair_desc + (size_t)i * kBigEntryWords;
        for (uint32_t w = 0; w < sizeof(PairDesc) / 16; ++w) dst[w] = src[w];
    }
}

// Shared-prime pairs of one chunk, a segment of pairs per warp at a time.  A
// warp claims blocks of 32 consecutive descriptors from the chunk's cursor
// (pair sizes vary widely) and stages up to kSegSlots of them in its shared
// slice, copying the next group's descriptors with asynchronous copies while
// the current group runs; consecutive staged pairs whose lists fit the
// warp's list arena form a segment.  The segment's lists are built side by side (float and residue
// products of the prime-power values), and all its (alpha, beta)
// combinations - the pairs' combination spaces laid end to end - run in
// lockstep rounds of 32: each lane steps from pair to pair, so rounds stay
// full across pair boundaries, and the events of every pair of the segment
// share the warp's queue (drained 32 at a time, one partial drain per
// segment).  Candidates and mod-16 survivors gather per pair in shared
// memory; products per pair are counted from the list sizes,
// 2 na nb - na - nb + 1 (one product per combination with a central value,
// none for the central pair, which is the analytic all-central product, two
// otherwise); each pair's counts go to its row once per segment.
constexpr uint32_t kPairWarps = 8;
constexpr uint32_t kSegSlots = 8;   // staged pairs (descriptors) per warp
constexpr uint32_t kSegList = 256;  // list entries of one segment (a pair has at most kWarpListCap)
static_assert(kSegList >= kWarpListCap, "every warp-sized pair fits a segment alone");

struct SegSlot {
    uint32_t size;       // na * nb combinations (0: not a warp-sized pair)
    uint32_t loff;       // first list entry of the pair's side 0 in the arena
    uint32_t cand, r16;  // counts gathered from the lanes and the event handlers
    uint32_t nab;        // na | nb << 16
    uint32_t step;       // ceil(2^16 / nb) | (32 / nb) << 17 | (32 mod nb) << 23
};

// A lane entering a pair of the segment does so at an offset below 32 (it
// stepped at most 32 past the previous pair's end), so off / nb is taken as
// off * ceil(2^16 / nb) >> 16, exact for off < 32 and nb < 2^8: the error term
// off * (ceil(2^16 / nb) - 2^16 / nb) / 2^16 stays below 32 / 2^16, less than the
// gap 1/nb between off / nb and the next integer.
__device__ __forceinline__ uint32_t seg_step(uint32_t nb) {
    return (65536u + nb - 1) / nb | (32u / nb) << 17 | (32u % nb) << 23;
}

// Event of a segment: beta index, alpha index, slot, flags (8 bits each).
__device__ __forceinline__ uint32_t seg_event(uint32_t kb, uint32_t ka, uint32_t k, uint32_t flags) {
    return kb | (ka << 8) | (k << 16) | (flags << 24);
}

__global__ void __launch_bounds__(kPairWarps * 32, 2) merged_kernel(const DeviceCache cache, const LaunchBuffers buf,
                                                                  uint32_t chunk0) {
    constexpr uint32_t kDescWords = sizeof(PairDesc) / 16;
    __shared__ __align__(16) PairDesc s_desc[kPairWarps][kSegSlots];
    __shared__ __align__(16) AlphaHot s_list[kPairWarps][kSegList];
    __shared__ uint32_t s_queue[kPairWarps][kQueue];
    __shared__ SegSlot s_slot[kPairWarps][kSegSlots];
    __shared__ __align__(16) uint4 s_raw[kPairWarps][kSegSlots * kDescWords];  // the next group, in flight
    // dynamic: root requests, then the wide tables
    extern __shared__ __align__(16) unsigned char s_dyn[];
    RootReq* s_req = reinterpret_cast<RootReq*>(s_dyn);
    uint8_t* s_tab = reinterpret_cast<uint8_t*>(s_req + kPairWarps * 32 * kReqPerLane);
    const uint32_t count = min(*buf.merged_count, buf.merged_cap);
    if (chunk0 >= count) return;
    const uint32_t n = min(count - chunk0, buf.desc_chunk);
    for (uint32_t i = threadIdx.x; i < kTable2Bytes; i += kPairWarps * 32) s_tab[i] = buf.tables[kTableBytes + i];
    __syncthreads();
    const uint32_t warp = threadIdx.x / 32, lane = threadIdx.x & 31;
    PairDesc* desc = s_desc[warp];
    AlphaHot* list = s_list[warp];
    uint32_t* q = s_queue[warp];
    SegSlot* slot = s_slot[warp];
    RootReq* wreq = s_req + warp * 32 * kReqPerLane;
    const uint32_t limit = (uint32_t)cache.limit;
    uint32_t qn = 0;
    // groups of up to kSegSlots descriptors, from blocks of 32 taken from the
    // cursor; the next group's descriptors are copied into s_raw while the
    // current one runs (asynchronous copies, one 16-byte word per lane)
    uint4* raw = s_raw[warp];
    uint32_t cb0 = 0, coff = 0;
    auto claim = [&]() {
        uint32_t b = 0;
        if (lane == 0) b = atomicAdd(buf.desc_next, 32u);
        cb0 = __shfl_sync(kFull, b, 0);
        coff = 0;
    };
    auto take = [&](uint32_t& g0, uint32_t& gn) -> bool {
        if (cb0 >= n) return false;
        const uint32_t b1 = min(cb0 + 32, n);
        g0 = cb0 + coff;
        gn = min(kSegSlots, b1 - g0);
        coff += kSegSlots;
        if (cb0 + coff >= b1) claim();
        return true;
    };
    auto prefetch = [&](uint32_t g0, uint32_t gn) {
        for (uint32_t w = lane; w < gn * kDescWords; w += 32) {
            const uint4* src = buf.pair_desc + (size_t)(g0 + w / kDescWords) * kBigEntryWords + w % kDescWords;
            const uint32_t dst = (uint32_t)__cvta_generic_to_shared(raw + w);
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    claim();
    uint32_t g0 = 0, ns = 0;
    bool have = take(g0, ns);
    if (have) prefetch(g0, ns);
    while (have) {
        asm volatile("cp.async.wait_all;" ::: "memory");
        __syncwarp();
        // staged with the dual pairs (both orientations live) first, so
        // that a segment's rounds mix dual and single-orientation lanes
        // at one boundary at most (word 2 of a descriptor holds ctx.m,
        // whose bit 31 is the dual flag)
        const bool dual_i = lane < ns && (raw[lane * kDescWords + 2].w >> 31) != 0;
        const uint32_t dmask = __ballot_sync(kFull, dual_i), vmask = (1u << ns) - 1u;
        auto dest = [&](uint32_t i) {
            const uint32_t below = (1u << i) - 1u;
            return ((dmask >> i) & 1u) ? (uint32_t)__popc(dmask & below)
                                       : (uint32_t)(__popc(dmask) + __popc(~dmask & vmask & below));
        };
        for (uint32_t w = lane; w < ns * kDescWords; w += 32)
            reinterpret_cast<uint4*>(desc)[dest(w / kDescWords) * kDescWords + w % kDescWords] = raw[w];
        __syncwarp();
        uint32_t n0 = 0, nn = 0;
        const bool more = take(n0, nn);
        if (more) prefetch(n0, nn);
        for (uint32_t first = 0; first < ns;) {
            // the segment: staged pairs first .. last - 1 whose lists fit the arena
            uint32_t entries = 0, combos = 0;
            if (lane >= first && lane < ns && desc[lane].state == 1) {
                const uint32_t na = desc[lane].free_count[0] + 1, nb = desc[lane].free_count[1] + 1;
                entries = na + nb;
                combos = na * nb;
            }
            uint32_t incl = entries;
#pragma unroll
            for (int d = 1; d < (int)kSegSlots; d <<= 1) {
                const uint32_t t = __shfl_up_sync(kFull, incl, d);
                if (lane >= (uint32_t)d) incl += t;
            }
            const uint32_t fits = __ballot_sync(kFull, lane >= first && lane < ns && incl <= kSegList);
            const uint32_t last = first + __popc(fits);
            uint32_t total = combos;
            if (lane >= first && lane < last) {
                slot[lane].size = combos;
                slot[lane].loff = incl - entries;
                slot[lane].cand = 0;
                slot[lane].r16 = 0;
                if (combos) {
                    const uint32_t na = desc[lane].free_count[0] + 1, nb = desc[lane].free_count[1] + 1;
                    slot[lane].nab = na | nb << 16;
                    slot[lane].step = seg_step(nb);
                }
            } else {
                total = 0;
            }
            const uint32_t built = __shfl_sync(kFull, incl, last - 1);
            total = __reduce_add_sync(kFull, total);
            __syncwarp();
            // lists of the segment, entry e of the arena by lane e mod 32
            for (uint32_t e = lane; e < built; e += 32) {
                uint32_t k = first;
                while (k + 1 < last && e >= slot[k + 1].loff) ++k;
                const uint32_t idx = e - slot[k].loff, na = desc[k].free_count[0] + 1;
                desc_value_hot(cache, desc[k], idx < na ? 0 : 1, idx < na ? idx : idx - na, list[e]);
            }
            __syncwarp();
            auto handle = [&](uint32_t ev, RootReq* slots) -> uint32_t {
                const uint32_t kb = ev & 0xFFu, ka = (ev >> 8) & 0xFFu, k = (ev >> 16) & 0xFFu;
                if (!index_ok(k, last, buf.error_flags) || k < first) return 0u;
                const PairDesc& D = desc[k];
                const uint32_t na = D.free_count[0] + 1, nb = D.free_count[1] + 1, la = slot[k].loff;
                if (!index_ok(ka, na, buf.error_flags) || !index_ok(kb, nb, buf.error_flags)) return 0u;
                const uint2 r = merged_event(ev >> 24, list[la + ka], list[la + na + kb], D.ctx, ka, kb, D.l, D.row,
                                             s_tab, kTabD2, limit, &buf, slots);
                if (r.x & 0xFFFFu) atomicAdd(&slot[k].cand, r.x & 0xFFFFu);
                if (r.y) atomicAdd(&slot[k].r16, r.y);
                return r.x >> 16;
            };
            auto hit = [&](uint32_t ev, uint32_t tags) {
                const uint32_t kb = ev & 0xFFu, ka = (ev >> 8) & 0xFFu, k = (ev >> 16) & 0xFFu;
                if (k >= first && k < last)
                    push_hits(&buf, tags, ka, kb, desc[k].l, pair_m(desc[k].ctx), desc[k].row, true);
            };
            // the lane's position: slot k, offset off in it, (ka, kb) = (off / nb, off mod nb)
            uint32_t k = first, off = lane, size = 0, na = 1, nb = 1, la = 0, ka = 0, kb = 0, q32 = 0, r32 = 0;
            PairCtx c{};
            bool dual = false;
            Acc acc{0, 0, 0, 0, 0, 0};
            auto enter = [&]() {
                while (k < last && off >= slot[k].size) {
                    off -= slot[k].size;
                    ++k;
                }
                if (k < last) {
                    const uint32_t nab = slot[k].nab, st = slot[k].step;
                    size = slot[k].size;
                    na = nab & 0xFFFFu;
                    nb = nab >> 16;
                    la = slot[k].loff;
                    ka = (off * (st & 0x1FFFFu)) >> 16;  // off < 32 here (see seg_step)
                    kb = off - ka * nb;
                    q32 = (st >> 17) & 63u;
                    r32 = st >> 23;
                    c = desc[k].ctx;
                    dual = pair_dual(c);
                }
            };
            enter();
            for (uint32_t base = 0; base < total; base += 32) {
                uint32_t flags = 0;
                if (k < last) {
                    const AlphaHot a = list[la + ka], bh = list[la + na + kb];
                    flags = eval_fast<2, true>(a, bh.re, bh.im, bh.ra, bh.ia, (bh.ra >> 31) != 0, c, s_tab, acc,
                                               dual);
                }
                if (queue_push(q, qn, flags != 0, seg_event(kb, ka, k, flags)))
                    drain(q, qn, 32, wreq, buf.error_flags, handle, hit);
                if (k < last) {
                    off += 32;
                    if (off < size) {
                        ka += q32;
                        kb += r32;
                        if (kb >= nb) {
                            kb -= nb;
                            ++ka;
                        }
                    } else {
                        if (acc.cand) atomicAdd(&slot[k].cand, acc.cand);
                        if (acc.r16) atomicAdd(&slot[k].r16, acc.r16);
                        acc.cand = acc.r16 = 0;
                        enter();
                    }
                }
            }
            while (qn) drain(q, qn, qn < 32 ? qn : 32, wreq, buf.error_flags, handle, hit);
            __syncwarp();
            // the segment's pairs to their rows
            if (lane >= first && lane < last && desc[lane].state == 1) {
                const PairDesc& D = desc[lane];
                const uint64_t pa = D.free_count[0] + 1, pb = D.free_count[1] + 1;
                const uint64_t cand = slot[lane].cand + (D.cc & 1u), r16 = slot[lane].r16 + ((D.cc >> 1) & 1u);
                const uint64_t prod = pair_products((uint32_t)pa, (uint32_t)pb);
                RowCounts* rc = &buf.rows[D.row];
                if (cand) {
                    atomicAdd(&rc->candidates, (unsigned long long)cand);
                    atomicAdd(&rc->mcandidates, (unsigned long long)cand);
                }
                if (r16) {
                    atomicAdd(&rc->r16, (unsigned long long)r16);
                    atomicAdd(&rc->mr16, (unsigned long long)r16);
                }
                atomicAdd(&rc->products, (unsigned long long)prod);
                atomicAdd(&rc->mproducts, (unsigned long long)prod);
            }
            __syncwarp();
            first = last;
        }
        ns = nn;
        have = more;
    }
}

// Shared-prime pairs too big for a warp: one CTA per pair, from the
// descriptor the warp kernel left in the big queue (so every thread builds
// list entries at once); each warp takes every fourth round of 32 (alpha,
// beta) pairs and drains its events through a warp queue as merged_kernel.
__global__ void __launch_bounds__(kMergedThreads, 4) merged_big_kernel(const DeviceCache cache, const LaunchBuffers buf) {
    constexpr uint32_t kWarps = kMergedThreads / 32;
    __shared__ PairDesc D;
    __shared__ __align__(16) AlphaHot s_list[kMergedListCap];
    __shared__ uint32_t s_qi;
    // dynamic: warp queues, root requests, then the compact tables
    extern __shared__ __align__(16) unsigned char s_dyn[];
    uint64_t* s_queue = reinterpret_cast<uint64_t*>(s_dyn);
    RootReq* s_req = reinterpret_cast<RootReq*>(s_queue + kWarps * kQueue);
    uint8_t* s_tab = reinterpret_cast<uint8_t*>(s_req + kWarps * 32 * kReqPerLane);
    for (uint32_t i = threadIdx.x; i < kTableBytes; i += kMergedThreads) s_tab[i] = buf.tables[i];
    const uint32_t warp = threadIdx.x / 32, lane = threadIdx.x & 31;
    uint64_t* q = s_queue + warp * kQueue;
    RootReq* wreq = s_req + warp * 32 * kReqPerLane;
    uint32_t qn = 0;
    const uint32_t count = min(*buf.big_count, buf.big_cap);
    for (;;) {
        // pairs are taken from a cursor: their sizes vary by orders of magnitude
        __syncthreads();
        if (threadIdx.x == 0) s_qi = atomicAdd(buf.big_next, 1u);
        __syncthreads();
        const uint32_t qi = s_qi;
        if (qi >= count) break;
        if (threadIdx.x < sizeof(PairDesc) / 16)
            reinterpret_cast<uint4*>(&D)[threadIdx.x] = buf.big_queue[(size_t)qi * kBigEntryWords + threadIdx.x];
        __syncthreads();
        const uint32_t na = D.free_count[0] + 1, nb = D.free_count[1] + 1;
        if (na + nb > kMergedListCap) {
            if (threadIdx.x == 0) atomicOr(buf.error_flags, 2u);
            continue;
        }
        for (uint32_t k = threadIdx.x; k < na + nb; k += kMergedThreads) {
            const int side = k < na ? 0 : 1;
            desc_value_hot(cache, D, side, side ? k - na : k, s_list[k]);
        }
        __syncthreads();
        Acc acc{0, 0, 0, 0, 0, 0};
        if (threadIdx.x == 0) {
            acc.prod += pair_products(na, nb);
            acc.cand += D.cc & 1u;
            acc.r16 += (D.cc >> 1) & 1u;
        }
        const PairCtx c = D.ctx;
        const uint32_t l = D.l, row = D.row;
        const uint32_t total = na * nb;
        auto handle = [&](uint64_t ev, RootReq* slots) -> uint32_t {
            const uint32_t kb = (uint32_t)(ev & 0xFFFFu), ka = (uint32_t)((ev >> 16) & 0xFFFFFFu);
            if (!index_ok(ka, na, buf.error_flags) || !index_ok(kb, nb, buf.error_flags)) return 0u;
            const uint2 r = merged_event((uint32_t)(ev >> 40), s_list[ka], s_list[na + kb], c, ka, kb, l, row, s_tab,
                                         kTabD, (uint32_t)cache.limit, &buf, slots);
            acc.cand += r.x & 0xFFFFu;
            acc.r16 += r.y;
            return r.x >> 16;
        };
        auto hit = [&](uint64_t ev, uint32_t tags) {
            const uint32_t kb = (uint32_t)(ev & 0xFFFFu), ka = (uint32_t)((ev >> 16) & 0xFFFFFFu);
            push_hits(&buf, tags, ka, kb, l, pair_m(c), row, true);
        };
        // lane's (ka, kb) for k = 32 warp + lane + 128 j, advanced incrementally
        uint32_t ka = (32 * warp + lane) / nb, kb = 32 * warp + lane - ka * nb;
        const uint32_t qs = kMergedThreads / nb, rs = kMergedThreads - qs * nb;
        const bool dual = pair_dual(c);
        for (uint32_t base = 32 * warp; base < total; base += kMergedThreads) {
            uint32_t flags = 0;
            if (base + lane < total) {
                const AlphaHot a = s_list[ka], bh = s_list[na + kb];
                flags = dual ? eval_fast<1>(a, bh.re, bh.im, bh.ra, bh.ia, (bh.ra >> 31) != 0, c, s_tab, acc)
                             : eval_fast<0>(a, bh.re, bh.im, bh.ra, bh.ia, (bh.ra >> 31) != 0, c, s_tab, acc);
            }
            if (queue_push(q, qn, flags != 0, make_event(kb, ka, flags))) drain(q, qn, 32, wreq, buf.error_flags, handle, hit);
            ka += qs;
            kb += rs;
            if (kb >= nb) {
                kb -= nb;
                ++ka;
            }
        }
        while (qn) drain(q, qn, qn < 32 ? qn : 32, wreq, buf.error_flags, handle, hit);
        flush_acc(acc, &buf.rows[row], true);
    }
}

// Exact work queued by the search kernels (rare: products whose window
// decision was within the float error bound, and possible hits).  Exact
// coordinates come from the cache (row values doubled) or, for pairs that
// share a split prime, from the two term groups rebuilt for the pair.
__global__ void __launch_bounds__(128) exact_kernel(const DeviceCache cache, const LaunchBuffers buf) {
    __shared__ __align__(16) uint8_t s_tab[kTableBytes];
    for (uint32_t i = threadIdx.x; i < kTableBytes; i += blockDim.x) s_tab[i] = buf.tables[i];
    __syncthreads();
    const uint32_t count = min(*buf.exact_count, buf.exact_cap);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const ExactItem it = buf.exact_queue[i];
        const uint32_t kind = it.kind & 3u, p = (it.kind >> 2) & 1u, o = (it.kind >> 3) & 1u;
        const bool shared_prime = (it.kind & 16u) != 0;
        i128 ar, ai, br, bi;
        if (shared_prime) {
            MergedShared S;
            merged_setup(cache, buf.row_info[it.row], make_uint4(it.l, it.m, it.row, 0u), S, 0xFFFFFFFFu);
            group_value(cache, S.g[0], it.a, ar, ai);
            group_value(cache, S.g[1], it.b, br, bi);
        } else {
            const ExactRec ea = cache.exact[it.a], eb = cache.exact[it.b];
            ar = 2 * (i128)ea.re;
            ai = 2 * (i128)ea.im;
            br = eb.re;
            bi = eb.im;
        }
        const uint32_t omask = kind == kExCount ? 3u : (o ? 2u : 1u);
        uint32_t c = 0, r = 0;
        exact_eval(ar, ai, br, bi, p == 1, omask, it.l, it.m, cache.limit, it.row, s_tab, buf, &c, &r);
        if (kind != kExHit) {
            RowCounts* rc = &buf.rows[it.row];
            atomicAdd(&rc->candidates, (unsigned long long)c);
            atomicAdd(&rc->r16, (unsigned long long)r);
            atomicAdd(&rc->exact, 1ull);
            if (shared_prime) {
                atomicAdd(&rc->mcandidates, (unsigned long long)c);
                atomicAdd(&rc->mr16, (unsigned long long)r);
            }
        }
    }
}

// Serving: a wave's row counters into the requests' device-resident state.
__global__ void __launch_bounds__(128) scatter_rows_kernel(const RowCounts* __restrict__ rows,
                                                           const uint32_t* __restrict__ slots, uint32_t n,
                                                           RowCounts* __restrict__ state) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        RowCounts c = rows[i];
        c.pad = 1;
        state[slots[i]] = c;
    }
}

// INT32 throughput probe: 8 independent chains per thread, each step one
// IMAD and one shift/logic pair (the multiply and logic pipes the search loop
// uses); the result is stored so nothing is eliminated.
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
    // per unrolled step: 8 chains x (IMAD + SHF + LOP3)
    double ops = (double)blocks * threads * iters * 8.0 * 3.0;
    return ms > 0 ? ops / (ms * 1e-3) : 0;
}

// ------------------------------------------------------------------ host side

void fill_row_info(const uint32_t* spf, const uint32_t* seg_off, uint64_t n, uint64_t l, RowInfo* R) {
    *R = RowInfo{};
    R->l = l;
    R->l2 = l * l;
    R->l4 = (u128)R->l2 * R->l2;
    R->n4 = (u128)(n * n) * (n * n);
    R->lmodA = mod_u128_small(R->l4, kModA);
    R->lmodD = mod_u128_small(R->l4, kModD);
    R->l2x2f = (float)(2 * R->l2);
    R->l4f = (float)R->l4;
    R->l2modA = (uint32_t)(R->l2 % kModA);
    R->l3 = l % 3 == 0;
    R->l5 = l % 5 == 0;
    R->leven = (l & 1) == 0;
    R->free_l = seg_off[l + 1] - seg_off[l] - 1;
    R->seg = seg_off[l];
    R->fixed = 1;
    uint64_t x = l;
    while (x > 1) {
        uint32_t p = spf[x], a = 0;
        do {
            x /= p;
            ++a;
        } while (x % p == 0);
        if ((p & 3u) == 1u) {
            R->sp[R->nsplit] = p;
            R->se[R->nsplit] = a;
            ++R->nsplit;
        } else {
            for (uint32_t t = 0; t < 2 * a; ++t) R->fixed *= p;
        }
        if (p == 2) continue;
        R->pinv[R->nodd] = inverse_odd(p);
        R->pthr[R->nodd] = 0xFFFFFFFFu / p;
        if ((p & 3u) == 1u) R->psplit |= 1u << R->nodd;
        ++R->nodd;
    }
}

void build_residue_tables(uint8_t* out) {
    auto is4 = [](uint32_t r, uint32_t m) {
        for (uint64_t x = 0; x < m; ++x)
            if (x * x % m * x % m * x % m == r) return true;
        return false;
    };
    for (uint32_t z = 0; z < kModA; ++z) {
        bool m16 = (z & 15u) <= 1u;
        bool m9 = is4(z % 9, 9) && is4(z % 13, 13);
        bool m5 = is4(z % 5, 5);
        out[kTabA + z] = (uint8_t)((m16 ? 1u : 0u) | ((m16 && m9 && m5) ? 2u : 0u) |
                                   ((m16 && m9 && z % 5 == 0) ? 4u : 0u));
    }
    bool r17[17], r37[37], r73[73];
    for (uint32_t z = 0; z < 17; ++z) r17[z] = is4(z, 17);
    for (uint32_t z = 0; z < 37; ++z) r37[z] = is4(z, 37);
    for (uint32_t z = 0; z < 73; ++z) r73[z] = is4(z, 73);
    uint32_t words[kTabDWords] = {};
    for (uint32_t z = 0; z < kModD; ++z)
        if (r17[z % 17] && r37[z % 37] && r73[z % 73]) words[z >> 5] |= 1u << (z & 31u);
    memcpy(out + kTabD, words, sizeof words);
    // wide copy: both tables over two periods
    uint8_t* wide = out + kTableBytes;
    for (uint32_t z = 0; z < 2 * kModA; ++z) wide[z] = out[kTabA + z % kModA];
    uint32_t words2[kTabD2Words] = {};
    for (uint32_t z = 0; z < 2 * kModD; ++z)
        if ((words[(z % kModD) >> 5] >> ((z % kModD) & 31u)) & 1u) words2[z >> 5] |= 1u << (z & 31u);
    memcpy(wide + kTabD2, words2, sizeof words2);
}

size_t batched_smem_bytes(int threads, uint32_t alpha_cap) {
    const uint32_t warps = (uint32_t)threads / 32;
    return (size_t)alpha_cap * sizeof(AlphaHot) +
           (size_t)warps * (kChunk + kCarry) * sizeof(PairCtx) + (size_t)warps * kQueue * sizeof(uint64_t) +
           (size_t)warps * 32 * kReqPerLane * sizeof(RootReq) + kTable2Bytes;
}

// Compiled (threads, min CTAs per SM) variants of the persistent kernel; the
// second number caps registers per thread (65536 / (threads * min)).
static const void* batched_fn(int threads, int min_blocks) {
    if (threads == 128) return min_blocks >= 6 ? (const void*)batched_kernel<128, 6> : (const void*)batched_kernel<128, 4>;
    if (threads == 512) return (const void*)batched_kernel<512, 1>;
    return min_blocks >= 3 ? (const void*)batched_kernel<256, 3> : (const void*)batched_kernel<256, 2>;
}

int batched_max_ctas_per_sm(int threads, int min_blocks, size_t smem) {
    const void* fn = batched_fn(threads, min_blocks);
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, threads, smem) != cudaSuccess) return 1;
    return n > 0 ? n : 1;
}

cudaError_t launch_batched(const DeviceCache& cache, const WorkItem* items, uint32_t n_items,
                           const BatchedConfig& cfg, const LaunchBuffers& buf, cudaStream_t stream) {
    size_t smem = batched_smem_bytes(cfg.threads, cfg.alpha_cap);
    const void* fn = batched_fn(cfg.threads, cfg.min_blocks);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    void* args[] = {(void*)&cache, (void*)&items, (void*)&n_items, (void*)&cfg.alpha_cap, (void*)&buf};
    return cudaLaunchKernel(fn, dim3(cfg.ctas), dim3(cfg.threads), args, smem, stream);
}

cudaError_t launch_plain(const DeviceCache& cache, uint64_t first_l, uint32_t n_rows, uint32_t alpha_cap,
                         const LaunchBuffers& buf, cudaStream_t stream) {
    (void)first_l;
    size_t smem = (size_t)alpha_cap * sizeof(AlphaHot) + kTableBytes;
    cudaError_t e = cudaFuncSetAttribute((const void*)plain_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    plain_kernel<<<n_rows * kSlices, kPlainThreads, smem, stream>>>(cache, alpha_cap, buf);
    return cudaGetLastError();
}

cudaError_t launch_merged(const DeviceCache& cache, uint64_t pair_bound, const LaunchBuffers& buf, int ctas,
                          cudaStream_t stream, uint32_t* launches) {
    *launches = 0;
    const size_t smem = kPairWarps * 32 * kReqPerLane * sizeof(RootReq) + kTable2Bytes;
    cudaError_t e = cudaFuncSetAttribute((const void*)merged_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    // chunks of the queue: set-up, then the warp kernel; launches past the
    // queue's actual length return at once
    const uint64_t pairs = pair_bound < buf.merged_cap ? pair_bound : buf.merged_cap;
    for (uint64_t c0 = 0; c0 < pairs; c0 += buf.desc_chunk) {
        const uint32_t n = (uint32_t)(pairs - c0 < buf.desc_chunk ? pairs - c0 : buf.desc_chunk);
        const int setup_ctas = (int)((n + 127) / 128 < (uint64_t)ctas * 4 ? (n + 127) / 128 : (uint64_t)ctas * 4);
        merged_setup_kernel<<<setup_ctas, 128, 0, stream>>>(cache, buf, (uint32_t)c0);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        e = cudaMemsetAsync(buf.desc_next, 0, sizeof(unsigned int), stream);
        if (e != cudaSuccess) return e;
        // 8-warp CTAs, two per SM: half the grid of the 4-warp kernels
        merged_kernel<<<(ctas + 1) / 2, kPairWarps * 32, smem, stream>>>(cache, buf, (uint32_t)c0);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        *launches += 2;
    }
    const size_t big_smem = (kMergedThreads / 32) * (kQueue * sizeof(uint64_t) + 32 * kReqPerLane * sizeof(RootReq)) +
                            kTableBytes;
    e = cudaFuncSetAttribute((const void*)merged_big_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)big_smem);
    if (e != cudaSuccess) return e;
    merged_big_kernel<<<ctas, kMergedThreads, big_smem, stream>>>(cache, buf);
    *launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_scatter_rows(const RowCounts* rows, const uint32_t* slots, uint32_t n, RowCounts* state,
                                cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    const uint32_t blocks = (n + 127) / 128 < 1024 ? (n + 127) / 128 : 1024;
    scatter_rows_kernel<<<blocks, 128, 0, stream>>>(rows, slots, n, state);
    return cudaGetLastError();
}

cudaError_t launch_exact(const DeviceCache& cache, const LaunchBuffers& buf, int ctas, cudaStream_t stream) {
    exact_kernel<<<ctas, 128, 0, stream>>>(cache, buf);
    return cudaGetLastError();
}

}  // namespace hss
