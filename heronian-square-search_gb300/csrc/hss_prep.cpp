// hss_prep.cpp - host construction of the Gaussian factor cache.
//
// Follows the reference's preparation (src/gpu_search_v42.cu:354-391 sieve and
// factor summary, :570-594 Gaussian primes and prime powers, :525-568 factor
// sets) but stores only what the kernels read: per integer x its free set and
// central value (the reference also stores the raw set, which the kernels here
// rebuild from free(x) and its conjugates), in a hot (float + residues) and an
// exact (int64) layout, built on all host threads.
#include "hss_prep.h"

#include <atomic>
#include <chrono>
#include <cmath>
#include <thread>

#include "hss_api_status.h"

namespace hss {
namespace {

using i128 = __int128;

struct G {
    i128 re, im;
};

inline G gmul(G a, G b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
inline G gconj(G a) { return {a.re, -a.im}; }

inline uint32_t residue64(int64_t v, uint32_t m) {
    int64_t r = v % (int64_t)m;
    return (uint32_t)(r < 0 ? r + m : r);
}

inline uint32_t pack64(int64_t v) {
    return residue64(v, kModA) | (residue64(v, kModD) << kShiftD);
}

inline HotRec make_hot(int64_t re, int64_t im, bool central) {
    HotRec h;
    h.re = (float)re;
    h.im = (float)im;
    h.rre = pack64(re) | (central ? kCentralBit : 0u);
    h.rim = pack64(im);
    return h;
}

// Number of powers p^j <= n (j >= 1).
inline uint32_t power_count(uint64_t p, uint64_t n) {
    uint32_t k = 0;
    for (uint64_t q = p; q <= n; q *= p) {
        ++k;
        if (q > n / p) break;
    }
    return k;
}

template <class F>
void parallel_for(uint64_t begin, uint64_t end, uint64_t grain, int threads, F&& body) {
    std::atomic<uint64_t> next{begin};
    auto work = [&]() {
        for (;;) {
            uint64_t lo = next.fetch_add(grain);
            if (lo >= end) break;
            uint64_t hi = lo + grain < end ? lo + grain : end;
            body(lo, hi);
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; ++t) pool.emplace_back(work);
    work();
    for (auto& th : pool) th.join();
}

// Writes the free set of x followed by its central value (x^2, 0) into
// [hot, exact) starting at `pos`.  Free vectors are generated position by
// position: for the first non-central index i and r_i < 2e_i, every value of
// the later primes (the pruning of gpu_search_v42.cu:525-552, expressed as a
// direct enumeration instead of a recursive set build).
struct SegmentWriter {
    const HostCache* cache;
    HotRec* hot;
    ExactRec* exact;
    uint32_t* owner;
    uint64_t x;
    uint64_t pos;
    const G* vals[8];
    uint32_t sizes[8];
    uint32_t count;

    void emit(G v, bool central) {
        int64_t re = (int64_t)v.re, im = (int64_t)v.im;
        hot[pos] = make_hot(re, im, central);
        exact[pos] = ExactRec{re, im};
        owner[pos] = (uint32_t)x;
        ++pos;
    }

    void suffix(uint32_t j, G acc) {
        if (j == count) {
            emit(acc, false);
            return;
        }
        for (uint32_t r = 0; r < sizes[j]; ++r) suffix(j + 1, gmul(acc, vals[j][r]));
    }
};

}  // namespace

NumberFactors factor_number(const uint32_t* spf, uint64_t x) {
    NumberFactors f{};
    f.fixed = 1;
    while (x > 1) {
        uint32_t p = spf[x], a = 0;
        do {
            x /= p;
            ++a;
        } while (x % p == 0);
        if (p % 4 == 1) {
            f.primes[f.count] = p;
            f.exps[f.count] = (uint8_t)a;
            ++f.count;
        } else {
            for (uint32_t i = 0; i < 2 * a; ++i) f.fixed *= p;
        }
    }
    return f;
}

int build_host_cache(uint64_t n, int threads, HostCache* out, std::string* err) {
    auto t0 = std::chrono::steady_clock::now();
    if (n < 1 || n > kMaxLimit) {
        *err = "limit out of range";
        return HSS_ERR_ARGUMENT;
    }
    if (threads < 1) threads = 1;
    HostCache& c = *out;
    c.limit = n;

    // Smallest-prime-factor sieve (gpu_search_v42.cu:355-363).
    c.spf.assign(n + 1, 0);
    for (uint64_t i = 2; i <= n; ++i) {
        if (c.spf[i]) continue;
        c.spf[i] = (uint32_t)i;
        if (i <= n / i)
            for (uint64_t j = i * i; j <= n; j += i)
                if (!c.spf[j]) c.spf[j] = (uint32_t)i;
    }
    c.spf[1] = 1;

    // Gaussian primes pi = u + iv with the smallest u, and the prime-power
    // values pi^r conj(pi)^(4a-r), r = 0..4a, for a = 1..2k with p^k <= N
    // (gpu_search_v42.cu:570-594).
    c.pp_base.assign(n + 1, UINT32_MAX);
    uint64_t pp_total = 0;
    uint32_t max_exp = 0;
    for (uint64_t p = 5; p <= n; p += 4) {
        if (c.spf[p] != p) continue;
        uint32_t max_a = 2 * power_count(p, n);
        c.pp_base[p] = (uint32_t)pp_total;
        pp_total += 2ull * max_a * max_a + 3ull * max_a;  // sum_{a=1}^{max_a} (4a+1)
        if (max_a > max_exp) max_exp = max_a;
    }
    if (pp_total >= UINT32_MAX) {
        *err = "prime-power table exceeds 32-bit indexing";
        return HSS_ERR_LIMIT;
    }
    c.max_exponent = max_exp;
    c.reference_flattened = pp_total;
    c.pp_hot.resize(pp_total);
    c.pp_exact.resize(2 * pp_total);
    parallel_for(5, n + 1, 1 << 16, threads, [&](uint64_t lo, uint64_t hi) {
        std::vector<G> powers;
        for (uint64_t p = lo; p < hi; ++p) {
            if (p % 4 != 1 || c.spf[p] != p) continue;
            uint64_t u = 1, v = 0;
            for (; u * u <= p; ++u) {
                v = (uint64_t)std::sqrt((double)(p - u * u));
                if (v * v == p - u * u) break;
            }
            uint32_t max_a = 2 * power_count(p, n);
            G pi{(i128)u, (i128)v};
            uint64_t pos = c.pp_base[p];
            for (uint32_t a = 1; a <= max_a; ++a) {
                powers.assign(4 * a + 1, G{1, 0});
                for (uint32_t r = 1; r <= 4 * a; ++r) powers[r] = gmul(powers[r - 1], pi);
                for (uint32_t r = 0; r <= 4 * a; ++r) {
                    G val = gmul(powers[r], gconj(powers[4 * a - r]));
                    c.pp_exact[2 * pos] = val.re;
                    c.pp_exact[2 * pos + 1] = val.im;
                    HotRec h;
                    h.re = i128_to_float(val.re);
                    h.im = i128_to_float(val.im);
                    h.rre = pack_residues(val.re) | (r == 2 * a ? kCentralBit : 0u);
                    h.rim = pack_residues(val.im);
                    c.pp_hot[pos] = h;
                    ++pos;
                }
            }
        }
    });

    // Segment sizes: free set (W-1)/2 plus the central value, W = prod(4e+1).
    c.seg_off.assign(n + 2, 0);
    std::vector<uint32_t> seg_len(n + 1, 0);
    std::atomic<uint64_t> ref_cached{0};
    parallel_for(1, n + 1, 1 << 16, threads, [&](uint64_t lo, uint64_t hi) {
        uint64_t local = 0;
        for (uint64_t x = lo; x < hi; ++x) {
            NumberFactors f = factor_number(c.spf.data(), x);
            uint64_t w = 1;
            for (uint32_t i = 0; i < f.count; ++i) w *= 4u * f.exps[i] + 1;
            seg_len[x] = (uint32_t)((w - 1) / 2 + 1);
            local += (w - 1) / 2 + 1 + w;  // free + central + raw, as the reference caches
        }
        ref_cached += local;
    });
    c.reference_cached = ref_cached.load();
    uint64_t total = 0;
    for (uint64_t x = 0; x <= n; ++x) {
        c.seg_off[x] = (uint32_t)total;
        total += seg_len[x];
        if (total >= UINT32_MAX) {
            *err = "factor cache exceeds 32-bit indexing";
            return HSS_ERR_LIMIT;
        }
    }
    c.seg_off[n + 1] = (uint32_t)total;
    c.records = total;
    c.hot.reset(new HotRec[total]);
    c.exact.reset(new ExactRec[total]);
    c.owner.reset(new uint32_t[total]);

    parallel_for(1, n + 1, 1 << 12, threads, [&](uint64_t lo, uint64_t hi) {
        for (uint64_t x = lo; x < hi; ++x) {
            NumberFactors f = factor_number(c.spf.data(), x);
            SegmentWriter w{};
            w.cache = &c;
            w.hot = c.hot.get();
            w.exact = c.exact.get();
            w.owner = c.owner.get();
            w.x = x;
            w.pos = c.seg_off[x];
            w.count = f.count;
            for (uint32_t i = 0; i < f.count; ++i) {
                const i128* base = &c.pp_exact[2 * (c.pp_base[f.primes[i]] + pp_exponent_offset(f.exps[i]))];
                w.vals[i] = reinterpret_cast<const G*>(base);
                w.sizes[i] = 4u * f.exps[i] + 1;
            }
            i128 prefix = (i128)f.fixed;  // fixed(x) * prod_{j<i} p_j^(2e_j)
            for (uint32_t i = 0; i < f.count; ++i) {
                uint32_t centre = 2u * f.exps[i];
                for (uint32_t r = 0; r < centre; ++r) {
                    G v = w.vals[i][r];
                    w.suffix(i + 1, G{prefix * v.re, prefix * v.im});
                }
                prefix *= w.vals[i][centre].re;
            }
            w.emit(G{(i128)x * (i128)x, 0}, true);
            if (w.pos != c.seg_off[x + 1]) std::abort();  // segment size invariant
        }
    });
    c.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return HSS_OK;
}

}  // namespace hss
