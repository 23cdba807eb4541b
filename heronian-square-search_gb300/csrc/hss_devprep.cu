// hss_devprep.cu - the factor cache built on the device.
//
// The same arrays, layout and values as build_host_cache (hss_prep.cpp, which
// follows src/gpu_search_v42.cu:354-391, :525-594), made by sm_103a kernels
// instead of host threads, so that opening a handle needs no host pass over
// 10^7 integers and no upload of the 3.4 GB cache:
//   1. spf[x]: trial division of every x by the primes up to sqrt(N) (those
//      few hundred primes come from a host sieve), one thread per x;
//   2. prime-power table: per split prime p its block size (sum over a of
//      4a+1, a <= 2 log_p N), an exclusive scan for pp_base, then a warp per
//      p finds pi = u + iv (smallest u, as the host) and writes
//      pi^r conj(pi)^(4a-r) for every a and r, exact and hot;
//   3. segment sizes (W(x)-1)/2 + 1 from the factorisation of x, an exclusive
//      scan for seg_off;
//   4. one thread per x writes its free set and central value, enumerating the
//      free vectors in the host's order with an odometer over the digits of
//      the later primes (64-bit products: every partial product divides x^2 in
//      the Gaussian integers, so its coordinates are at most x^2 < 2^50).
// The host keeps copies of spf and seg_off (the item builder reads them).
#include <cuda_runtime.h>
#include <math.h>

#include <chrono>
#include <vector>

#include "hss_api_status.h"
#include "hss_prep.h"

namespace hss {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ uint32_t residue64(int64_t v, uint32_t m) {
    const int64_t r = v % (int64_t)m;
    return (uint32_t)(r < 0 ? r + m : r);
}

__device__ __forceinline__ uint32_t pack64(int64_t v) {
    return residue64(v, kModA) | (residue64(v, kModD) << kShiftD);
}

// Number of powers p^j <= n (j >= 1), as the host's power_count.
__device__ __forceinline__ uint32_t power_count(uint64_t p, uint64_t n) {
    uint32_t k = 0;
    for (uint64_t q = p; q <= n; q *= p) {
        ++k;
        if (q > n / p) break;
    }
    return k;
}

struct Factors {
    uint32_t primes[8];
    uint32_t exps[8];
    uint32_t count;
    uint64_t fixed;
};

__device__ Factors factor(const uint32_t* spf, uint32_t x) {
    Factors f;
    f.count = 0;
    f.fixed = 1;
    while (x > 1) {
        const uint32_t p = spf[x];
        uint32_t a = 0;
        do {
            x /= p;
            ++a;
        } while (x % p == 0);
        if (p % 4 == 1) {
            f.primes[f.count] = p;
            f.exps[f.count] = a;
            ++f.count;
        } else {
            for (uint32_t i = 0; i < 2 * a; ++i) f.fixed *= p;
        }
    }
    return f;
}

__global__ void sieve_kernel(uint32_t* spf, uint32_t n, const uint32_t* primes, uint32_t nprimes) {
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x <= n; x += gridDim.x * blockDim.x) {
        if (x < 2) {
            spf[x] = x;  // spf[0] = 0, spf[1] = 1
            continue;
        }
        uint32_t s = x;
        for (uint32_t i = 0; i < nprimes; ++i) {
            const uint32_t p = primes[i];
            if (p * p > x) break;
            if (x % p == 0) {
                s = p;
                break;
            }
        }
        spf[x] = s;
    }
}

// Block sizes of the prime-power table (0 unless p is a split prime) and
// the largest exponent covered.
__global__ void pp_size_kernel(const uint32_t* spf, uint32_t n, uint64_t* size, unsigned int* max_exp) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p <= n; p += gridDim.x * blockDim.x) {
        uint64_t s = 0;
        if (p >= 5 && p % 4 == 1 && spf[p] == p) {
            const uint32_t max_a = 2 * power_count(p, n);
            s = 2ull * max_a * max_a + 3ull * max_a;  // sum_{a=1}^{max_a} (4a+1)
            atomicMax(max_exp, max_a);
        }
        size[p] = s;
    }
}

struct Gauss {
    __int128 re, im;
};

__device__ __forceinline__ Gauss gmul(Gauss a, Gauss b) {
    return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}

// Exact floor(sqrt(r)) for r < 2^26 (float estimate, integer correction).
__device__ __forceinline__ uint32_t isqrt32(uint32_t r) {
    uint32_t v = (uint32_t)sqrtf((float)r);
    while (v * v > r) --v;
    while ((v + 1) * (v + 1) <= r) ++v;
    return v;
}

// A warp per integer p <= N; split primes only: the lanes try u = 1, 2, ...
// 32 at a time for p - u^2 a square (the smallest such u, as the host), then
// take the block's entries (a, r) in turn, each pi^r conj(pi)^(4a-r) by
// repeated products (at most 4a <= 8 log_5 N of them, no per-thread arrays).
__global__ void pp_fill_kernel(const uint32_t* spf, uint32_t n, const uint64_t* offs, uint32_t* pp_base,
                               HotRec* pp_hot, __int128* pp_exact) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warps = gridDim.x * blockDim.x / 32;
    for (uint32_t p = (blockIdx.x * blockDim.x + threadIdx.x) / 32; p <= n; p += warps) {
        if (!(p >= 5 && p % 4 == 1 && spf[p] == p)) {
            if (lane == 0) pp_base[p] = 0xFFFFFFFFu;
            continue;
        }
        uint32_t u = 0;
        for (uint32_t u0 = 1; (uint64_t)u0 * u0 <= p; u0 += 32) {
            const uint32_t uu = u0 + lane;
            bool sq = false;
            if ((uint64_t)uu * uu <= p) {
                const uint32_t rem = p - uu * uu, v = isqrt32(rem);
                sq = v * v == rem;
            }
            const uint32_t m = __ballot_sync(0xFFFFFFFFu, sq);
            if (m) {
                u = u0 + __ffs(m) - 1;
                break;
            }
        }
        const uint32_t v = isqrt32(p - u * u);
        const uint32_t max_a = 2 * power_count(p, n);
        const uint64_t base = offs[p];
        if (lane == 0) pp_base[p] = (uint32_t)base;
        const Gauss pi{(__int128)u, (__int128)v}, pc{(__int128)u, -(__int128)v};
        const uint32_t total = 2 * max_a * max_a + 3 * max_a;
        for (uint32_t k = lane; k < total; k += 32) {
            uint32_t a = 1, r = k;
            while (r >= 4 * a + 1) {
                r -= 4 * a + 1;
                ++a;
            }
            Gauss val{1, 0};
            for (uint32_t j = 0; j < r; ++j) val = gmul(val, pi);
            for (uint32_t j = 0; j < 4 * a - r; ++j) val = gmul(val, pc);
            pp_exact[2 * (base + k)] = val.re;
            pp_exact[2 * (base + k) + 1] = val.im;
            HotRec h;
            h.re = i128_to_float(val.re);
            h.im = i128_to_float(val.im);
            h.rre = pack_residues(val.re) | (r == 2 * a ? kCentralBit : 0u);
            h.rim = pack_residues(val.im);
            pp_hot[base + k] = h;
        }
    }
}

// Segment lengths (free set + central value), the reference's cached-value
// count (free + central + raw per x) and the longest segment.
__global__ void seg_size_kernel(const uint32_t* spf, uint32_t n, uint64_t* len, unsigned long long* ref_cached,
                                unsigned int* longest) {
    unsigned long long local = 0;
    uint32_t lmax = 0;
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x <= n + 1; x += gridDim.x * blockDim.x) {
        if (x == 0 || x == n + 1) {
            len[x] = 0;
            continue;
        }
        const Factors f = factor(spf, x);
        uint64_t w = 1;
        for (uint32_t i = 0; i < f.count; ++i) w *= 4u * f.exps[i] + 1;
        len[x] = (w - 1) / 2 + 1;
        local += (w - 1) / 2 + 1 + w;
        lmax = max(lmax, (uint32_t)((w - 1) / 2 + 1));
    }
    for (int d = 16; d > 0; d >>= 1) {
        local += __shfl_down_sync(0xFFFFFFFFu, local, d);
        lmax = max(lmax, __shfl_down_sync(0xFFFFFFFFu, lmax, d));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(ref_cached, local);
        atomicMax(longest, lmax);
    }
}

__global__ void narrow_kernel(const uint64_t* in, uint32_t* out, uint32_t count) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
        out[i] = (uint32_t)in[i];
}

struct Writer {
    HotRec* hot;
    ExactRec* exact;
    uint32_t* owner;
    uint32_t x;
    uint64_t pos, end;  // end: the next segment's start
    __device__ void emit(int64_t re, int64_t im, bool central) {
        if (pos >= end) {  // more values than the segment holds: counted by the caller's check
            ++pos;
            return;
        }
        HotRec h;
        h.re = (float)re;
        h.im = (float)im;
        h.rre = pack64(re) | (central ? kCentralBit : 0u);
        h.rim = pack64(im);
        hot[pos] = h;
        exact[pos] = ExactRec{re, im};
        owner[pos] = x;
        ++pos;
    }
};

__device__ __forceinline__ void cmul64(int64_t ar, int64_t ai, int64_t br, int64_t bi, int64_t& re, int64_t& im) {
    re = ar * br - ai * bi;
    im = ar * bi + ai * br;
}

// Free set of x, then its central value: for the first non-central index i
// and r_i < 2e_i, every digit combination of the later primes with the
// earlier digit most significant (the host's recursion order).
__global__ void seg_fill_kernel(const uint32_t* spf, uint32_t n, const uint32_t* seg_off, const uint32_t* pp_base,
                                const __int128* pp_exact, HotRec* hot, ExactRec* exact, uint32_t* owner,
                                unsigned int* err) {
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x <= n; x += gridDim.x * blockDim.x) {
        if (x == 0) continue;
        const Factors f = factor(spf, x);
        Writer w{hot, exact, owner, x, seg_off[x], seg_off[x + 1]};
        const __int128* vals[8];
        uint32_t sizes[8];
        for (uint32_t i = 0; i < f.count; ++i) {
            vals[i] = pp_exact + 2 * ((uint64_t)pp_base[f.primes[i]] + pp_exponent_offset(f.exps[i]));
            sizes[i] = 4u * f.exps[i] + 1;
        }
        int64_t prefix = (int64_t)f.fixed;  // fixed(x) * prod_{j<i} p_j^(2e_j)
        for (uint32_t i = 0; i < f.count; ++i) {
            const uint32_t centre = 2u * f.exps[i];
            for (uint32_t r = 0; r < centre; ++r) {
                // stack[j]: product through term j - 1; digits of terms i+1 .. count-1
                int64_t sr[9], si[9];
                uint32_t dig[8];
                sr[i + 1] = prefix * (int64_t)vals[i][2 * r];
                si[i + 1] = prefix * (int64_t)vals[i][2 * r + 1];
                for (uint32_t j = i + 1; j < f.count; ++j) {
                    dig[j] = 0;
                    cmul64(sr[j], si[j], (int64_t)vals[j][0], (int64_t)vals[j][1], sr[j + 1], si[j + 1]);
                }
                for (;;) {
                    w.emit(sr[f.count], si[f.count], false);
                    // advance the odometer, last digit fastest; done when every digit wrapped
                    uint32_t j = f.count;
                    bool more = false;
                    while (j > i + 1) {
                        --j;
                        if (++dig[j] < sizes[j]) {
                            more = true;
                            break;
                        }
                        dig[j] = 0;
                    }
                    if (!more) break;
                    for (uint32_t k = j; k < f.count; ++k)
                        cmul64(sr[k], si[k], (int64_t)vals[k][2 * dig[k]], (int64_t)vals[k][2 * dig[k] + 1],
                               sr[k + 1], si[k + 1]);
                }
            }
            prefix *= (int64_t)vals[i][2 * centre];
        }
        w.emit((int64_t)x * (int64_t)x, 0, true);
        if (w.pos != seg_off[x + 1]) atomicOr(err, 1u);  // segment size invariant
    }
}

// Exclusive scan of count 64-bit values (in place allowed): tile sums, a
// single-block scan of the tile sums, then each tile scanned with its offset.
constexpr uint32_t kScanTile = 4 * kThreads;

__device__ __forceinline__ uint64_t block_exclusive(uint64_t v, uint64_t* s_warp, uint64_t* total) {
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x / 32;
    uint64_t incl = v;
    for (int d = 1; d < 32; d <<= 1) {
        const uint64_t t = __shfl_up_sync(0xFFFFFFFFu, incl, d);
        if (lane >= (uint32_t)d) incl += t;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint64_t ws = lane < kThreads / 32 ? s_warp[lane] : 0;
        uint64_t wi = ws;
        for (int d = 1; d < 32; d <<= 1) {
            const uint64_t t = __shfl_up_sync(0xFFFFFFFFu, wi, d);
            if (lane >= (uint32_t)d) wi += t;
        }
        if (lane < kThreads / 32) s_warp[lane] = wi - ws;
        if (lane == kThreads / 32 - 1) *total = wi;
    }
    __syncthreads();
    const uint64_t r = s_warp[warp] + incl - v;
    __syncthreads();
    return r;
}

__global__ void scan_tiles_kernel(const uint64_t* in, uint64_t count, uint64_t* tile_sums) {
    __shared__ uint64_t s_warp[kThreads / 32];
    __shared__ uint64_t total;
    const uint64_t base = (uint64_t)blockIdx.x * kScanTile + 4ull * threadIdx.x;
    uint64_t v = 0;
    for (uint32_t k = 0; k < 4; ++k)
        if (base + k < count) v += in[base + k];
    block_exclusive(v, s_warp, &total);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

__global__ void scan_sums_kernel(uint64_t* tile_sums, uint32_t tiles, uint64_t* grand) {
    __shared__ uint64_t s_warp[kThreads / 32];
    __shared__ uint64_t total;
    uint64_t carry = 0;
    for (uint32_t b = 0; b < tiles; b += kThreads) {
        const uint64_t v = b + threadIdx.x < tiles ? tile_sums[b + threadIdx.x] : 0;
        const uint64_t e = block_exclusive(v, s_warp, &total);
        if (b + threadIdx.x < tiles) tile_sums[b + threadIdx.x] = carry + e;
        carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) *grand = carry;
}

__global__ void scan_apply_kernel(const uint64_t* in, uint64_t count, const uint64_t* tile_sums, uint64_t* out) {
    __shared__ uint64_t s_warp[kThreads / 32];
    __shared__ uint64_t total;
    const uint64_t base = (uint64_t)blockIdx.x * kScanTile + 4ull * threadIdx.x;
    uint64_t v[4], sum = 0;
    for (uint32_t k = 0; k < 4; ++k) {
        v[k] = base + k < count ? in[base + k] : 0;
        sum += v[k];
    }
    __syncthreads();  // in and out may alias: every read of the tile precedes its writes
    uint64_t run = tile_sums[blockIdx.x] + block_exclusive(sum, s_warp, &total);
    for (uint32_t k = 0; k < 4; ++k) {
        if (base + k < count) out[base + k] = run;
        run += v[k];
    }
}

// Exclusive scan of in[0 .. count) into out; *grand (device) receives the total.
cudaError_t exclusive_scan(const uint64_t* in, uint64_t* out, uint64_t count, uint64_t* tile_sums, uint64_t* grand,
                           cudaStream_t st) {
    const uint32_t tiles = (uint32_t)((count + kScanTile - 1) / kScanTile);
    scan_tiles_kernel<<<tiles, kThreads, 0, st>>>(in, count, tile_sums);
    scan_sums_kernel<<<1, kThreads, 0, st>>>(tile_sums, tiles, grand);
    scan_apply_kernel<<<tiles, kThreads, 0, st>>>(in, count, tile_sums, out);
    return cudaGetLastError();
}

template <class T>
cudaError_t dalloc(T** p, size_t count, std::vector<void*>* owned) {
    cudaError_t e = cudaMalloc((void**)p, (count ? count : 1) * sizeof(T));
    if (e == cudaSuccess) owned->push_back(*p);
    return e;
}

}  // namespace

int build_device_cache(uint64_t n, int sm_count, CUstream_st* st, DeviceBuild* out, std::string* err) {
    auto t0 = std::chrono::steady_clock::now();
    if (n < 1 || n > kMaxLimit) {
        *err = "limit out of range";
        return HSS_ERR_ARGUMENT;
    }
    DeviceBuild& b = *out;
    b.limit = n;
    std::vector<void*> scratch;
    auto cleanup = [&]() {
        for (void* p : scratch) cudaFree(p);
        scratch.clear();
    };
    auto release = [&]() {  // on failure the cache arrays go too
        cleanup();
        for (void* p : b.owned) cudaFree(p);
        b.owned.clear();
    };
    auto fail = [&](cudaError_t e) {
        release();
        *err = cudaGetErrorString(e);
        return HSS_ERR_CUDA;
    };
#define DEV(call)                          \
    do {                                   \
        cudaError_t e_ = (call);           \
        if (e_ != cudaSuccess) return fail(e_); \
    } while (0)
    // primes up to sqrt(n) for the sieve (a few hundred)
    uint32_t root = (uint32_t)sqrt((double)n);
    while ((uint64_t)(root + 1) * (root + 1) <= n) ++root;
    while ((uint64_t)root * root > n) --root;
    std::vector<uint32_t> small_primes;
    {
        std::vector<uint8_t> comp(root + 1, 0);
        for (uint32_t i = 2; i <= root; ++i) {
            if (comp[i]) continue;
            small_primes.push_back(i);
            for (uint64_t j = (uint64_t)i * i; j <= root; j += i) comp[j] = 1;
        }
    }
    const int grid = sm_count * 8;
    uint32_t* d_primes = nullptr;
    uint64_t *d_u64 = nullptr, *d_tiles = nullptr, *d_grand = nullptr;
    unsigned int* d_flags = nullptr;  // [0] max exponent, [1] longest segment, [2] fill error
    unsigned long long* d_refc = nullptr;
    DEV(dalloc(&d_primes, small_primes.size(), &scratch));
    DEV(dalloc(&d_u64, n + 2, &scratch));
    DEV(dalloc(&d_tiles, (n + 2 + kScanTile - 1) / kScanTile + 1, &scratch));
    DEV(dalloc(&d_grand, 1, &scratch));
    DEV(dalloc(&d_flags, 4, &scratch));
    DEV(dalloc(&d_refc, 1, &scratch));
    DEV(cudaMemsetAsync(d_flags, 0, 4 * sizeof(unsigned int), st));
    DEV(cudaMemsetAsync(d_refc, 0, sizeof(unsigned long long), st));
    if (!small_primes.empty())
        DEV(cudaMemcpyAsync(d_primes, small_primes.data(), small_primes.size() * sizeof(uint32_t),
                            cudaMemcpyHostToDevice, st));

    // 1. smallest prime factors
    DEV(dalloc(&b.spf, n + 1, &b.owned));
    sieve_kernel<<<grid, kThreads, 0, st>>>(b.spf, (uint32_t)n, d_primes, (uint32_t)small_primes.size());
    DEV(cudaGetLastError());

    // 2. prime-power table
    pp_size_kernel<<<grid, kThreads, 0, st>>>(b.spf, (uint32_t)n, d_u64, d_flags + 0);
    DEV(cudaGetLastError());
    DEV(exclusive_scan(d_u64, d_u64, n + 1, d_tiles, d_grand, st));
    uint64_t pp_total = 0;
    DEV(cudaMemcpyAsync(&pp_total, d_grand, sizeof pp_total, cudaMemcpyDeviceToHost, st));
    DEV(cudaStreamSynchronize(st));
    if (pp_total >= UINT32_MAX) {
        release();
        *err = "prime-power table exceeds 32-bit indexing";
        return HSS_ERR_LIMIT;
    }
    b.reference_flattened = pp_total;
    b.pp_count = pp_total;
    DEV(dalloc(&b.pp_base, n + 1, &b.owned));
    DEV(dalloc(&b.pp_hot, pp_total, &b.owned));
    DEV(dalloc(&b.pp_exact, 2 * pp_total, &b.owned));
    pp_fill_kernel<<<grid, kThreads, 0, st>>>(b.spf, (uint32_t)n, d_u64, b.pp_base, b.pp_hot, b.pp_exact);
    DEV(cudaGetLastError());

    // 3. segment offsets
    seg_size_kernel<<<grid, kThreads, 0, st>>>(b.spf, (uint32_t)n, d_u64, d_refc, d_flags + 1);
    DEV(cudaGetLastError());
    DEV(exclusive_scan(d_u64, d_u64, n + 2, d_tiles, d_grand, st));
    uint64_t records = 0;
    unsigned int flags[4];
    unsigned long long refc = 0;
    DEV(cudaMemcpyAsync(&records, d_grand, sizeof records, cudaMemcpyDeviceToHost, st));
    DEV(cudaMemcpyAsync(flags, d_flags, sizeof flags, cudaMemcpyDeviceToHost, st));
    DEV(cudaMemcpyAsync(&refc, d_refc, sizeof refc, cudaMemcpyDeviceToHost, st));
    DEV(cudaStreamSynchronize(st));
    if (records >= UINT32_MAX) {
        release();
        *err = "factor cache exceeds 32-bit indexing";
        return HSS_ERR_LIMIT;
    }
    b.records = records;
    b.max_exponent = flags[0];
    b.longest = flags[1];
    b.reference_cached = refc;
    DEV(dalloc(&b.seg_off, n + 2, &b.owned));
    narrow_kernel<<<grid, kThreads, 0, st>>>(d_u64, b.seg_off, (uint32_t)(n + 2));
    DEV(cudaGetLastError());

    // 4. records
    DEV(dalloc(&b.hot, records, &b.owned));
    DEV(dalloc(&b.exact, records, &b.owned));
    DEV(dalloc(&b.owner, records, &b.owned));
    seg_fill_kernel<<<grid, kThreads, 0, st>>>(b.spf, (uint32_t)n, b.seg_off, b.pp_base, b.pp_exact, b.hot, b.exact,
                                               b.owner, d_flags + 2);
    DEV(cudaGetLastError());

    // host copies the item builder reads
    b.spf_host.resize(n + 1);
    b.seg_off_host.resize(n + 2);
    DEV(cudaMemcpyAsync(b.spf_host.data(), b.spf, (n + 1) * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    DEV(cudaMemcpyAsync(b.seg_off_host.data(), b.seg_off, (n + 2) * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    DEV(cudaMemcpyAsync(flags, d_flags, sizeof flags, cudaMemcpyDeviceToHost, st));
    DEV(cudaStreamSynchronize(st));
#undef DEV
    if (flags[2]) {
        release();
        *err = "device cache build: a segment's size disagrees with its enumeration";
        return HSS_ERR_LIMIT;
    }
    cleanup();
    b.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return HSS_OK;
}

}  // namespace hss
