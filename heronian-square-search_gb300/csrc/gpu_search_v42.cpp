// gpu_search_v42.cpp - command-line drop-in for the reference GPU search.
//
//   gpu_search_v42 LIMIT FIRST_L LAST_L RESULTS_FILE [GPU [STATE_FILE]]
//
// Same contract as the reference program (src/gpu_search_v42.cu:610-632 and
// Search::run :393-495), so scripts/gpu_queue.py, coverage_audit.py and
// verify_all_results.py work unchanged:
//   * 4-6 arguments, else the usage line on stderr and exit 2;
//   * stderr: "flattened N Gaussian values", "cached N Gaussian pair values",
//     "prepared in S seconds" (sizes recomputed for the same limit);
//   * the state file (when given) is read first: stored limit/end must match
//     and FIRST_L <= resume <= LAST_L + 1, then the search resumes at
//     `resume`; a file without a limit key (empty or truncated before it)
//     starts the range afresh, as the reference does; a value that is not an
//     integer is skipped (the reference's std::stoull would end the process);
//   * results are appended as "l m n area", skipping triples already in the
//     file; every hit has passed the device's 256-bit Heron recheck;
//   * after every batch of at most 512 roots: state written to STATE.tmp then
//     renamed (keys version, limit, begin, end, resume, candidates; candidates
//     counted from process start), and one stdout line
//     "PROGRESS resume R candidates C seconds S";
//   * SIGTERM / SIGINT stop at the next batch boundary with a checkpoint.
// Differences: a checkpoint mismatch or a device error exits 2 / 1 instead of
// 0 (the reference returns 0, gpu_search_v42.cu:442-445, 461-465); the mode
// (batched by default) can be set with HSS_MODE=plain.
//
// Invoked as gpu_search_v36 (the same program under the name the heavy-root
// queue looks for, experiments/heavy/heavy_queue.py:36-45) it takes a 7th
// argument MIN_WEIGHT and follows experiments/heavy/gpu_search_v36.cu:
//   * only roots l whose branch weight W(l) = prod over split primes p^e of l
//     of (4e + 1) is at least MIN_WEIGHT are searched (all roots when 0);
//   * batches are 4096 root positions when MIN_WEIGHT > 0;
//   * the state also holds "min_weight", which must match on resume, and
//     "begin" is the first root of the whole range;
//   * with a state file and MIN_WEIGHT > 0, STATE.done is rewritten after
//     every batch: "limit N", "min_weight W", then every searched root of the
//     completed prefix, one per line (scripts/coverage_audit.py:71-99).
#include <signal.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <array>
#include <atomic>
#include <chrono>
#include <fstream>
#include <iostream>
#include <set>
#include <string>
#include <vector>

#include "../../include/hss.h"

namespace {

std::atomic<bool> stop_requested{false};

void on_signal(int) { stop_requested.store(true); }

bool parse_u64(const char* s, uint64_t* out) {
    if (!s || !*s) return false;
    char* end = nullptr;
    unsigned long long v = strtoull(s, &end, 10);
    if (*end) return false;
    *out = v;
    return true;
}

std::string decimal(unsigned __int128 v) {
    if (v == 0) return "0";
    std::string s;
    while (v) {
        s.push_back(char('0' + (int)(v % 10)));
        v /= 10;
    }
    return std::string(s.rbegin(), s.rend());
}

int usage(bool heavy_cli) {
    if (heavy_cli)
        std::cerr << "usage: gpu_search LIMIT FIRST_L LAST_L RESULTS_FILE [GPU [STATE_FILE [MIN_WEIGHT]]]\n";
    else
        std::cerr << "usage: gpu_search LIMIT FIRST_L LAST_L RESULTS_FILE [GPU [STATE_FILE]]\n";
    return 2;
}

// Branch weight of l: prod (4e + 1) over its primes p = 1 mod 4 with exponent
// e (experiments/heavy/gpu_search_v36.cu:51-56), by trial division.
uint32_t branch_weight(uint64_t l) {
    uint32_t w = 1;
    for (uint64_t p = 2; p * p <= l; p += (p == 2 ? 1 : 2)) {
        if (l % p) continue;
        uint32_t e = 0;
        while (l % p == 0) {
            l /= p;
            ++e;
        }
        if (p % 4 == 1) w *= 4 * e + 1;
    }
    if (l > 1 && l % 4 == 1) w *= 5;
    return w;
}

bool heavy_name(const char* argv0) {
    const char* slash = strrchr(argv0, '/');
    return strcmp(slash ? slash + 1 : argv0, "gpu_search_v36") == 0;
}

}  // namespace

int main(int argc, char** argv) {
    const bool heavy_cli = heavy_name(argv[0]);
    if (argc < 5 || argc > (heavy_cli ? 8 : 7)) return usage(heavy_cli);
    uint64_t n = 0, first = 0, last = 0, device = 0, min_weight = 0;
    if (!parse_u64(argv[1], &n) || !parse_u64(argv[2], &first) || !parse_u64(argv[3], &last))
        return usage(heavy_cli);
    if (argc >= 6 && !parse_u64(argv[5], &device)) return usage(heavy_cli);
    if (argc == 8 && (!parse_u64(argv[7], &min_weight) || min_weight > 0xFFFFFFFFull)) return usage(heavy_cli);
    const std::string results_file = argv[4];
    const std::string state_file = argc >= 7 ? argv[6] : "";
    if (n < 1 || n > HSS_MAX_LIMIT || first < 1 || first > last || last > n) {
        std::cerr << "invalid range: need 1 <= FIRST_L <= LAST_L <= LIMIT <= " << HSS_MAX_LIMIT << "\n";
        return 2;
    }
    signal(SIGTERM, on_signal);
    signal(SIGINT, on_signal);

    // checkpoint (gpu_search_v42.cu:433-447), validated before any device work
    uint64_t begin = first;
    if (!state_file.empty()) {
        std::ifstream state(state_file);
        std::string key, value;
        uint64_t stored_limit = 0, stored_end = 0, saved = first, stored_weight = 0;
        while (state >> key >> value) {
            uint64_t v = 0;
            if (!parse_u64(value.c_str(), &v)) continue;
            if (key == "limit") stored_limit = v;
            if (key == "end") stored_end = v;
            if (key == "resume") saved = v;
            if (key == "min_weight") stored_weight = v;
        }
        // a resume beyond last + 1 cannot come from this range (the
        // reference would take it and search nothing); rejected here
        if (stored_limit && (stored_limit != n || stored_end != last || saved < first || saved > last + 1 ||
                             (heavy_cli && stored_weight != min_weight))) {
            std::cerr << (heavy_cli ? "checkpoint does not match requested range or weight\n"
                                    : "checkpoint does not match requested range\n");
            return 2;
        }
        begin = saved;
    }

    const char* mode_env = getenv("HSS_MODE");
    const int mode = (mode_env && strcmp(mode_env, "plain") == 0) ? HSS_MODE_PLAIN : HSS_MODE_BATCHED;

    auto prep_start = std::chrono::steady_clock::now();
    hss_t* h = nullptr;
    int s = hss_open(n, (int)device, nullptr, &h);
    if (s) {
        std::cerr << "hss_open: " << hss_strerror(s) << "\n";
        return 1;
    }
    uint64_t records = 0, flattened = 0, cached = 0;
    hss_info(h, nullptr, &records, &flattened, &cached, nullptr);
    std::cerr << "flattened " << flattened << " Gaussian values\n";
    std::cerr << "cached " << cached << " Gaussian pair values\n";
    std::cerr << "prepared in "
              << std::chrono::duration<double>(std::chrono::steady_clock::now() - prep_start).count()
              << " seconds\n";

    // results file: created in append mode, existing triples reloaded
    // (gpu_search_v42.cu:448-452)
    std::set<std::array<uint64_t, 3>> seen;
    {
        std::ofstream touch(results_file, std::ios::app);
        std::ifstream old(results_file);
        uint64_t l, m, root;
        std::string area;
        while (old >> l >> m >> root >> area) seen.insert({l, m, root});
    }
    std::ofstream out(results_file, std::ios::app);

    auto start = std::chrono::steady_clock::now();
    uint64_t next = begin, candidates = 0;
    std::vector<hss_hit> hits(4096);
    const uint64_t batch_size = min_weight ? 4096 : 512;
    std::vector<uint64_t> heavy_done;  // searched roots of the completed prefix (.done)
    if (min_weight)
        for (uint64_t l = first; l < begin; ++l)
            if (branch_weight(l) >= min_weight) heavy_done.push_back(l);
    int rc = 0;
    while (next <= last && !stop_requested.load()) {
        uint64_t batch_last = std::min<uint64_t>(next + batch_size - 1, last);
        hss_counts counts{};
        uint32_t nhits = 0;
        if (min_weight) {
            // the batch's heavy roots, each its own interval, in one launch sequence
            std::vector<uint64_t> ls;
            for (uint64_t l = next; l <= batch_last; ++l)
                if (branch_weight(l) >= min_weight) ls.push_back(l);
            s = HSS_OK;
            if (!ls.empty()) {
                std::vector<hss_counts> per(ls.size());
                s = hss_search_many(h, ls.data(), ls.data(), (uint32_t)ls.size(), per.data(), &counts, hits.data(),
                                    (uint32_t)hits.size(), &nhits);
            }
            if (!s) heavy_done.insert(heavy_done.end(), ls.begin(), ls.end());
        } else {
            s = hss_search(h, next, batch_last, mode, &counts, nullptr, hits.data(), (uint32_t)hits.size(), &nhits);
        }
        if (s) {
            std::cerr << hss_strerror(s) << ": " << hss_last_error(h) << "\n";
            rc = 1;
            break;
        }
        candidates += counts.candidates;
        for (uint32_t i = 0; i < nhits && i < hits.size(); ++i) {
            const hss_hit& hit = hits[i];
            if (!hit.heron_ok) {
                std::cerr << "rejected internal hit " << hit.l << ' ' << hit.m << ' ' << hit.n << "\n";
                continue;
            }
            if (!seen.insert({hit.l, hit.m, hit.n}).second) continue;
            __int128 a4 = ((__int128)hit.area4_hi << 64) | (__int128)hit.area4_lo;
            unsigned __int128 area = (unsigned __int128)(a4 < 0 ? -a4 : a4) / 4;
            out << hit.l << ' ' << hit.m << ' ' << hit.n << ' ' << decimal(area) << '\n';
        }
        out.flush();
        next = batch_last + 1;
        if (!state_file.empty() && min_weight) {
            std::string done_file = state_file + ".done", tmp = done_file + ".tmp";
            {
                std::ofstream done(tmp);
                done << "limit " << n << "\nmin_weight " << min_weight << '\n';
                for (uint64_t l : heavy_done) done << l << '\n';
            }
            if (rename(tmp.c_str(), done_file.c_str()) != 0) {
                std::cerr << "cannot write " << done_file << "\n";
                rc = 1;
                break;
            }
        }
        if (!state_file.empty()) {
            std::string tmp = state_file + ".tmp";
            {
                std::ofstream st(tmp);
                st << "version 1\nlimit " << n << "\nbegin " << (heavy_cli ? first : begin) << "\nend " << last
                   << "\nresume " << next << "\ncandidates " << candidates << '\n';
                if (heavy_cli) st << "min_weight " << min_weight << '\n';
            }
            if (rename(tmp.c_str(), state_file.c_str()) != 0) {
                std::cerr << "cannot write state file " << state_file << "\n";
                rc = 1;
                break;
            }
        }
        double seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
        std::cout << "PROGRESS resume " << next << " candidates " << candidates << " seconds "
                  << (uint64_t)seconds << std::endl;
    }
    hss_close(h);
    return rc;
}
