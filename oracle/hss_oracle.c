/*
 * hss_oracle.c - CPU oracle for the square-sided Heronian triangle search.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA path is
 * compared against: only tests/, __graft_entry__.smoke() and bench.py (its
 * cpu_baseline / reference arm) may load it.  Nothing in the product library
 * links, calls or falls back to it.
 *
 * It is a plain-C restatement of the reference's CPU search
 * (src/search_v18.cpp), which defines what a "candidate" is and which roots
 * are hits.  Each function below names the reference lines it follows.
 * Parity is pinned against the reference's own known-answer cases
 * (scripts/smoke_test.py:8-25), its archived interval counts
 * (evidence/benchmarks/gpu-opt-benchmark.json:15-20, v45-ab.json:9-12) and
 * against the reference binary itself built from source (oracle/Makefile,
 * target `ref`), whose outputs are committed as JSON under tests/golden.
 *
 * Besides the reference's counters (pairs, candidates) it also reports, per
 * root row, the counters the GPU kernels export: processed pairs Q, Gaussian
 * products P, candidates C and candidates whose z passes the mod-16 test R.
 */
#define _GNU_SOURCE
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef __int128 i128;
typedef unsigned __int128 u128;

typedef struct { i128 re, im; } gauss_t;

/* Per-integer factor summary (search_v18.cpp:65-71, filled at :169-195). */
typedef struct {
    uint32_t primes[8];   /* distinct primes p = 1 (mod 4), increasing */
    uint8_t exps[8];
    uint8_t count;
    uint64_t fixed;       /* product of p^(2a) over p = 2 or p = 3 (mod 4) */
    uint32_t inert_part;  /* product of distinct primes p = 3 (mod 4) */
} ora_number_t;

/* Gaussian prime-power table for one split prime (search_v18.cpp:73-76). */
typedef struct {
    uint32_t offsets[32];   /* offsets[a] = first value of exponent a */
    uint32_t max_a;
    gauss_t *values;
} ora_prime_t;

typedef struct {
    const gauss_t *values;
    uint32_t size;      /* 4e+1 */
    uint32_t central;   /* 2e   */
} ora_term_t;

typedef struct {
    uint64_t l, m, n;
    i128 area4;
} ora_hit_t;

typedef struct {
    uint64_t limit;
    uint32_t *spf;
    ora_number_t *info;
    ora_prime_t **prime;    /* indexed by p, NULL unless p is a split prime */
    uint8_t mod625[625], mod9[9], mod7[7], mod13[13], mod17[17];
} ora_tables_t;

/* Per-row, per-thread scratch (the reference keeps these thread_local,
 * search_v18.cpp:92-94). */
typedef struct {
    const ora_tables_t *t;
    uint64_t l, m;
    u128 l4, m4, n4;
    i128 lower_d, upper_d;
    uint32_t flags;
    uint64_t products, candidates, r16;
    ora_hit_t *hits;
    size_t nhits, cap_hits;
} ora_ctx_t;

static gauss_t g_mul(gauss_t a, gauss_t b) {          /* search_v18.cpp:100-102 */
    gauss_t r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
    return r;
}

static gauss_t g_conj(gauss_t a) {                    /* search_v18.cpp:108-110 */
    gauss_t r = {a.re, -a.im};
    return r;
}

static uint64_t gcd_u64(uint64_t a, uint64_t b) {
    while (b) { uint64_t r = a % b; a = b; b = r; }
    return a;
}

/* 128-bit value modulo a small modulus (search_v18.cpp:132-138).  Always
 * inlined: every caller passes a constant modulus, so the compiler replaces
 * the divisions by multiplications, as the reference's template residue<P>
 * gets them. */
static inline __attribute__((always_inline)) uint32_t mod_u128(u128 v, uint32_t p) {
    uint64_t shift = (uint64_t)(((u128)1 << 64) % p);
    uint64_t lo = (uint64_t)v % p, hi = (uint64_t)(v >> 64) % p;
    return (uint32_t)((lo + hi * shift) % p);
}

/* Table of fourth-power residues modulo M (search_v18.cpp:140-145). */
static void fourth_residue_table(uint8_t *table, uint32_t modulus) {
    memset(table, 0, modulus);
    for (uint64_t x = 0; x < modulus; ++x) table[(x * x % modulus) * x % modulus * x % modulus] = 1;
}

/* ---------------------------------------------------------------- 256-bit */

/* 4x64-bit little-endian limbs; product truncated to 256 bits as in
 * search_v18.cpp:35-54. */
static void mul256(const uint64_t a[4], const uint64_t b[4], uint64_t out[4]) {
    uint64_t acc[8] = {0};
    for (int i = 0; i < 4; ++i) {
        u128 carry = 0;
        for (int j = 0; j < 4; ++j) {
            u128 cur = (u128)a[i] * b[j] + acc[i + j] + carry;
            acc[i + j] = (uint64_t)cur;
            carry = cur >> 64;
        }
        for (int k = i + 4; carry && k < 8; ++k) {
            u128 cur = (u128)acc[k] + carry;
            acc[k] = (uint64_t)cur;
            carry = cur >> 64;
        }
    }
    memcpy(out, acc, 4 * sizeof(uint64_t));
}

static void set256(uint64_t out[4], u128 v) {
    out[0] = (uint64_t)v; out[1] = (uint64_t)(v >> 64); out[2] = 0; out[3] = 0;
}

/* Heron recheck of a hit in 256-bit arithmetic (search_v18.cpp:481-501):
 * the four Heron factors of sides l^2, m^2, n^2 are positive and their
 * product equals area4^2. */
int hss_oracle_heron_ok(uint64_t l, uint64_t m, uint64_t n, i128 area4) {
    uint64_t x = l * l, y = m * m, z = n * n;
    i128 f[4] = {(i128)x + y + z, -(i128)x + y + z, (i128)x - y + z, (i128)x + y - z};
    if (f[0] <= 0 || f[1] <= 0 || f[2] <= 0 || f[3] <= 0 || area4 % 4 != 0) return 0;
    uint64_t h[4], t[4];
    set256(h, (u128)f[0]);
    for (int i = 1; i < 4; ++i) { set256(t, (u128)f[i]); mul256(h, t, h); }
    i128 a = area4 < 0 ? -area4 : area4;
    uint64_t e[4], ea[4];
    set256(ea, (u128)a);
    mul256(ea, ea, e);
    return memcmp(h, e, sizeof h) == 0;
}

/* ---------------------------------------------------------------- prepare */

static uint64_t ipow(uint64_t a, uint32_t n) {
    uint64_t r = 1;
    while (n--) r *= a;
    return r;
}

/* Smallest-prime-factor sieve, per-integer factor summary and the Gaussian
 * prime-power tables (search_v18.cpp:159-197, 285-309). */
static ora_tables_t *tables_build(uint64_t n) {
    ora_tables_t *t = calloc(1, sizeof *t);
    t->limit = n;
    t->spf = calloc(n + 1, sizeof(uint32_t));
    t->info = calloc(n + 1, sizeof(ora_number_t));
    t->prime = calloc(n + 1, sizeof(ora_prime_t *));
    for (uint64_t i = 2; i <= n; ++i) {
        if (t->spf[i]) continue;
        t->spf[i] = (uint32_t)i;
        if (i <= n / i)
            for (uint64_t j = i * i; j <= n; j += i)
                if (!t->spf[j]) t->spf[j] = (uint32_t)i;
    }
    t->spf[1] = 1;
    for (uint64_t i = 1; i <= n; ++i) {
        ora_number_t *info = &t->info[i];
        uint64_t x = i, fixed = 1;
        info->inert_part = 1;
        while (x > 1) {
            uint32_t p = t->spf[x], a = 0;
            do { x /= p; ++a; } while (x % p == 0);
            if (p % 4 == 1) {
                info->primes[info->count] = p;
                info->exps[info->count] = (uint8_t)a;
                ++info->count;
            } else {
                fixed *= ipow(p, 2 * a);
                if (p % 4 == 3) info->inert_part *= p;
            }
        }
        info->fixed = fixed;
    }
    /* Gaussian primes pi = u + iv with the smallest u, and for each exponent a
     * up to twice the largest power of p below n the 4a+1 values
     * pi^r * conj(pi)^(4a-r) (search_v18.cpp:285-309). */
    for (uint64_t p = 5; p <= n; p += 4) {
        if (t->spf[p] != p) continue;
        uint64_t u = 1, v = 0;
        for (; u * u <= p; ++u) {
            v = (uint64_t)sqrt((double)(p - u * u));
            if (v * v == p - u * u) break;
        }
        ora_prime_t *d = calloc(1, sizeof *d);
        uint32_t max_a = 0;
        for (uint64_t power = p; power <= n; power *= p) ++max_a;
        max_a *= 2;
        d->max_a = max_a;
        size_t total = 0;
        for (uint32_t a = 1; a <= max_a; ++a) total += 4 * a + 1;
        d->values = malloc(total * sizeof(gauss_t));
        gauss_t pi = {(i128)u, (i128)v};
        gauss_t *powers = malloc((4 * max_a + 1) * sizeof(gauss_t));
        size_t pos = 0;
        for (uint32_t a = 1; a <= max_a; ++a) {
            d->offsets[a] = (uint32_t)pos;
            powers[0].re = 1; powers[0].im = 0;
            for (uint32_t r = 1; r <= 4 * a; ++r) powers[r] = g_mul(powers[r - 1], pi);
            for (uint32_t r = 0; r <= 4 * a; ++r)
                d->values[pos++] = g_mul(powers[r], g_conj(powers[4 * a - r]));
        }
        free(powers);
        t->prime[p] = d;
    }
    fourth_residue_table(t->mod625, 625);
    fourth_residue_table(t->mod9, 9);
    fourth_residue_table(t->mod7, 7);
    fourth_residue_table(t->mod13, 13);
    fourth_residue_table(t->mod17, 17);
    return t;
}

static void tables_free(ora_tables_t *t) {
    if (!t) return;
    for (uint64_t p = 0; p <= t->limit; ++p)
        if (t->prime[p]) { free(t->prime[p]->values); free(t->prime[p]); }
    free(t->prime);
    free(t->info);
    free(t->spf);
    free(t);
}

/* ------------------------------------------------------------- candidates */

static void push_hit(ora_ctx_t *c, uint64_t root, i128 area4) {
    for (size_t i = 0; i < c->nhits; ++i)
        if (c->hits[i].l == c->l && c->hits[i].m == c->m && c->hits[i].n == root) return;
    if (c->nhits == c->cap_hits) {
        c->cap_hits = c->cap_hits ? 2 * c->cap_hits : 16;
        c->hits = realloc(c->hits, c->cap_hits * sizeof(ora_hit_t));
    }
    ora_hit_t h = {c->l, c->m, root, area4};
    c->hits[c->nhits++] = h;
}

/* Largest r with r^4 <= z, for z <= limit^4 (the reference seeds with a
 * floating-point fourth root and corrects exactly, search_v18.cpp:472-474). */
static uint64_t fourth_root_floor(u128 z, uint64_t limit) {
    uint64_t r = (uint64_t)sqrtl(sqrtl((long double)z));
    while (r > 0 && (u128)r * r * r * r > z) --r;
    while (r < limit && (u128)(r + 1) * (r + 1) * (r + 1) * (r + 1) <= z) ++r;
    return r;
}

/* The candidate test: the counter is bumped on entry, then z = l^4+m^4-d is
 * range-checked, filtered by fourth-power residues and tested exactly
 * (search_v18.cpp:455-479). */
static void test_d(ora_ctx_t *c, i128 d, i128 area4) {
    const ora_tables_t *t = c->t;
    ++c->candidates;
    i128 signed_z = (i128)c->l4 + (i128)c->m4 - d;
    if (signed_z < 0 || (u128)signed_z < c->m4 || (u128)signed_z > c->n4) return;
    u128 z = (u128)signed_z;
    uint32_t low = (uint32_t)z & 15;
    if (low != 0 && low != 1) return;
    ++c->r16;
    if (c->flags & 2U) {
        if (mod_u128(z, 625) != 0) return;
    } else if (!t->mod625[mod_u128(z, 625)]) return;
    if (!t->mod9[mod_u128(z, 9)] || !t->mod7[mod_u128(z, 7)] || !t->mod13[mod_u128(z, 13)] ||
        !t->mod17[mod_u128(z, 17)])
        return;
    uint64_t root = fourth_root_floor(z, t->limit);
    if ((u128)root * root * root * root != z) return;
    if (gcd_u64(gcd_u64(c->l, c->m), root) != 1) return;
    if ((c->l % 5 && c->m % 5 && root % 5) || root < c->m || root > t->limit) return;
    if (!hss_oracle_heron_ok(c->l, c->m, root, area4)) {
        fprintf(stderr, "oracle: rejected internal hit %llu %llu %llu\n", (unsigned long long)c->l,
                (unsigned long long)c->m, (unsigned long long)root);
        return;
    }
    push_hit(c, root, area4);
}

/* One orientation (D, 4A) of a product: area filters and the sign window
 * [l^4+m^4-N^4, l^4] for +D and -D (search_v18.cpp:441-453). */
static void test_pair(ora_ctx_t *c, i128 d, i128 area4) {
    if (area4 == 0 || ((uint64_t)area4 & 7) != 0) return;
    int positive = d >= c->lower_d && d <= c->upper_d;
    int negative = -d >= c->lower_d && -d <= c->upper_d;
    if (!positive && !negative) return;
    u128 a = (u128)(area4 < 0 ? -area4 : area4);
    if (mod_u128(a, 3) != 0) return;
    if ((c->flags & 1U) && mod_u128(a, 9) != 0) return;
    if ((c->flags & 2U) && mod_u128(a, 5) != 0) return;
    if (positive) test_d(c, d, area4);
    if (negative && d != 0) test_d(c, -d, area4);
}

/* Both orientations of a product (search_v18.cpp:436-439). */
static void test_all(ora_ctx_t *c, gauss_t z) {
    ++c->products;
    test_pair(c, z.re, z.im);
    if (z.re != z.im && z.re != -z.im) test_pair(c, z.im, z.re);
}

/* Depth-first product over the merged terms with the central/free pruning
 * that keeps one of each conjugate pair (search_v18.cpp:373-434; the
 * reference's unrolled depth 1-4 cases enumerate the same products). */
static void enumerate(ora_ctx_t *c, const ora_term_t *terms, uint32_t count, uint32_t depth,
                      gauss_t z, int free_choice) {
    const ora_term_t *term = &terms[depth];
    uint32_t last = free_choice ? term->size - 1 : term->central;
    if (depth + 1 == count) {  /* the last term: the products themselves */
        for (uint32_t r = 0; r <= last; ++r) test_all(c, g_mul(z, term->values[r]));
        return;
    }
    for (uint32_t r = 0; r <= last; ++r)
        enumerate(c, terms, count, depth + 1, g_mul(z, term->values[r]),
                  free_choice || r < term->central);
}

typedef struct {
    uint64_t products, candidates, r16, processed;
} ora_row_counts_t;

/* All m in [l, N] for one root l (search_v18.cpp:329-371); with step > 1
 * only m = m0, m0 + step, ... (a bounded sample of the row for timing). */
static void process_row_stride(ora_ctx_t *c, uint64_t l, uint64_t m0, uint64_t step,
                               ora_row_counts_t *out) {
    const ora_tables_t *t = c->t;
    const uint64_t n = t->limit;
    const ora_number_t *a = &t->info[l];
    c->l = l;
    c->l4 = (u128)l * l * l * l;
    c->n4 = (u128)n * n * n * n;
    c->products = c->candidates = c->r16 = 0;
    uint64_t processed = 0;
    for (uint64_t m = m0; m <= n; m += step) {
        if ((l & 1) == 0 && (m & 1) == 0) continue;
        const ora_number_t *b = &t->info[m];
        if (a->inert_part > 1 && gcd_u64(a->inert_part, m) > 1) continue;
        ora_term_t terms[16];
        uint32_t count = 0, i = 0, j = 0;
        while (i < a->count || j < b->count) {
            uint32_t p, e;
            if (j == b->count || (i < a->count && a->primes[i] < b->primes[j])) {
                p = a->primes[i]; e = a->exps[i++];
            } else if (i == a->count || b->primes[j] < a->primes[i]) {
                p = b->primes[j]; e = b->exps[j++];
            } else {
                p = a->primes[i]; e = (uint32_t)a->exps[i] + b->exps[j]; ++i; ++j;
            }
            const ora_prime_t *d = t->prime[p];
            terms[count].values = d->values + d->offsets[e];
            terms[count].size = 4 * e + 1;
            terms[count].central = 2 * e;
            ++count;
        }
        if (count == 0) continue;
        ++processed;
        c->m = m;
        c->m4 = (u128)m * m * m * m;
        c->lower_d = (i128)c->l4 + (i128)c->m4 - (i128)c->n4;
        c->upper_d = (i128)c->l4;
        c->flags = ((l % 3 == 0 || m % 3 == 0) ? 1U : 0U) | ((l % 5 != 0 && m % 5 != 0) ? 2U : 0U);
        gauss_t base = {(i128)2 * (i128)a->fixed * (i128)b->fixed, 0};
        enumerate(c, terms, count, 0, base, 0);
    }
    out->products = c->products;
    out->candidates = c->candidates;
    out->r16 = c->r16;
    out->processed = processed;
}

static void process_row(ora_ctx_t *c, uint64_t l, ora_row_counts_t *out) {
    process_row_stride(c, l, l, 1, out);
}

/* ------------------------------------------------------------ public API */

/* Hit record as returned to callers: area4 split into two 64-bit halves. */
typedef struct {
    uint64_t l, m, n;
    uint64_t area4_lo;
    int64_t area4_hi;
} hss_oracle_hit_t;

typedef struct {
    const ora_tables_t *t;
    uint64_t first, last;
    _Atomic uint64_t next;
    ora_row_counts_t *rows;
    pthread_mutex_t lock;
    ora_hit_t *hits;
    size_t nhits, cap;
} ora_job_t;

static void *worker(void *arg) {
    ora_job_t *job = arg;
    ora_ctx_t c;
    memset(&c, 0, sizeof c);
    c.t = job->t;
    for (;;) {
        uint64_t l = atomic_fetch_add(&job->next, 1);
        if (l > job->last) break;
        process_row(&c, l, &job->rows[l - job->first]);
    }
    pthread_mutex_lock(&job->lock);
    for (size_t i = 0; i < c.nhits; ++i) {
        if (job->nhits == job->cap) {
            job->cap = job->cap ? 2 * job->cap : 16;
            job->hits = realloc(job->hits, job->cap * sizeof(ora_hit_t));
        }
        job->hits[job->nhits++] = c.hits[i];
    }
    pthread_mutex_unlock(&job->lock);
    free(c.hits);
    return NULL;
}

static int hit_cmp(const void *x, const void *y) {
    const ora_hit_t *a = x, *b = y;
    if (a->l != b->l) return a->l < b->l ? -1 : 1;
    if (a->m != b->m) return a->m < b->m ? -1 : 1;
    if (a->n != b->n) return a->n < b->n ? -1 : 1;
    return 0;
}

/* Opaque prepared tables, so one preparation can serve many searches. */
void *hss_oracle_prepare(uint64_t limit) {
    if (limit == 0 || limit > 100000000ULL) return NULL;
    return tables_build(limit);
}

void hss_oracle_release(void *tables) { tables_free((ora_tables_t *)tables); }

/*
 * Search root rows first..last (1 <= first <= last <= limit) on `threads`
 * threads.  Per-row arrays (length last-first+1, any may be NULL) receive
 * candidates, products, processed pairs and mod-16 survivors.  Hits are
 * sorted by (l, m, n), deduplicated and copied up to `hit_cap`; the total is
 * returned in *nhits.  Returns 0, or -1 on invalid arguments.
 */
int hss_oracle_search(void *tables, uint64_t first, uint64_t last, int threads,
                      uint64_t *row_candidates, uint64_t *row_products, uint64_t *row_processed,
                      uint64_t *row_r16, hss_oracle_hit_t *hits, uint32_t hit_cap,
                      uint32_t *nhits) {
    ora_tables_t *t = tables;
    if (!t || first == 0 || first > last || last > t->limit) return -1;
    if (threads < 1) threads = 1;
    uint64_t rows = last - first + 1;
    if ((uint64_t)threads > rows) threads = (int)rows;
    ora_job_t job;
    memset(&job, 0, sizeof job);
    job.t = t;
    job.first = first;
    job.last = last;
    atomic_init(&job.next, first);
    job.rows = calloc(rows, sizeof(ora_row_counts_t));
    pthread_mutex_init(&job.lock, NULL);
    pthread_t *tid = malloc(threads * sizeof(pthread_t));
    for (int i = 0; i < threads; ++i) pthread_create(&tid[i], NULL, worker, &job);
    for (int i = 0; i < threads; ++i) pthread_join(tid[i], NULL);
    free(tid);
    for (uint64_t r = 0; r < rows; ++r) {
        if (row_candidates) row_candidates[r] = job.rows[r].candidates;
        if (row_products) row_products[r] = job.rows[r].products;
        if (row_processed) row_processed[r] = job.rows[r].processed;
        if (row_r16) row_r16[r] = job.rows[r].r16;
    }
    qsort(job.hits, job.nhits, sizeof(ora_hit_t), hit_cmp);
    size_t unique = 0;
    for (size_t i = 0; i < job.nhits; ++i)
        if (unique == 0 || hit_cmp(&job.hits[unique - 1], &job.hits[i]) != 0)
            job.hits[unique++] = job.hits[i];
    for (size_t i = 0; i < unique && i < hit_cap; ++i) {
        hits[i].l = job.hits[i].l;
        hits[i].m = job.hits[i].m;
        hits[i].n = job.hits[i].n;
        hits[i].area4_lo = (uint64_t)job.hits[i].area4;
        hits[i].area4_hi = (int64_t)(job.hits[i].area4 >> 64);
    }
    if (nhits) *nhits = (uint32_t)unique;
    free(job.hits);
    free(job.rows);
    pthread_mutex_destroy(&job.lock);
    return 0;
}

/* Strided sample of rows, for timing the CPU search on a bounded share of a
 * batch: job j searches root ls[j] over m = m0s[j], m0s[j] + step, ... <= N,
 * one job per thread at a time.  Per job, *logical receives the number of m
 * visited (the logical pairs) and *candidates the candidates counted.
 * Returns 0, or -1 on invalid arguments. */
typedef struct {
    const ora_tables_t *t;
    const uint64_t *ls, *m0s;
    uint64_t step;
    uint32_t njobs;
    _Atomic uint32_t next;
    uint64_t *logical, *candidates;
} ora_sample_t;

static void *sample_worker(void *arg) {
    ora_sample_t *s = arg;
    ora_ctx_t c;
    memset(&c, 0, sizeof c);
    c.t = s->t;
    for (;;) {
        uint32_t j = atomic_fetch_add(&s->next, 1);
        if (j >= s->njobs) break;
        ora_row_counts_t out;
        process_row_stride(&c, s->ls[j], s->m0s[j], s->step, &out);
        if (s->logical) s->logical[j] = (s->t->limit - s->m0s[j]) / s->step + 1;
        if (s->candidates) s->candidates[j] = out.candidates;
    }
    free(c.hits);
    return NULL;
}

int hss_oracle_sample(void *tables, const uint64_t *ls, const uint64_t *m0s, uint64_t step,
                      uint32_t njobs, int threads, uint64_t *logical, uint64_t *candidates) {
    ora_tables_t *t = tables;
    if (!t || !ls || !m0s || step == 0 || njobs == 0) return -1;
    for (uint32_t j = 0; j < njobs; ++j)
        if (ls[j] == 0 || m0s[j] < ls[j] || m0s[j] > t->limit) return -1;
    if (threads < 1) threads = 1;
    if ((uint32_t)threads > njobs) threads = (int)njobs;
    ora_sample_t s;
    memset(&s, 0, sizeof s);
    s.t = t;
    s.ls = ls;
    s.m0s = m0s;
    s.step = step;
    s.njobs = njobs;
    atomic_init(&s.next, 0);
    s.logical = logical;
    s.candidates = candidates;
    pthread_t *tid = malloc(threads * sizeof(pthread_t));
    for (int i = 0; i < threads; ++i) pthread_create(&tid[i], NULL, sample_worker, &s);
    for (int i = 0; i < threads; ++i) pthread_join(tid[i], NULL);
    free(tid);
    return 0;
}

/* Exported for tests of single products: the candidate count and mod-16
 * survivors that one product z = re + i*im contributes for pair (l, m). */
int hss_oracle_product(void *tables, uint64_t l, uint64_t m, int64_t re_hi, uint64_t re_lo,
                       int64_t im_hi, uint64_t im_lo, uint64_t *candidates, uint64_t *r16) {
    ora_tables_t *t = tables;
    if (!t || l == 0 || l > m || m > t->limit) return -1;
    ora_ctx_t c;
    memset(&c, 0, sizeof c);
    c.t = t;
    c.l = l;
    c.m = m;
    uint64_t n = t->limit;
    c.l4 = (u128)l * l * l * l;
    c.m4 = (u128)m * m * m * m;
    c.n4 = (u128)n * n * n * n;
    c.lower_d = (i128)c.l4 + (i128)c.m4 - (i128)c.n4;
    c.upper_d = (i128)c.l4;
    c.flags = ((l % 3 == 0 || m % 3 == 0) ? 1U : 0U) | ((l % 5 != 0 && m % 5 != 0) ? 2U : 0U);
    gauss_t z = {((i128)re_hi << 64) | re_lo, ((i128)im_hi << 64) | im_lo};
    test_all(&c, z);
    *candidates = c.candidates;
    *r16 = c.r16;
    free(c.hits);
    return 0;
}

/* ------------------------------------------------------------------- CLI */
#ifdef HSS_ORACLE_MAIN
/* hss_oracle LIMIT FIRST LAST THREADS [--rows]
 * Prints one JSON object with the interval's logical pairs, processed
 * pairs, products, candidates, mod-16 survivors and hits (l m n area). */
int main(int argc, char **argv) {
    if (argc < 5 || argc > 6) {
        fprintf(stderr, "usage: hss_oracle LIMIT FIRST LAST THREADS [--rows]\n");
        return 2;
    }
    uint64_t n = strtoull(argv[1], NULL, 10), first = strtoull(argv[2], NULL, 10),
             last = strtoull(argv[3], NULL, 10);
    int threads = atoi(argv[4]);
    int rows_flag = argc == 6 && strcmp(argv[5], "--rows") == 0;
    if (!n || !first || first > last || last > n || threads < 1) return 2;
    void *t = hss_oracle_prepare(n);
    uint64_t rows = last - first + 1;
    uint64_t *cand = calloc(rows, 8), *prod = calloc(rows, 8), *proc = calloc(rows, 8),
             *r16 = calloc(rows, 8);
    hss_oracle_hit_t hits[64];
    uint32_t nh = 0;
    hss_oracle_search(t, first, last, threads, cand, prod, proc, r16, hits, 64, &nh);
    uint64_t pairs = 0, C = 0, P = 0, Q = 0, R = 0;
    for (uint64_t r = 0; r < rows; ++r) {
        pairs += n - (first + r) + 1;
        C += cand[r]; P += prod[r]; Q += proc[r]; R += r16[r];
    }
    printf("{\"limit\": %llu, \"first\": %llu, \"last\": %llu, \"pairs\": %llu, \"processed\": %llu, "
           "\"products\": %llu, \"candidates\": %llu, \"r16\": %llu, \"hits\": [",
           (unsigned long long)n, (unsigned long long)first, (unsigned long long)last,
           (unsigned long long)pairs, (unsigned long long)Q, (unsigned long long)P,
           (unsigned long long)C, (unsigned long long)R);
    for (uint32_t i = 0; i < nh && i < 64; ++i) {
        i128 a = ((i128)hits[i].area4_hi << 64) | hits[i].area4_lo;
        if (a < 0) a = -a;
        u128 area = (u128)a / 4;
        char buf[48];
        int pos = 47;
        buf[pos] = 0;
        do { buf[--pos] = (char)('0' + (int)(area % 10)); area /= 10; } while (area);
        printf("%s\"%llu %llu %llu %s\"", i ? ", " : "", (unsigned long long)hits[i].l,
               (unsigned long long)hits[i].m, (unsigned long long)hits[i].n, buf + pos);
    }
    printf("]");
    if (rows_flag) {
        printf(", \"row_candidates\": [");
        for (uint64_t r = 0; r < rows; ++r) printf("%s%llu", r ? ", " : "", (unsigned long long)cand[r]);
        printf("], \"row_products\": [");
        for (uint64_t r = 0; r < rows; ++r) printf("%s%llu", r ? ", " : "", (unsigned long long)prod[r]);
        printf("]");
    }
    printf("}\n");
    hss_oracle_release(t);
    free(cand); free(prod); free(proc); free(r16);
    return 0;
}
#endif
