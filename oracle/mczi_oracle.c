/*
 * mczi_oracle.c -- CPU restatement of the MC/ZI k-mer hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker for the GPU
 * library and the timed CPU baseline; it is never linked into, called by or
 * used as a fallback for the product path (mczi_gb300/ and libmczi_gpu.so).
 *
 * What it restates (reference file:line, paths inside the MCZI project):
 *  - FASTX -> maximal A/C/G/T fragments, split at any other byte, fragments
 *    shorter than the minimum length dropped: helicase `split_non_actg`
 *    as configured at src/lib.rs:3264-3308 (min_len = k) and src/zi.rs:203-221.
 *    helicase 0.1.1 is not vendored; the N-splitting behaviour is pinned by
 *    src/lib.rs:6070-6100 and src/zi.rs:315-330.  Lower-case a/c/g/t are
 *    treated as bases like MC's own `base_bits` (src/lib.rs:3030-3038).
 *  - MC base code A0 C1 G2 T3, MSB-first k-mer value, canonical = min(fwd, rc)
 *    by the rolling update of src/lib.rs:3589-3614 and src/zi.rs:224-238.
 *  - Abundance counting: exact counts, kept iff count > x
 *    (src/lib.rs:2400-2425, 2545-2570, 6027-6068).  The k <= 32 KFF writer
 *    stores min(count, x + 1, 255) in one byte (src/lib.rs:2489-2506).
 *  - fof dataset presence: each k-mer counted at most once per dataset, kept
 *    iff the number of datasets > x; empty when x >= #datasets
 *    (src/lib.rs:637-703, 2213-2247, 4450-4522).
 *  - ZI subtraction: canonical k-mers of query fragments (len >= k) absent
 *    from the set of canonical k-mers of the index fragments
 *    (src/zi.rs:114-175).  sshash-lib internals are not restated; only the
 *    membership answer is.
 *  - KFF bytes (src/lib.rs:1633-1670, 3071-3121) and the greedy simplitig
 *    FASTA writer (src/lib.rs:1469-1533, 1598-1631), byte for byte.
 *
 * The minimizer machinery of the reference is deliberately absent: the
 * (canonical k-mer, count) set MC emits equals exact counting over all
 * fragments because every window lands in exactly one partition.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef unsigned __int128 u128;

/* ------------------------------------------------------------------ */
/* base codes                                                           */
/* ------------------------------------------------------------------ */

static int8_t g_code[256];
static int g_code_ready = 0;

static void init_codes(void) {
    if (g_code_ready) return;
    for (int i = 0; i < 256; i++) g_code[i] = -1;
    g_code['A'] = 0; g_code['a'] = 0;
    g_code['C'] = 1; g_code['c'] = 1;
    g_code['G'] = 2; g_code['g'] = 2;
    g_code['T'] = 3; g_code['t'] = 3;
    g_code_ready = 1;
}

/* ------------------------------------------------------------------ */
/* FASTX fragment extraction                                            */
/* ------------------------------------------------------------------ */

typedef struct {
    uint8_t *codes;     /* concatenated fragment codes (0..3) */
    uint64_t n_codes;
    uint64_t cap_codes;
    uint64_t *frag_off; /* n_frag + 1 offsets into codes */
    uint64_t n_frag;
    uint64_t cap_frag;
} frags_t;

static void frags_push_code(frags_t *f, uint8_t c) {
    if (f->n_codes == f->cap_codes) {
        f->cap_codes = f->cap_codes ? f->cap_codes * 2 : 1024;
        f->codes = (uint8_t *)realloc(f->codes, f->cap_codes);
    }
    f->codes[f->n_codes++] = c;
}

static void frags_close(frags_t *f, uint64_t start, uint64_t min_len) {
    uint64_t len = f->n_codes - start;
    if (len == 0) return;
    if (len < min_len) { f->n_codes = start; return; }
    if (f->n_frag + 2 > f->cap_frag) {
        f->cap_frag = f->cap_frag ? f->cap_frag * 2 : 256;
        f->frag_off = (uint64_t *)realloc(f->frag_off, f->cap_frag * sizeof(uint64_t));
    }
    f->frag_off[f->n_frag] = start;
    f->n_frag++;
    f->frag_off[f->n_frag] = f->n_codes;
}

/* Returns 0 on success, 1 if the input does not start like a FASTX record
 * (the reference skips such inputs with MC_WARN, src/lib.rs:3371-3392). */
static int parse_fastx(const uint8_t *buf, uint64_t len, uint64_t min_len, frags_t *f) {
    init_codes();
    if (!f->frag_off) {
        f->cap_frag = 256;
        f->frag_off = (uint64_t *)malloc(f->cap_frag * sizeof(uint64_t));
        f->frag_off[0] = 0;
    }
    uint64_t p = 0;
    while (p < len && (buf[p] == '\n' || buf[p] == '\r')) p++;
    if (p >= len) return 0;
    int fastq;
    if (buf[p] == '>') fastq = 0;
    else if (buf[p] == '@') fastq = 1;
    else return 1;

    uint64_t start = f->n_codes;
    if (!fastq) {
        /* FASTA: header lines start with '>'; every other line is sequence */
        int at_line_start = 1, in_header = 0;
        for (; p < len; p++) {
            uint8_t c = buf[p];
            if (c == '\n') { at_line_start = 1; in_header = 0; continue; }
            if (at_line_start) {
                at_line_start = 0;
                if (c == '>') {
                    frags_close(f, start, min_len); start = f->n_codes;
                    in_header = 1; continue;
                }
            }
            if (in_header || c == '\r') continue;
            int8_t code = g_code[c];
            if (code < 0) { frags_close(f, start, min_len); start = f->n_codes; }
            else frags_push_code(f, (uint8_t)code);
        }
        frags_close(f, start, min_len);
    } else {
        /* FASTQ: four-line records, line 1 of each record is the sequence */
        uint64_t line = 0;
        for (; p < len; p++) {
            uint8_t c = buf[p];
            if (c == '\n') {
                if ((line & 3) == 1) { frags_close(f, start, min_len); start = f->n_codes; }
                line++;
                continue;
            }
            if ((line & 3) != 1 || c == '\r') continue;
            int8_t code = g_code[c];
            if (code < 0) { frags_close(f, start, min_len); start = f->n_codes; }
            else frags_push_code(f, (uint8_t)code);
        }
        frags_close(f, start, min_len);
    }
    return 0;
}

static void frags_free(frags_t *f) {
    free(f->codes); free(f->frag_off);
    memset(f, 0, sizeof(*f));
}

/* ------------------------------------------------------------------ */
/* open-addressing table: u128 key -> (u64 count, u32 last dataset)     */
/* ------------------------------------------------------------------ */

#define EMPTY_KEY (~(u128)0) /* never canonical: its reverse complement is 0 */

typedef struct {
    u128 *keys;
    uint64_t *counts;
    uint32_t *last;
    uint64_t cap, n;
} table_t;

static inline uint64_t mix64(uint64_t x) {
    x ^= x >> 33; x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ULL;
    return x ^ (x >> 33);
}

static inline uint64_t key_hash(u128 k) {
    return mix64((uint64_t)k ^ mix64((uint64_t)(k >> 64) + 0x9e3779b97f4a7c15ULL));
}

static void table_init(table_t *t, uint64_t cap) {
    uint64_t c = 64;
    while (c < cap) c <<= 1;
    t->cap = c; t->n = 0;
    t->keys = (u128 *)malloc(c * sizeof(u128));
    t->counts = (uint64_t *)calloc(c, sizeof(uint64_t));
    t->last = (uint32_t *)malloc(c * sizeof(uint32_t));
    for (uint64_t i = 0; i < c; i++) { t->keys[i] = EMPTY_KEY; t->last[i] = 0xffffffffu; }
}

static void table_free(table_t *t) {
    free(t->keys); free(t->counts); free(t->last);
    memset(t, 0, sizeof(*t));
}

static uint64_t table_slot(table_t *t, u128 key);

static void table_grow(table_t *t) {
    table_t nt;
    table_init(&nt, t->cap * 2);
    for (uint64_t i = 0; i < t->cap; i++) {
        if (t->keys[i] == EMPTY_KEY) continue;
        uint64_t s = table_slot(&nt, t->keys[i]);
        nt.keys[s] = t->keys[i];
        nt.counts[s] = t->counts[i];
        nt.last[s] = t->last[i];
        nt.n++;
    }
    table_free(t);
    *t = nt;
}

static uint64_t table_slot(table_t *t, u128 key) {
    uint64_t m = t->cap - 1, s = key_hash(key) & m;
    while (t->keys[s] != EMPTY_KEY && t->keys[s] != key) s = (s + 1) & m;
    return s;
}

/* abundance: count += 1 (saturating like Count::saturating_add) */
static void table_add(table_t *t, u128 key) {
    if ((t->n + 1) * 10 > t->cap * 7) table_grow(t);
    uint64_t s = table_slot(t, key);
    if (t->keys[s] == EMPTY_KEY) { t->keys[s] = key; t->n++; }
    if (t->counts[s] != UINT64_MAX) t->counts[s]++;
}

/* presence: count += 1 only for the first occurrence in dataset d */
static void table_add_presence(table_t *t, u128 key, uint32_t d) {
    if ((t->n + 1) * 10 > t->cap * 7) table_grow(t);
    uint64_t s = table_slot(t, key);
    if (t->keys[s] == EMPTY_KEY) { t->keys[s] = key; t->n++; }
    if (t->last[s] != d) { t->last[s] = d; t->counts[s]++; }
}

static int table_contains(const table_t *t, u128 key) {
    uint64_t m = t->cap - 1, s = key_hash(key) & m;
    while (t->keys[s] != EMPTY_KEY) {
        if (t->keys[s] == key) return 1;
        s = (s + 1) & m;
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* canonical k-mer enumeration                                          */
/* ------------------------------------------------------------------ */

static inline u128 kmer_mask(int k) {
    return k == 64 ? ~(u128)0 : (((u128)1 << (2 * k)) - 1);
}

/* Calls fn(ctx, canonical) for every window of every fragment. */
typedef void (*kmer_fn)(void *ctx, u128 canon);

static void for_each_kmer(const frags_t *f, uint64_t frag_lo, uint64_t frag_hi, int k,
                          kmer_fn fn, void *ctx) {
    const u128 mask = kmer_mask(k);
    const int hs = 2 * (k - 1);
    for (uint64_t fi = frag_lo; fi < frag_hi; fi++) {
        uint64_t a = f->frag_off[fi], b = f->frag_off[fi + 1];
        if (b - a < (uint64_t)k) continue;
        u128 fwd = 0, rev = 0;
        for (uint64_t i = a; i < b; i++) {
            u128 bits = f->codes[i];
            fwd = ((fwd << 2) | bits) & mask;
            rev = (rev >> 2) | ((bits ^ 3) << hs);
            if (i + 1 - a >= (uint64_t)k) fn(ctx, fwd < rev ? fwd : rev);
        }
    }
}

/* ------------------------------------------------------------------ */
/* results                                                              */
/* ------------------------------------------------------------------ */

typedef struct {
    u128 key;
    uint64_t count;
} rec_t;

typedef struct {
    rec_t *recs;
    uint64_t n;
    int status; /* 0 ok, <0 invalid config */
    uint64_t skipped_inputs;
} result_t;

static int rec_cmp(const void *a, const void *b) {
    u128 x = ((const rec_t *)a)->key, y = ((const rec_t *)b)->key;
    return x < y ? -1 : (x > y ? 1 : 0);
}

/* ------------------------------------------------------------------ */
/* sharded parallel counting                                            */
/* ------------------------------------------------------------------ */

typedef struct {
    u128 *v;
    uint64_t n, cap;
} vec_t;

static inline void vec_push(vec_t *v, u128 x) {
    if (v->n == v->cap) {
        v->cap = v->cap ? v->cap * 2 : 4096;
        v->v = (u128 *)realloc(v->v, v->cap * sizeof(u128));
    }
    v->v[v->n++] = x;
}

typedef struct {
    vec_t *shards;
    int n_shards;
} shard_ctx;

static void shard_push(void *c, u128 key) {
    shard_ctx *s = (shard_ctx *)c;
    vec_push(&s->shards[(key_hash(key) >> 32) % (uint64_t)s->n_shards], key);
}

/* Generates all canonical k-mers of `f` into per-thread, per-shard vectors. */
static vec_t *gen_sharded(const frags_t *f, int k, int threads, int n_shards) {
    vec_t *all = (vec_t *)calloc((size_t)threads * n_shards, sizeof(vec_t));
#pragma omp parallel num_threads(threads)
    {
        int t = 0, nt = 1;
#ifdef _OPENMP
        t = omp_get_thread_num(); nt = omp_get_num_threads();
#endif
        uint64_t lo = f->n_frag * (uint64_t)t / nt, hi = f->n_frag * (uint64_t)(t + 1) / nt;
        shard_ctx c = { all + (size_t)t * n_shards, n_shards };
        for_each_kmer(f, lo, hi, k, shard_push, &c);
    }
    return all;
}

/* mode 0: abundance, mode 1: dataset presence (one dataset per input). */
static result_t *count_impl(const uint8_t *const *bufs, const uint64_t *lens, int n_inputs,
                            int k, uint64_t x, int mode, int threads) {
    result_t *r = (result_t *)calloc(1, sizeof(result_t));
    if (k < 1 || k > 64 || n_inputs < 1) { r->status = -1; return r; }
    if (threads < 1) threads = 1;
    const int n_shards = threads * 4;
    table_t *tables = (table_t *)calloc(n_shards, sizeof(table_t));
    for (int s = 0; s < n_shards; s++) table_init(&tables[s], 1024);

    if (mode == 1 && x >= (uint64_t)n_inputs) goto collect; /* src/lib.rs:644-648 */

    if (mode == 0) {
        frags_t f = {0};
        for (int i = 0; i < n_inputs; i++)
            if (parse_fastx(bufs[i], lens[i], (uint64_t)k, &f)) r->skipped_inputs++;
        vec_t *all = gen_sharded(&f, k, threads, n_shards);
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1)
        for (int s = 0; s < n_shards; s++) {
            for (int t = 0; t < threads; t++) {
                vec_t *v = &all[(size_t)t * n_shards + s];
                for (uint64_t i = 0; i < v->n; i++) table_add(&tables[s], v->v[i]);
                free(v->v); v->v = NULL;
            }
        }
        free(all);
        frags_free(&f);
    } else {
        for (int d = 0; d < n_inputs; d++) {
            frags_t f = {0};
            if (parse_fastx(bufs[d], lens[d], (uint64_t)k, &f)) r->skipped_inputs++;
            vec_t *all = gen_sharded(&f, k, threads, n_shards);
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1)
            for (int s = 0; s < n_shards; s++) {
                for (int t = 0; t < threads; t++) {
                    vec_t *v = &all[(size_t)t * n_shards + s];
                    for (uint64_t i = 0; i < v->n; i++)
                        table_add_presence(&tables[s], v->v[i], (uint32_t)d);
                    free(v->v); v->v = NULL;
                }
            }
            free(all);
            frags_free(&f);
        }
    }

collect:;
    uint64_t total = 0;
    for (int s = 0; s < n_shards; s++)
        for (uint64_t i = 0; i < tables[s].cap; i++)
            if (tables[s].keys[i] != EMPTY_KEY && tables[s].counts[i] > x) total++;
    r->recs = (rec_t *)malloc((total ? total : 1) * sizeof(rec_t));
    for (int s = 0; s < n_shards; s++) {
        for (uint64_t i = 0; i < tables[s].cap; i++) {
            if (tables[s].keys[i] != EMPTY_KEY && tables[s].counts[i] > x) {
                r->recs[r->n].key = tables[s].keys[i];
                r->recs[r->n].count = tables[s].counts[i];
                r->n++;
            }
        }
        table_free(&tables[s]);
    }
    free(tables);
    qsort(r->recs, r->n, sizeof(rec_t), rec_cmp);
    return r;
}

/* ------------------------------------------------------------------ */
/* order-independent digest of a count's kept records                   */
/* ------------------------------------------------------------------ */

/* One kept record's digest word; the digest of a result is the record
 * count, the sum of the counts, and the wrapping sum and the xor of these
 * words, so it does not depend on record order. */
static inline uint64_t rec_digest(u128 key, uint64_t count) {
    return mix64(mix64(mix64((uint64_t)key) ^ (uint64_t)(key >> 64)) + count);
}

/* Pass of a key in the digest's hash-range passes: a mix of the key hash, so
 * that the keys of one pass spread over all table slots and shards. */
static inline int key_pass(uint64_t h, int passes) {
    return (int)(((mix64(h ^ 0x5851f42d4c957f2dULL) >> 32) * (uint64_t)passes) >> 32);
}

/* The canonical k-mers of fragments [lo, hi) that fall in pass `p`, pushed to
 * their shard vectors (the rolling update of for_each_kmer, inlined). */
static void gen_pass_range(const frags_t *f, uint64_t lo, uint64_t hi, int k, int p, int passes,
                           vec_t *shards, int n_shards, const table_t *index) {
    const u128 mask = kmer_mask(k);
    const int hs = 2 * (k - 1);
    for (uint64_t fi = lo; fi < hi; fi++) {
        uint64_t a = f->frag_off[fi], b = f->frag_off[fi + 1];
        if (b - a < (uint64_t)k) continue;
        u128 fwd = 0, rev = 0;
        for (uint64_t i = a; i < b; i++) {
            u128 bits = f->codes[i];
            fwd = ((fwd << 2) | bits) & mask;
            rev = (rev >> 2) | ((bits ^ 3) << hs);
            if (i + 1 - a < (uint64_t)k) continue;
            u128 c = fwd < rev ? fwd : rev;
            uint64_t h = key_hash(c);
            if (passes > 1 && key_pass(h, passes) != p) continue;
            uint64_t sh = (h >> 32) % (uint64_t)n_shards;
            if (index && table_contains(&index[sh], c)) continue; /* ZI: present in the index */
            vec_push(&shards[sh], c);
        }
    }
}

static void insert_pass(const frags_t *f, int k, int p, int passes, int threads, int n_shards,
                        table_t *tables, int presence, uint32_t d, const table_t *index) {
    vec_t *all = (vec_t *)calloc((size_t)threads * n_shards, sizeof(vec_t));
#pragma omp parallel num_threads(threads)
    {
        int t = 0, nt = 1;
#ifdef _OPENMP
        t = omp_get_thread_num(); nt = omp_get_num_threads();
#endif
        uint64_t lo = f->n_frag * (uint64_t)t / nt, hi = f->n_frag * (uint64_t)(t + 1) / nt;
        gen_pass_range(f, lo, hi, k, p, passes, all + (size_t)t * n_shards, n_shards, index);
    }
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1)
    for (int s = 0; s < n_shards; s++) {
        for (int t = 0; t < threads; t++) {
            vec_t *v = &all[(size_t)t * n_shards + s];
            for (uint64_t i = 0; i < v->n; i++) {
                if (presence) table_add_presence(&tables[s], v->v[i], d);
                else table_add(&tables[s], v->v[i]);
            }
            free(v->v); v->v = NULL;
        }
    }
    free(all);
}

/* Digest (out[0] records, out[1] sum of counts, out[2] wrapping sum and
 * out[3] xor of rec_digest) of the records with count > x that
 * oracle_count would return for the same arguments, computed in `passes`
 * passes over disjoint ranges of the k-mer hash so that memory stays bounded
 * (each pass re-enumerates every k-mer and keeps only its own range).
 * Returns 0, or -1 for an invalid configuration. */
int oracle_count_digest(const uint8_t *const *bufs, const uint64_t *lens, int n_inputs, int k, uint64_t x,
                        int mode, int threads, int passes, uint64_t *out, uint64_t *skipped) {
    out[0] = out[1] = out[2] = out[3] = 0;
    *skipped = 0;
    if (k < 1 || k > 64 || n_inputs < 1 || passes < 1) return -1;
    if (threads < 1) threads = 1;
    const int n_shards = threads * 4;
    frags_t all = {0};
    if (mode == 0) {
        for (int i = 0; i < n_inputs; i++)
            if (parse_fastx(bufs[i], lens[i], (uint64_t)k, &all)) (*skipped)++;
    } else {
        for (int i = 0; i < n_inputs; i++) {
            frags_t g = {0};
            if (parse_fastx(bufs[i], lens[i], (uint64_t)k, &g)) (*skipped)++;
            frags_free(&g);
        }
        if (x >= (uint64_t)n_inputs) return 0; /* src/lib.rs:644-648 */
    }
    uint64_t *part = (uint64_t *)calloc((size_t)n_shards * 4, sizeof(uint64_t));
    for (int p = 0; p < passes; p++) {
        table_t *tables = (table_t *)calloc(n_shards, sizeof(table_t));
        for (int s = 0; s < n_shards; s++) table_init(&tables[s], 1024);
        if (mode == 0) {
            insert_pass(&all, k, p, passes, threads, n_shards, tables, 0, 0, NULL);
        } else {
            for (int d = 0; d < n_inputs; d++) {
                frags_t g = {0};
                parse_fastx(bufs[d], lens[d], (uint64_t)k, &g);
                insert_pass(&g, k, p, passes, threads, n_shards, tables, 1, (uint32_t)d, NULL);
                frags_free(&g);
            }
        }
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1)
        for (int s = 0; s < n_shards; s++) {
            uint64_t *q = part + (size_t)s * 4;
            for (uint64_t i = 0; i < tables[s].cap; i++) {
                if (tables[s].keys[i] == EMPTY_KEY || tables[s].counts[i] <= x) continue;
                uint64_t w = rec_digest(tables[s].keys[i], tables[s].counts[i]);
                q[0]++; q[1] += tables[s].counts[i]; q[2] += w; q[3] ^= w;
            }
            table_free(&tables[s]);
        }
        free(tables);
    }
    for (int s = 0; s < n_shards; s++) {
        out[0] += part[s * 4]; out[1] += part[s * 4 + 1]; out[2] += part[s * 4 + 2]; out[3] ^= part[s * 4 + 3];
    }
    free(part);
    frags_free(&all);
    return 0;
}

/* Digest of the ZI absent set that oracle_zi_absent would return (each
 * record with count 1), in `passes` hash-range passes over the queries; the
 * index set is built once, sharded like the passes' tables.  Returns 0, or -1
 * for an invalid k. */
int oracle_zi_absent_digest(const uint8_t *index_buf, uint64_t index_len, const uint8_t *const *qbufs,
                            const uint64_t *qlens, int n_queries, int k, int threads, int passes, uint64_t *out) {
    out[0] = out[1] = out[2] = out[3] = 0;
    if (k < 1 || k > 64 || passes < 1) return -1;
    if (threads < 1) threads = 1;
    const int n_shards = threads * 4;
    table_t *index = (table_t *)calloc(n_shards, sizeof(table_t));
    for (int s = 0; s < n_shards; s++) table_init(&index[s], 1024);
    frags_t fi = {0};
    parse_fastx(index_buf, index_len, 1, &fi); /* sequences of any length; only those >= k give k-mers */
    insert_pass(&fi, k, 0, 1, threads, n_shards, index, 0, 0, NULL);
    frags_free(&fi);
    frags_t q = {0};
    for (int i = 0; i < n_queries; i++) parse_fastx(qbufs[i], qlens[i], (uint64_t)k, &q);
    uint64_t *part = (uint64_t *)calloc((size_t)n_shards * 4, sizeof(uint64_t));
    for (int p = 0; p < passes; p++) {
        table_t *tables = (table_t *)calloc(n_shards, sizeof(table_t));
        for (int s = 0; s < n_shards; s++) table_init(&tables[s], 1024);
        insert_pass(&q, k, p, passes, threads, n_shards, tables, 0, 0, index);
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1)
        for (int s = 0; s < n_shards; s++) {
            uint64_t *o = part + (size_t)s * 4;
            for (uint64_t i = 0; i < tables[s].cap; i++) {
                if (tables[s].keys[i] == EMPTY_KEY) continue;
                uint64_t w = rec_digest(tables[s].keys[i], 1);
                o[0]++; o[1] += 1; o[2] += w; o[3] ^= w;
            }
            table_free(&tables[s]);
        }
        free(tables);
    }
    for (int s = 0; s < n_shards; s++) {
        out[0] += part[s * 4]; out[1] += part[s * 4 + 1]; out[2] += part[s * 4 + 2]; out[3] ^= part[s * 4 + 3];
        table_free(&index[s]);
    }
    free(part);
    free(index);
    frags_free(&q);
    return 0;
}

/* Digest of given records with the same definition (for checking a result
 * copied from elsewhere against oracle_count_digest). */
void oracle_records_digest(const uint64_t *key_lo, const uint64_t *key_hi, const uint64_t *counts, uint64_t n,
                           uint64_t *out) {
    out[0] = out[1] = out[2] = out[3] = 0;
    for (uint64_t i = 0; i < n; i++) {
        u128 key = ((u128)(key_hi ? key_hi[i] : 0) << 64) | key_lo[i];
        uint64_t w = rec_digest(key, counts[i]);
        out[0]++; out[1] += counts[i]; out[2] += w; out[3] ^= w;
    }
}

/* ------------------------------------------------------------------ */
/* exported API (ctypes)                                                */
/* ------------------------------------------------------------------ */

/* Abundance (mode 0) or fof presence (mode 1) counting; records with
 * count > x, sorted by canonical k-mer. */
void *oracle_count(const uint8_t *const *bufs, const uint64_t *lens, int n_inputs, int k,
                   uint64_t x, int mode, int threads) {
    return count_impl(bufs, lens, n_inputs, k, x, mode, threads);
}

typedef struct {
    table_t *t;
    const uint8_t *unused;
} set_ctx;

static void set_insert(void *c, u128 key) { table_add((table_t *)c, key); }

typedef struct {
    const table_t *index;
    table_t *absent;
} absent_ctx;

static void absent_probe(void *c, u128 key) {
    absent_ctx *a = (absent_ctx *)c;
    if (!table_contains(a->index, key)) table_add(a->absent, key);
}

/* ZI: canonical query k-mers absent from the index, sorted; count = the
 * k-mer's absent occurrences in the queries (the sum over the set is MCZI's
 * not_filtered_kmers, src/mczi.rs:1661-1720, 1895-1914). */
void *oracle_zi_absent(const uint8_t *index_buf, uint64_t index_len,
                       const uint8_t *const *qbufs, const uint64_t *qlens, int n_queries, int k) {
    result_t *r = (result_t *)calloc(1, sizeof(result_t));
    if (k < 1 || k > 64) { r->status = -1; return r; }
    table_t index, absent;
    table_init(&index, 1024);
    table_init(&absent, 1024);
    frags_t f = {0};
    /* the index keeps sequences of length >= 1 (src/zi.rs:143-150); only
     * those of length >= k contribute k-mers */
    if (parse_fastx(index_buf, index_len, 1, &f)) r->skipped_inputs++;
    for_each_kmer(&f, 0, f.n_frag, k, set_insert, &index);
    frags_free(&f);
    for (int q = 0; q < n_queries; q++) {
        frags_t g = {0};
        if (parse_fastx(qbufs[q], qlens[q], (uint64_t)k, &g)) r->skipped_inputs++;
        absent_ctx a = { &index, &absent };
        for_each_kmer(&g, 0, g.n_frag, k, absent_probe, &a);
        frags_free(&g);
    }
    r->recs = (rec_t *)malloc((absent.n ? absent.n : 1) * sizeof(rec_t));
    for (uint64_t i = 0; i < absent.cap; i++) {
        if (absent.keys[i] == EMPTY_KEY) continue;
        r->recs[r->n].key = absent.keys[i];
        r->recs[r->n].count = absent.counts[i];
        r->n++;
    }
    qsort(r->recs, r->n, sizeof(rec_t), rec_cmp);
    table_free(&index);
    table_free(&absent);
    return r;
}

int oracle_result_status(const void *h) { return ((const result_t *)h)->status; }
uint64_t oracle_result_len(const void *h) { return ((const result_t *)h)->n; }
uint64_t oracle_result_skipped(const void *h) { return ((const result_t *)h)->skipped_inputs; }

void oracle_result_copy(const void *h, uint64_t *key_lo, uint64_t *key_hi, uint64_t *counts) {
    const result_t *r = (const result_t *)h;
    for (uint64_t i = 0; i < r->n; i++) {
        key_lo[i] = (uint64_t)r->recs[i].key;
        key_hi[i] = (uint64_t)(r->recs[i].key >> 64);
        counts[i] = r->recs[i].count;
    }
}

void oracle_result_free(void *h) {
    result_t *r = (result_t *)h;
    if (!r) return;
    free(r->recs);
    free(r);
}

/* Fragment extraction, exported for packer parity: writes the fragment
 * codes (one byte per base, 0..3) and n_frag + 1 offsets.  Call with NULL
 * outputs to query sizes. */
int oracle_fragments(const uint8_t *buf, uint64_t len, uint64_t min_len, uint8_t *codes,
                     uint64_t *offsets, uint64_t *n_codes, uint64_t *n_frag) {
    frags_t f = {0};
    int skipped = parse_fastx(buf, len, min_len, &f);
    if (codes) memcpy(codes, f.codes, f.n_codes);
    if (offsets) {
        if (f.n_frag) memcpy(offsets, f.frag_off, (f.n_frag + 1) * sizeof(uint64_t));
        else offsets[0] = 0;
    }
    *n_codes = f.n_codes;
    *n_frag = f.n_frag;
    frags_free(&f);
    return skipped;
}

/* ------------------------------------------------------------------ */
/* writers: KFF and simplitig FASTA                                     */
/* ------------------------------------------------------------------ */

static void put_u32(FILE *o, uint32_t v) {
    uint8_t b[4] = { (uint8_t)(v >> 24), (uint8_t)(v >> 16), (uint8_t)(v >> 8), (uint8_t)v };
    fwrite(b, 1, 4, o);
}

static void put_u64(FILE *o, uint64_t v) {
    uint8_t b[8];
    for (int i = 0; i < 8; i++) b[i] = (uint8_t)(v >> (56 - 8 * i));
    fwrite(b, 1, 8, o);
}

/* KFF file: count_size 1 (k <= 32 abundance, counts saturated at
 * min(x + 1, 255)), 4 (fof presence, u32) or 8 (k > 32 abundance, u64). */
int oracle_write_kff(const char *path, const uint64_t *key_lo, const uint64_t *key_hi,
                     const uint64_t *counts, uint64_t n, int k, int m, uint64_t x,
                     int count_size) {
    FILE *o = fopen(path, "wb");
    if (!o) return -1;
    char fb[512];
    int fbl = snprintf(fb, sizeof fb,
                       "producer=MC\nk=%d\nm=%d\nthreshold=%llu\nfilter=count>threshold\ncanonical=1\n",
                       k, m, (unsigned long long)x);
    fwrite("KFF", 1, 3, o);
    uint8_t ver[5] = { 1, 0, 0x1b, 1, 1 };
    fwrite(ver, 1, 5, o);
    put_u32(o, (uint32_t)fbl);
    fwrite(fb, 1, (size_t)fbl, o);
    const char *names[6] = { "k", "max", "data_size", "ordered", "m", "threshold" };
    uint64_t vals[6] = { (uint64_t)k, 1, (uint64_t)count_size, 0, (uint64_t)m, x };
    fwrite("v", 1, 1, o);
    put_u64(o, 6);
    for (int i = 0; i < 6; i++) {
        fwrite(names[i], 1, strlen(names[i]) + 1, o);
        put_u64(o, vals[i]);
    }
    fwrite("r", 1, 1, o);
    put_u64(o, n);
    const int nb = (k + 3) / 4;
    const uint64_t sat = (x + 1) < 255 ? (x + 1) : 255;
    for (uint64_t i = 0; i < n; i++) {
        uint8_t be[16];
        for (int j = 0; j < 8; j++) {
            be[j] = (uint8_t)(key_hi[i] >> (56 - 8 * j));
            be[8 + j] = (uint8_t)(key_lo[i] >> (56 - 8 * j));
        }
        fwrite(be + 16 - nb, 1, (size_t)nb, o);
        if (count_size == 1) {
            uint8_t c = (uint8_t)(counts[i] < sat ? counts[i] : sat);
            fwrite(&c, 1, 1, o);
        } else if (count_size == 4) {
            put_u32(o, (uint32_t)counts[i]);
        } else {
            put_u64(o, counts[i]);
        }
    }
    fwrite("KFF", 1, 3, o);
    fclose(o);
    return 0;
}

static const char BASES[4] = { 'A', 'C', 'G', 'T' };

static int base_code(char b) {
    switch (b) { case 'A': return 0; case 'C': return 1; case 'G': return 2; default: return 3; }
}

static char complement(char b) {
    switch (b) { case 'A': return 'T'; case 'C': return 'G'; case 'G': return 'C'; default: return 'A'; }
}

static void revcomp(char *s, uint64_t n) {
    for (uint64_t i = 0; i < n / 2; i++) {
        char l = complement(s[i]), r = complement(s[n - 1 - i]);
        s[i] = r; s[n - 1 - i] = l;
    }
    if (n & 1) s[n / 2] = complement(s[n / 2]);
}

/* canonical k-mer of the last k-1 bases of seq followed by `base`
 * (src/lib.rs:1559-1581) */
static u128 suffix_extension(const char *seq, uint64_t len, int k, char base) {
    const u128 mask = kmer_mask(k);
    const int hs = 2 * (k - 1);
    u128 fwd = 0, rev = 0;
    for (uint64_t i = len - (uint64_t)(k - 1); i < len; i++) {
        u128 b = (u128)base_code(seq[i]);
        fwd = ((fwd << 2) | b) & mask;
        rev = (rev >> 2) | ((b ^ 3) << hs);
    }
    u128 b = (u128)base_code(base);
    fwd = ((fwd << 2) | b) & mask;
    rev = (rev >> 2) | ((b ^ 3) << hs);
    return fwd < rev ? fwd : rev;
}

static int table_remove(table_t *t, u128 key) {
    /* tombstone-free deletion by backward shift */
    uint64_t m = t->cap - 1, s = key_hash(key) & m;
    while (t->keys[s] != EMPTY_KEY && t->keys[s] != key) s = (s + 1) & m;
    if (t->keys[s] == EMPTY_KEY) return 0;
    uint64_t hole = s, j = s;
    for (;;) {
        j = (j + 1) & m;
        if (t->keys[j] == EMPTY_KEY) break;
        uint64_t home = key_hash(t->keys[j]) & m;
        /* move j into hole if home is not in (hole, j] cyclically */
        int in_range = hole <= j ? (home > hole && home <= j) : (home > hole || home <= j);
        if (!in_range) {
            t->keys[hole] = t->keys[j];
            t->counts[hole] = t->counts[j];
            t->last[hole] = t->last[j];
            hole = j;
        }
    }
    t->keys[hole] = EMPTY_KEY;
    t->counts[hole] = 0;
    t->n--;
    return 1;
}

static void extend_forward(char **seq, uint64_t *len, uint64_t *cap, int k, table_t *rem) {
    for (;;) {
        int extended = 0;
        for (int bi = 0; bi < 4; bi++) {
            u128 e = suffix_extension(*seq, *len, k, BASES[bi]);
            if (table_remove(rem, e)) {
                if (*len + 1 >= *cap) { *cap *= 2; *seq = (char *)realloc(*seq, *cap); }
                (*seq)[(*len)++] = BASES[bi];
                extended = 1;
                break;
            }
        }
        if (!extended) return;
    }
}

static int u128_cmp(const void *a, const void *b) {
    u128 x = *(const u128 *)a, y = *(const u128 *)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

/* Greedy simplitig FASTA (src/lib.rs:1469-1533): seeds in ascending order,
 * extend forward with A,C,G,T priority, reverse-complement, extend again,
 * reverse-complement back; ">MC_simplitig_<i> kmers=<n>", 80-column lines.
 * `first_index` is the index of the last record already written. */
int64_t oracle_write_simplitigs(const char *path, const uint64_t *key_lo, const uint64_t *key_hi,
                                uint64_t n, int k, uint64_t first_index) {
    FILE *o = fopen(path, "wb");
    if (!o) return -1;
    table_t rem;
    table_init(&rem, n * 2 + 64);
    u128 *seeds = (u128 *)malloc((n ? n : 1) * sizeof(u128));
    uint64_t ns = 0;
    for (uint64_t i = 0; i < n; i++) {
        u128 key = ((u128)key_hi[i] << 64) | key_lo[i];
        uint64_t s = table_slot(&rem, key);
        if (rem.keys[s] == EMPTY_KEY) { rem.keys[s] = key; rem.n++; seeds[ns++] = key; }
    }
    qsort(seeds, ns, sizeof(u128), u128_cmp);
    uint64_t cap = 256;
    char *seq = (char *)malloc(cap);
    uint64_t idx = first_index;
    for (uint64_t si = 0; si < ns; si++) {
        if (!table_remove(&rem, seeds[si])) continue;
        uint64_t len = (uint64_t)k;
        if (cap <= len + 1) { cap = len * 2 + 2; seq = (char *)realloc(seq, cap); }
        for (int j = 0; j < k; j++) seq[j] = BASES[(seeds[si] >> (2 * (k - 1 - j))) & 3];
        extend_forward(&seq, &len, &cap, k, &rem);
        revcomp(seq, len);
        extend_forward(&seq, &len, &cap, k, &rem);
        revcomp(seq, len);
        idx++;
        fprintf(o, ">MC_simplitig_%llu kmers=%llu\n", (unsigned long long)idx,
                (unsigned long long)(len - (uint64_t)k + 1));
        for (uint64_t p = 0; p < len; p += 80) {
            uint64_t l = len - p < 80 ? len - p : 80;
            fwrite(seq + p, 1, l, o);
            fputc('\n', o);
        }
    }
    free(seq);
    free(seeds);
    table_free(&rem);
    fclose(o);
    return (int64_t)idx;
}
