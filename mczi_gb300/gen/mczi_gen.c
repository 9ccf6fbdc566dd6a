/*
 * mczi_gen.c -- deterministic synthetic FASTA workloads for MC and ZI.
 *
 * SplitMix64 streams as in the reference read simulators
 * (bench/simulate_reads_from_genome.rs:14-35); genomes are i.i.d. uniform
 * A/C/G/T, 2 bits per draw (bench/simulate_long_reads.rs:166-180).  Reads are
 * taken at uniform positions and reverse-complemented with probability 1/2.
 * Errors are drawn per output base: substitution (to one of the three other
 * bases), insertion (a random base, genome not advanced) or deletion (one
 * genome base skipped).  Read lengths are fixed or log-normal; the normal
 * deviate is an Irwin-Hall sum and exp() is computed by plain arithmetic so
 * that x86_64 and aarch64 produce identical bytes (build with
 * -ffp-contract=off).
 *
 * Output FASTA: one line per read, headers ">r<i>".
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static inline uint64_t splitmix_next(uint64_t *s) {
    *s += 0x9E3779B97F4A7C15ULL;
    uint64_t z = *s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

static const char ACGT[4] = { 'A', 'C', 'G', 'T' };

static inline char comp(char b) {
    switch (b) { case 'A': return 'T'; case 'C': return 'G'; case 'G': return 'C'; default: return 'A'; }
}

/* Uniform random genome of `len` ASCII bases; parallel over 1 Mbp blocks,
 * each block seeded from (seed, block index). */
void gen_genome(uint64_t seed, uint64_t len, uint8_t *out, int threads) {
    const uint64_t block = 1u << 20;
    int64_t nblocks = (int64_t)((len + block - 1) / block);
#pragma omp parallel for num_threads(threads > 0 ? threads : 1) schedule(static)
    for (int64_t b = 0; b < nblocks; b++) {
        uint64_t s = seed ^ (0xA0761D6478BD642FULL * (uint64_t)(b + 1));
        uint64_t lo = (uint64_t)b * block, hi = lo + block < len ? lo + block : len;
        uint64_t r = 0;
        int left = 0;
        for (uint64_t i = lo; i < hi; i++) {
            if (left == 0) { r = splitmix_next(&s); left = 32; }
            out[i] = (uint8_t)ACGT[r & 3];
            r >>= 2;
            left--;
        }
    }
}

/* Overwrites the genome with `copies` copies of each of `n_segments` random
 * segments of `seg_len` bases, placed in disjoint equally spaced slots with a
 * seeded jitter. */
void gen_insert_repeats(uint8_t *genome, uint64_t len, uint64_t seed, int n_segments,
                        int seg_len, int copies) {
    uint64_t s = seed;
    uint64_t slots = (uint64_t)n_segments * (uint64_t)copies;
    if (slots == 0 || (uint64_t)seg_len * slots > len) return;
    uint64_t stride = len / slots;
    uint8_t *seg = (uint8_t *)malloc((size_t)seg_len);
    for (int si = 0; si < n_segments; si++) {
        for (int j = 0; j < seg_len; j++) seg[j] = (uint8_t)ACGT[splitmix_next(&s) & 3];
        for (int c = 0; c < copies; c++) {
            uint64_t slot = (uint64_t)c * (uint64_t)n_segments + (uint64_t)si;
            uint64_t room = stride - (uint64_t)seg_len;
            uint64_t pos = slot * stride + (room ? splitmix_next(&s) % room : 0);
            memcpy(genome + pos, seg, (size_t)seg_len);
        }
    }
    free(seg);
}

/* Copy of `genome` with a fraction `rate` of positions substituted. */
void gen_variant(const uint8_t *genome, uint64_t len, uint64_t seed, double rate, uint8_t *out) {
    memcpy(out, genome, (size_t)len);
    uint64_t s = seed;
    uint64_t n = (uint64_t)((double)len * rate);
    for (uint64_t i = 0; i < n; i++) {
        uint64_t pos = splitmix_next(&s) % len;
        uint64_t r = splitmix_next(&s);
        char b = (char)out[pos];
        char nb;
        do { nb = ACGT[r & 3]; r >>= 2; } while (nb == b && r);
        if (nb == b) nb = comp(b);
        out[pos] = (uint8_t)nb;
    }
}

static double exp_arith(double x) {
    /* exp(x) = (exp(x / 1024))^1024, inner by a 7-term Taylor series */
    double y = x / 1024.0, t = 1.0, sum = 1.0;
    for (int i = 1; i <= 7; i++) { t = t * y / (double)i; sum += t; }
    for (int i = 0; i < 10; i++) sum = sum * sum;
    return sum;
}

static double normal_irwin_hall(uint64_t *s) {
    double acc = 0.0;
    for (int i = 0; i < 12; i++) acc += (double)(splitmix_next(s) >> 11) * (1.0 / 9007199254740992.0);
    return acc - 6.0;
}

static int digits(uint64_t v) {
    int d = 1;
    while (v >= 10) { v /= 10; d++; }
    return d;
}

typedef struct {
    uint64_t n;
    uint32_t *len;
    uint64_t *pos;
    uint8_t *rc;
    uint64_t *seed;
    uint64_t *off;
    uint64_t bytes;
} layout_t;

static void make_layout(layout_t *L, uint64_t glen, uint64_t seed, uint64_t total_bases, int len_mode,
                        double len_param, double sigma, int min_len, int max_len, double p_del) {
    uint64_t s = seed;
    uint64_t cap = 1024, n = 0, acc = 0;
    L->len = (uint32_t *)malloc(cap * sizeof(uint32_t));
    L->pos = (uint64_t *)malloc(cap * sizeof(uint64_t));
    L->rc = (uint8_t *)malloc(cap);
    L->seed = (uint64_t *)malloc(cap * sizeof(uint64_t));
    while (acc < total_bases) {
        if (n == cap) {
            cap *= 2;
            L->len = (uint32_t *)realloc(L->len, cap * sizeof(uint32_t));
            L->pos = (uint64_t *)realloc(L->pos, cap * sizeof(uint64_t));
            L->rc = (uint8_t *)realloc(L->rc, cap);
            L->seed = (uint64_t *)realloc(L->seed, cap * sizeof(uint64_t));
        }
        uint64_t l;
        if (len_mode == 0) {
            l = (uint64_t)len_param;
        } else {
            double v = len_param * exp_arith(sigma * normal_irwin_hall(&s));
            l = (uint64_t)(v + 0.5);
            if (l < (uint64_t)min_len) l = (uint64_t)min_len;
            if (l > (uint64_t)max_len) l = (uint64_t)max_len;
        }
        /* genome span consumed: allow for deletions with a margin */
        uint64_t span = l + (uint64_t)((double)l * p_del * 4.0) + 64;
        if (span > glen) span = glen;
        if (l > glen) l = glen;
        uint64_t room = glen - span + 1;
        L->len[n] = (uint32_t)l;
        L->pos[n] = splitmix_next(&s) % room;
        L->rc[n] = (uint8_t)(splitmix_next(&s) & 1);
        L->seed[n] = splitmix_next(&s);
        acc += l;
        n++;
    }
    L->n = n;
    L->off = (uint64_t *)malloc((n + 1) * sizeof(uint64_t));
    uint64_t b = 0;
    for (uint64_t i = 0; i < n; i++) {
        L->off[i] = b;
        b += 2 + (uint64_t)digits(i) + 1 + L->len[i] + 1; /* ">r" i "\n" seq "\n" */
    }
    L->off[n] = b;
    L->bytes = b;
}

static void free_layout(layout_t *L) {
    free(L->len); free(L->pos); free(L->rc); free(L->seed); free(L->off);
}

/* Writes reads as FASTA into `out` (capacity `cap`).  Returns the number of
 * bytes the output needs; writes nothing when out == NULL or cap is short.
 * len_mode 0: fixed length len_param; 1: log-normal with median len_param and
 * shape sigma, clipped to [min_len, max_len]. */
uint64_t gen_reads_fasta(const uint8_t *genome, uint64_t glen, uint64_t seed, uint64_t total_bases,
                         int len_mode, double len_param, double sigma, int min_len, int max_len,
                         double p_sub, double p_ins, double p_del, int threads, uint8_t *out,
                         uint64_t cap, uint64_t *n_reads) {
    layout_t L;
    make_layout(&L, glen, seed, total_bases, len_mode, len_param, sigma, min_len, max_len, p_del);
    uint64_t bytes = L.bytes;
    if (n_reads) *n_reads = L.n;
    if (out && cap >= bytes) {
        const uint32_t t_sub = (uint32_t)(p_sub * 4294967296.0);
        const uint32_t t_ins = t_sub + (uint32_t)(p_ins * 4294967296.0);
        const uint32_t t_del = t_ins + (uint32_t)(p_del * 4294967296.0);
#pragma omp parallel for num_threads(threads > 0 ? threads : 1) schedule(dynamic, 256)
        for (int64_t i = 0; i < (int64_t)L.n; i++) {
            uint8_t *o = out + L.off[i];
            int h = 0;
            o[h++] = '>';
            o[h++] = 'r';
            int d = digits((uint64_t)i);
            uint64_t v = (uint64_t)i;
            for (int j = d - 1; j >= 0; j--) { o[h + j] = (uint8_t)('0' + v % 10); v /= 10; }
            h += d;
            o[h++] = '\n';
            uint8_t *q = o + h;
            uint64_t s = L.seed[i];
            uint64_t g = L.pos[i];
            uint32_t l = L.len[i];
            for (uint32_t j = 0; j < l; j++) {
                uint64_t r = splitmix_next(&s);
                uint32_t u = (uint32_t)r;
                uint32_t alt = (uint32_t)(r >> 32);
                char b;
                if (g >= glen) g = glen - 1;
                if (u < t_sub) {
                    char orig = (char)genome[g++];
                    b = ACGT[alt & 3];
                    if (b == orig) b = ACGT[((alt & 3) + 1 + ((alt >> 2) % 3)) & 3];
                } else if (u < t_ins) {
                    b = ACGT[alt & 3];
                } else if (u < t_del) {
                    g++;
                    if (g >= glen) g = glen - 1;
                    b = (char)genome[g++];
                } else {
                    b = (char)genome[g++];
                }
                q[j] = (uint8_t)b;
            }
            if (L.rc[i]) {
                for (uint32_t a = 0, z = l ? l - 1 : 0; a < z; a++, z--) {
                    char x = comp((char)q[a]), y = comp((char)q[z]);
                    q[a] = (uint8_t)y; q[z] = (uint8_t)x;
                }
                if (l & 1) q[l / 2] = (uint8_t)comp((char)q[l / 2]);
            }
            q[l] = '\n';
        }
    }
    free_layout(&L);
    return bytes;
}

/* Genome as FASTA records of `chunk` bases overlapping by `overlap` bases
 * (the k-mer set of the chunks equals that of the genome when
 * overlap = k - 1).  Returns bytes needed; writes when out != NULL and cap
 * suffices. */
uint64_t gen_chunked_fasta(const uint8_t *genome, uint64_t glen, uint64_t chunk, uint64_t overlap,
                           uint8_t *out, uint64_t cap) {
    if (chunk <= overlap) return 0;
    uint64_t step = chunk - overlap, b = 0, i = 0;
    for (uint64_t p = 0; p < glen; p += step, i++) {
        uint64_t l = p + chunk < glen ? chunk : glen - p;
        b += 2 + (uint64_t)digits(i) + 1 + l + 1;
        if (p + chunk >= glen) break;
    }
    if (!out || cap < b) return b;
    uint64_t w = 0;
    i = 0;
    for (uint64_t p = 0; p < glen; p += step, i++) {
        uint64_t l = p + chunk < glen ? chunk : glen - p;
        out[w++] = '>';
        out[w++] = 'g';
        int d = digits(i);
        uint64_t v = i;
        for (int j = d - 1; j >= 0; j--) { out[w + (uint64_t)j] = (uint8_t)('0' + v % 10); v /= 10; }
        w += (uint64_t)d;
        out[w++] = '\n';
        memcpy(out + w, genome + p, (size_t)l);
        w += l;
        out[w++] = '\n';
        if (p + chunk >= glen) break;
    }
    return b;
}

/* Fingerprint of a byte buffer (to tell whether two machines generated the
 * same workload): every 1 MiB block is folded 8 bytes at a time by a
 * rotate-xor-multiply chain seeded with its block index, and the blocks'
 * mixed values are summed, so the result depends on every byte and its
 * position and the blocks can be hashed in parallel. */
static inline uint64_t fp_mix(uint64_t x) {
    x ^= x >> 33; x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ULL;
    return x ^ (x >> 33);
}

uint64_t gen_fingerprint(const uint8_t *buf, uint64_t len, int threads) {
    const uint64_t block = 1u << 20;
    int64_t nblocks = (int64_t)((len + block - 1) / block);
    uint64_t total = 0;
#pragma omp parallel for num_threads(threads > 0 ? threads : 1) schedule(static) reduction(+ : total)
    for (int64_t b = 0; b < nblocks; b++) {
        uint64_t lo = (uint64_t)b * block, hi = lo + block < len ? lo + block : len;
        uint64_t h = fp_mix((uint64_t)b + 1), i = lo;
        for (; i + 8 <= hi; i += 8) {
            uint64_t w;
            memcpy(&w, buf + i, 8);
            h ^= w;
            h = ((h << 29) | (h >> 35)) * 0x9E3779B97F4A7C15ULL;
        }
        for (; i < hi; i++) h = (h ^ buf[i]) * 0x100000001B3ULL;
        total += fp_mix(h ^ (hi - lo));
    }
    return total ^ fp_mix(len);
}
