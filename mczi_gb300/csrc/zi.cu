// zi.cu -- ZI on the GPU: a device-resident SSHash-style dictionary of the
// index k-mers and a streamed probe of query k-mers.
//
// Replaces ZI's build_dictionary (src/zi.rs:114-141, sshash-lib
// DictionaryBuilder::build_from_sequences) and its query loop
// collect_query_kmers_absent_from_index (src/zi.rs:152-175: per window
// `lookup(window).is_found()`, absent canonical k-mers into a set).
//
// Dictionary (all in HBM):
//   * the index's 2-bit stream, exactly as K1 packs it;
//   * its superkmers (K2), grouped into buckets by minimizer;
//   * an MPHF over the distinct minimizer keys, BBHash-style (Limasset et
//     al., "Fast and scalable minimal perfect hashing for massive key sets",
//     SEA 2017): level l keeps a bit array of gamma * (keys left) bits; a key
//     whose hashed position is hit by no other key owns that bit, the rest
//     retry at level l + 1; the index of a key is the rank of its bit;
//   * bucket offsets (CSR) from MPHF index to superkmer list.
// Membership of a query k-mer: its superkmer's minimizer key -> MPHF ->
// bucket -> compare against the canonical k-mers of the bucket's superkmers.
// The minimizer value is a function of the canonical k-mer (both strands hold
// the same canonical m-mers), so a present k-mer always finds its index
// superkmer in that bucket; a key outside the MPHF's set lands in an
// arbitrary bucket (whose stored key differs: all its windows are absent) or
// none.  sshash-lib's own layout is not reproduced; only its answers are.
//
// Streaming: one lookup per query superkmer (consecutive windows share the
// minimizer), like sshash's streaming query.  Absent windows are emitted as
// run descriptors, expanded once into (k-mer, input) records bucketed by
// k-mer hash, and deduplicated per bucket in shared memory (zi_dedup).
#include "api_internal.h"
#include "host_io.h"
#include "mczi_common.cuh"
#include "scan.cuh"

#include <cooperative_groups.h>
#include <cooperative_groups/reduce.h>

#include <algorithm>
#include <cstring>
#include <vector>

namespace mczi {

namespace {

constexpr int ZI_THREADS = 256;
constexpr uint64_t MPHF_NOT_FOUND = ~0ull;
constexpr int Q_CHUNK = 8;

// Blocked Bloom filter over the index's minimizer keys: three bits of one
// 64-bit word per key, about 32 bits per key.  Most minimizers of foreign
// reads fail it with one load (usually from L2) instead of walking the MPHF
// levels and the bucket's stored key, all random accesses.
__host__ __device__ __forceinline__ uint64_t mfilter_hash(uint32_t key) {
  uint64_t x = (uint64_t)key * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
  x ^= x >> 31;
  x *= 0xBF58476D1CE4E5B9ull;
  return x ^ (x >> 29);
}
__device__ __forceinline__ unsigned long long mfilter_bits(uint64_t h) {
  return (1ull << (h & 63)) | (1ull << ((h >> 6) & 63)) | (1ull << ((h >> 12) & 63));
}

__global__ void k_zi_mfilter_set(const uint32_t* __restrict__ keys, uint64_t n, unsigned long long* filter,
                                 uint64_t mask) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t h = mfilter_hash(keys[i]);
    atomicOr(&filter[(h >> 32) & mask], mfilter_bits(h));
  }
}

struct MphfView {
  const unsigned long long* bits;
  const uint32_t* rank;
  int levels;
  uint64_t off[MPHF_MAX_LEVELS];
  uint64_t size[MPHF_MAX_LEVELS];
};

__host__ __device__ __forceinline__ uint64_t level_seed(int l) {
  uint64_t z = 0x9E3779B97F4A7C15ull * (uint64_t)(l + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  return z ^ (z >> 27);
}

__device__ __forceinline__ uint64_t level_pos(uint32_t key, int l, uint64_t size) {
  const uint64_t h = mix64(((uint64_t)key << 7) ^ level_seed(l));
  return ((h & 0xffffffffull) * size) >> 32;
}

__device__ __forceinline__ uint64_t mphf_lookup(const MphfView& v, uint32_t key) {
  for (int l = 0; l < v.levels; l++) {
    const uint64_t p = v.off[l] + level_pos(key, l, v.size[l]);
    const unsigned long long w = v.bits[p >> 6];
    const uint32_t b = (uint32_t)(p & 63);
    if ((w >> b) & 1ull) return (uint64_t)v.rank[p >> 6] + (uint64_t)__popcll(w & ((1ull << b) - 1ull));
  }
  return MPHF_NOT_FOUND;
}

// ---- distinct keys of the index superkmers
__global__ void k_zi_key_set(const uint32_t* __restrict__ key, uint64_t n, unsigned long long* tab, uint64_t mask,
                             uint32_t* status) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t k = key[i];
    const unsigned long long want = ((unsigned long long)k << 32) | 1ull;
    uint64_t s = mix64((uint64_t)k ^ 0x2545F4914F6CDD1Dull) & mask;
    bool done = false;
    for (uint64_t probe = 0; probe <= mask; probe++) {
      unsigned long long cur = tab[s];
      if (cur == 0ull) {
        const unsigned long long prev = atomicCAS(&tab[s], 0ull, want);
        if (prev == 0ull) { done = true; break; }
        cur = prev;
      }
      if ((uint32_t)(cur >> 32) == k) { done = true; break; }
      s = (s + 1) & mask;
    }
    if (!done) set_status(status, ST_MINTAB_FULL);
  }
}

__global__ void k_zi_key_compact(const unsigned long long* __restrict__ tab, uint64_t slots, uint32_t* out,
                                 unsigned long long* n_out) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < slots; i += (uint64_t)gridDim.x * blockDim.x) {
    const unsigned long long v = tab[i];
    if (v) out[atomicAdd(n_out, 1ull)] = (uint32_t)(v >> 32);
  }
}

// ---- BBHash levels
__global__ void k_bb_mark(const uint32_t* __restrict__ keys, uint64_t n, int level, uint64_t size,
                          unsigned long long* A, unsigned long long* Cw) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t p = level_pos(keys[i], level, size);
    const unsigned long long bit = 1ull << (p & 63);
    const unsigned long long old = atomicOr(&A[p >> 6], bit);
    if (old & bit) atomicOr(&Cw[p >> 6], bit);
  }
}

__global__ void k_bb_next(const uint32_t* __restrict__ keys, uint64_t n, int level, uint64_t size,
                          const unsigned long long* __restrict__ Cw, uint32_t* next, unsigned long long* n_next) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t key = keys[i];
    const uint64_t p = level_pos(key, level, size);
    if ((Cw[p >> 6] >> (p & 63)) & 1ull) next[atomicAdd(n_next, 1ull)] = key;
  }
}

__global__ void k_bb_clear(unsigned long long* A, const unsigned long long* __restrict__ Cw, uint64_t words) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < words; i += (uint64_t)gridDim.x * blockDim.x)
    A[i] &= ~Cw[i];
}

__global__ void k_bb_popc(const unsigned long long* __restrict__ bits, uint64_t words, uint32_t* pc) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < words; i += (uint64_t)gridDim.x * blockDim.x)
    pc[i] = (uint32_t)__popcll(bits[i]);
}

// ---- buckets
__global__ void k_zi_bucket_count(const uint32_t* __restrict__ key, uint64_t n, MphfView v, uint64_t n_keys,
                                  uint32_t* cnt, uint32_t* status) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t b = mphf_lookup(v, key[i]);
    if (b >= n_keys) { set_status(status, ST_BAD_INDEX); continue; }
    atomicAdd(&cnt[b], 1u);
  }
}

__global__ void k_zi_bucket_fill(const uint64_t* __restrict__ desc, const uint32_t* __restrict__ key, uint64_t n,
                                 MphfView v, uint64_t n_keys, uint32_t* cursor, uint64_t* sk,
                                 uint32_t* __restrict__ bucket_key) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t b = mphf_lookup(v, key[i]);
    if (b >= n_keys) continue;
    sk[atomicAdd(&cursor[b], 1u)] = desc[i];
    bucket_key[b] = key[i];  // every superkmer of a bucket carries the same key
  }
}

struct ProbeArgs {
  const uint64_t* qdesc;
  const uint32_t* qkey;
  const unsigned long long* n_q;
  const uint32_t* qpacked;
  const uint32_t* ipacked;
  const uint64_t* sk;
  const uint32_t* bucket_off;
  uint64_t n_keys;
  MphfView v;
  int k;
  uint64_t* out_desc;
  uint32_t* out_key;
  unsigned long long* n_runs;
  unsigned long long* n_absent_windows;
  uint64_t cap;
  const uint32_t* bucket_key;
  const unsigned long long* mfilter;
  uint64_t mf_mask;
};

// the bases after position p of the packed stream, one word load per 16
struct BaseStream {
  const uint32_t* wp;
  uint32_t word, q;
  __device__ __forceinline__ void init(const uint32_t* packed, uint64_t p) {
    wp = packed + (p >> 4);
    q = (uint32_t)(p & 15);
    word = *wp << (2 * q);
  }
  __device__ __forceinline__ uint32_t next() {
    const uint32_t b = word >> 30;
    word <<= 2;
    if (++q == 16) {
      q = 0;
      word = *++wp;
    }
    return b;
  }
};

template <class K, class R>
__device__ __forceinline__ void roll_set(R& r, const uint32_t* packed, uint64_t s0, int k) {
  r.init(k);
  if constexpr (sizeof(K) == 8) {
    r.set(field64(packed, s0, k), k);
  } else {
    if (k > 32) r.set(field64(packed, s0, k - 32), field64(packed, s0 + (uint64_t)(k - 32), 32), k);
    else r.set(0ull, field64(packed, s0, k), k);
  }
}

// The probe works in tiles of PROBE_TILE query superkmers per CTA.
//   A. every thread classifies a share of the tile: a minimizer the index
//      does not hold fails the minimizer filter (one load) or maps to an
//      arbitrary bucket whose stored key differs, so every k-mer of that
//      superkmer is absent (equal canonical k-mers have
//      equal minimizers) and the whole superkmer is one absent run, emitted
//      without rolling it; the others go to the tile's list with their bucket;
//   B. the threads compare the listed superkmers with their buckets, so all
//      lanes do comparison work (foreign reads, about half of a query, no
//      longer leave most lanes idle behind a few comparing ones).
// Absent runs collect in shared memory and leave with one pair of global
// atomics per tile (single-address global atomics per warp had become the
// probe's bottleneck); a tile whose runs overflow the buffer appends the rest
// directly.
constexpr int PROBE_TILE = 1024;
constexpr int PROBE_RUNS = 3072;

struct ProbeSmem {
  uint64_t run_d[PROBE_RUNS];
  uint32_t run_k[PROBE_RUNS];
  uint32_t list_i[PROBE_TILE];
  uint32_t list_b[PROBE_TILE];
  uint32_t n_run, n_list;
  unsigned long long w;  // windows of the buffered runs
  unsigned long long base;
};

__device__ __forceinline__ void tile_run(const ProbeArgs& a, ProbeSmem& sm, uint64_t start, uint32_t len,
                                         uint32_t key) {
  const uint32_t idx = atomicAdd(&sm.n_run, 1u);
  if (idx < (uint32_t)PROBE_RUNS) {
    sm.run_d[idx] = (start << 24) | (uint64_t)(len - 1);
    sm.run_k[idx] = key;
    atomicAdd(&sm.w, (unsigned long long)len);
    return;
  }
  // buffer full: straight to the output
  const unsigned long long g = atomicAdd(a.n_runs, 1ull);
  atomicAdd(a.n_absent_windows, (unsigned long long)len);
  if (g < a.cap) {
    a.out_desc[g] = (start << 24) | (uint64_t)(len - 1);
    a.out_key[g] = key;
  }
}

template <class K, class R>
__global__ void __launch_bounds__(ZI_THREADS) k_zi_probe(ProbeArgs a) {
  __shared__ ProbeSmem sm;
  const uint64_t n = *a.n_q;
  const int k = a.k;
  for (uint64_t t0 = (uint64_t)blockIdx.x * PROBE_TILE; t0 < n; t0 += (uint64_t)gridDim.x * PROBE_TILE) {
    if (threadIdx.x == 0) { sm.n_run = 0; sm.n_list = 0; sm.w = 0; }
    __syncthreads();
    // A. classify
    for (int t = threadIdx.x; t < PROBE_TILE; t += blockDim.x) {
      const uint64_t i = t0 + (uint64_t)t;
      if (i >= n) break;
      const uint64_t d = a.qdesc[i];
      const uint32_t key = a.qkey[i];
      const uint64_t h = mfilter_hash(key);
      const unsigned long long fb = mfilter_bits(h);
      const uint64_t b = (a.mfilter[(h >> 32) & a.mf_mask] & fb) == fb ? mphf_lookup(a.v, key) : MPHF_NOT_FOUND;
      if (b < a.n_keys && a.bucket_key[b] == key) {
        const uint32_t l = atomicAdd(&sm.n_list, 1u);
        sm.list_i[l] = (uint32_t)t;
        sm.list_b[l] = (uint32_t)b;
      } else {
        tile_run(a, sm, d >> 24, (uint32_t)(d & 0xffffffu) + 1u, key);
      }
    }
    __syncthreads();
    // B. compare the listed superkmers with their buckets
    const uint32_t nl = sm.n_list;
    for (uint32_t l = threadIdx.x; l < nl; l += blockDim.x) {
      const uint64_t i = t0 + sm.list_i[l];
      const uint32_t b = sm.list_b[l];
      const uint64_t d = a.qdesc[i];
      const uint64_t s0 = d >> 24;
      const uint32_t nw = (uint32_t)(d & 0xffffffu) + 1u;
      const uint32_t key = a.qkey[i];
      const uint32_t blo = a.bucket_off[b], bhi = a.bucket_off[b + 1];
      int64_t run = -1;
      for (uint32_t c0 = 0; c0 < nw; c0 += Q_CHUNK) {
        const uint32_t cn = min((uint32_t)Q_CHUNK, nw - c0);
        K q[Q_CHUNK];
        {
          R r;
          roll_set<K, R>(r, a.qpacked, s0 + c0, k);
          BaseStream bs;
          bs.init(a.qpacked, s0 + c0 + (uint64_t)k);
#pragma unroll
          for (int t = 0; t < Q_CHUNK; t++) {
            if (t < (int)cn) {
              if (t > 0) r.push(bs.next());
              q[t] = r.canon();
            }
          }
        }
        const uint32_t full = (cn == 32) ? 0xffffffffu : ((1u << cn) - 1u);
        uint32_t found = 0;
        for (uint32_t j = blo; j < bhi && found != full; j++) {
          const uint64_t e = a.sk[j];
          const uint64_t e0 = e >> 24;
          const uint32_t en = (uint32_t)(e & 0xffffffu) + 1u;
          R r;
          roll_set<K, R>(r, a.ipacked, e0, k);
          BaseStream bs;
          bs.init(a.ipacked, e0 + (uint64_t)k);
          for (uint32_t u = 0; u < en; u++) {
            if (u > 0) r.push(bs.next());
            const K ek = r.canon();
#pragma unroll
            for (int t = 0; t < Q_CHUNK; t++)
              if (t < (int)cn && key_eq(q[t], ek)) found |= 1u << t;
            if (found == full) break;
          }
        }
        for (uint32_t t = 0; t < cn; t++) {
          const bool absent = !((found >> t) & 1u);
          if (absent) {
            if (run < 0) run = (int64_t)(c0 + t);
          } else if (run >= 0) {
            tile_run(a, sm, s0 + (uint64_t)run, c0 + t - (uint32_t)run, key);
            run = -1;
          }
        }
      }
      if (run >= 0) tile_run(a, sm, s0 + (uint64_t)run, nw - (uint32_t)run, key);
    }
    __syncthreads();
    // C. the tile's buffered runs, in one piece
    const uint32_t nr = min(sm.n_run, (uint32_t)PROBE_RUNS);
    if (threadIdx.x == 0) {
      sm.base = nr ? atomicAdd(a.n_runs, (unsigned long long)nr) : 0ull;
      if (sm.w) atomicAdd(a.n_absent_windows, sm.w);
    }
    __syncthreads();
    for (uint32_t r = threadIdx.x; r < nr; r += blockDim.x) {
      const unsigned long long g = sm.base + r;
      if (g < a.cap) {
        a.out_desc[g] = sm.run_d[r];
        a.out_key[g] = sm.run_k[r];
      }
    }
    __syncthreads();
  }
}


// ---- dedup of the absent windows
// Absent k-mers are mostly distinct (sequencing errors, foreign reads), and
// their runs are short and scattered, so regenerating them per counting round
// would pay a scattered packed-stream gather per run and per round.  Instead:
//   1. expand: each absent run is rolled once, in emission order (close to
//      stream order), into flat (k-mer, input) records partitioned into 2^b1
//      buckets (b1 <= 8) by the top bits of the k-mer hash: a histogram pass
//      gives every CTA its own range of each bucket, then the CTA takes about
//      a thousand runs at a time, counting-sorts their records by bucket in
//      shared memory and writes each bucket's share as one contiguous piece
//      (a run of more than DD_LONG windows is written record by record);
//   2. split: when more buckets are needed, one CTA per bucket splits it by
//      the next b2 <= 9 bits, with the same tile-sorted writes;
//   3. dedup: a persistent CTA takes one final bucket at a time (sized to
//      about half its shared-memory table) and deduplicates it there, in
//      sub-rounds over the next 20 hash bits when the bucket is larger; a
//      sub-round that overflows is redone as two (no estimate can change the
//      result).
constexpr int DD_MAX_BITS1 = 8;
constexpr int DD_NB1 = 1 << DD_MAX_BITS1;
constexpr int DD_MAX_BITS = 17;  // final buckets: level 1 (<= 8 bits) + level 2 (<= 9 bits)
constexpr int DD_NB2 = 1 << (DD_MAX_BITS - DD_MAX_BITS1);
constexpr int DD_CTAS = 304;
constexpr int DD_THREADS = 512;
constexpr int DDK_THREADS = 1024;
constexpr uint32_t DD_PROBE_LIMIT = 256;
constexpr uint32_t DD_LONG = 64;  // longer runs bypass the shared-memory tile
constexpr int DD_RPT = 2;         // runs per thread in one expand tile

// records in one shared-memory tile of the sorted scatters (key, input id and
// bucket per record: about 90 KB for 64-bit keys, 76 KB for 128-bit keys)
template <class K> struct DdTile;
template <> struct DdTile<K64> { static constexpr uint32_t CAP = 8192; };
template <> struct DdTile<K128> { static constexpr uint32_t CAP = 4096; };
template <class K> constexpr size_t dd_tile_bytes() { return (size_t)DdTile<K>::CAP * (sizeof(K) + 3); }
// the split's tile: a 16-bit bucket per record (up to 9 bits)
template <class K> constexpr size_t dd_split_tile_bytes() { return (size_t)DdTile<K>::CAP * (sizeof(K) + 4); }

// exclusive block scan of one u32 per thread; ws holds 32 words
__device__ __forceinline__ uint32_t dd_block_scan(uint32_t v, uint32_t* total, uint32_t* ws) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  uint32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[wid] = x;
  __syncthreads();
  if (wid == 0) {
    uint32_t t = lane < nw ? ws[lane] : 0u;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    ws[lane] = t;
  }
  __syncthreads();
  const uint32_t r = x - v + (wid ? ws[wid - 1] : 0u);
  *total = ws[nw - 1];
  __syncthreads();
  return r;
}

struct ExpandArgs {
  const uint64_t* runs;        // start << 24 | (windows - 1)
  uint64_t n_runs;
  const uint32_t* packed;
  const uint64_t* input_base;  // n_inputs + 1 first bases
  int n_inputs;
  int with_ids;                // per-input results: record each window's input
  int k;
  int bits1;                   // level-1 bucket bits (0 .. 8)
  uint32_t* hist;              // [2^bits1][DD_CTAS]
  const uint32_t* pre;         // exclusive scan of hist (scatter pass)
  void* keys_out;
  uint16_t* ids_out;
};

// hash bits [64 - hi - n, 64 - hi): a digit below the top `hi` bits
__device__ __forceinline__ uint32_t dd_digit(uint64_t h, int hi, int n) {
  return n == 0 ? 0u : (uint32_t)(h >> (64 - hi - n)) & ((1u << n) - 1u);
}

// Level-1 bucket of a rolled window, a function of its canonical k-mer
// without forming it: for k <= 32 the sum of the two strands' multiplicative
// hashes (the top half of one 64-bit product each, on the FMA pipe; a sum of
// two uniform values mod 2^32 stays uniform, their minimum would not), for
// longer k the strand-symmetric hash.  Level 2 and the dedup take their
// digits from key_hash of the stored key, an independent hash.
__device__ __forceinline__ uint32_t dd_level1(const Roll64& r, int n) {
  const uint32_t a = (uint32_t)((r.fwd * 0x9E3779B97F4A7C15ull) >> 32);
  const uint32_t b = (uint32_t)((r.rev * 0x9E3779B97F4A7C15ull) >> 32);
  return n == 0 ? 0u : (a + b) >> (32 - n);
}
__device__ __forceinline__ uint32_t dd_level1(const Roll128& r, int n) {
  return n == 0 ? 0u : (uint32_t)(sym_hash(r) >> (64 - n));
}


// the input of a run: largest j with input_base[j] <= start; the last answer
// is kept, as consecutive runs of a slice mostly come from the same input
struct InputCursor {
  int cur = -1;
  uint64_t lo = 0, hi = 0;
  __device__ __forceinline__ uint16_t of(const ExpandArgs& a, uint64_t s0) {
    if (cur < 0 || s0 < lo || s0 >= hi) {
      int l2 = 0, h2 = a.n_inputs;
      while (h2 - l2 > 1) { const int mid = (l2 + h2) >> 1; if (a.input_base[mid] <= s0) l2 = mid; else h2 = mid; }
      cur = l2;
      lo = a.input_base[l2];
      hi = a.input_base[l2 + 1];
    }
    return (uint16_t)cur;
  }
};

__device__ __forceinline__ void dd_slice(uint64_t n, uint64_t* lo, uint64_t* hi) {
  const uint64_t per = (n + DD_CTAS - 1) / DD_CTAS;
  *lo = min(per * blockIdx.x, n);
  *hi = min(*lo + per, n);
}

// histogram pass: records per (level-1 bucket, CTA)
template <class K, class R>
__global__ void __launch_bounds__(DD_THREADS) k_zi_expand_count(ExpandArgs a) {
  __shared__ uint32_t c[DD_NB1];
  const int nb = 1 << a.bits1;
  for (int i = threadIdx.x; i < nb; i += DD_THREADS) c[i] = 0u;
  __syncthreads();
  uint64_t lo, hi;
  dd_slice(a.n_runs, &lo, &hi);
  const int k = a.k;
  for (uint64_t i = lo + threadIdx.x; i < hi; i += DD_THREADS) {
    const uint64_t d = a.runs[i];
    const uint64_t s0 = d >> 24;
    const uint32_t nw = (uint32_t)(d & 0xffffffu) + 1u;
    R r;
    roll_set<K, R>(r, a.packed, s0, k);
    BaseStream bs;
    bs.init(a.packed, s0 + (uint64_t)k);
    for (uint32_t u = 0; u < nw; u++) {
      if (u > 0) r.push(bs.next());
      atomicAdd(&c[dd_level1(r, a.bits1)], 1u);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nb; i += DD_THREADS) a.hist[(uint64_t)i * DD_CTAS + blockIdx.x] = c[i];
}

// scatter pass over the same slices.  Per tile: the threads' runs are laid
// out by a block scan of their window counts (the threads whose runs fit in
// the tile are a prefix); the records are rolled once to count them per
// bucket, once more to place them in bucket order in shared memory, and the
// tile is written out bucket by bucket at the CTA's cursors.
template <class K, class R>
__global__ void __launch_bounds__(DD_THREADS) k_zi_expand_scatter(ExpandArgs a) {
  constexpr uint32_t CAP = DdTile<K>::CAP;
  extern __shared__ __align__(16) uint8_t smem[];
  K* skey = reinterpret_cast<K*>(smem);
  uint16_t* sid = reinterpret_cast<uint16_t*>(smem + (size_t)CAP * sizeof(K));
  uint8_t* sb = reinterpret_cast<uint8_t*>(sid + CAP);
  __shared__ uint32_t gcur[DD_NB1], gdst[DD_NB1], tcnt[DD_NB1], tstart[DD_NB1];
  __shared__ uint32_t ws[32];
  const int nb = 1 << a.bits1;
  const int tid = threadIdx.x;
  for (int i = tid; i < nb; i += DD_THREADS) {
    gcur[i] = a.pre[(uint64_t)i * DD_CTAS + blockIdx.x];
    tcnt[i] = 0u;
  }
  uint64_t lo, hi;
  dd_slice(a.n_runs, &lo, &hi);
  const int k = a.k;
  K* kout = reinterpret_cast<K*>(a.keys_out);
  uint16_t* iout = a.with_ids ? a.ids_out : nullptr;
  InputCursor ic;
  __syncthreads();
  for (uint64_t base = lo; base < hi;) {
    const uint64_t r0 = base + (uint64_t)tid * DD_RPT;
    uint64_t d[DD_RPT];
    uint32_t nwt = 0;
#pragma unroll
    for (int q = 0; q < DD_RPT; q++) {
      d[q] = r0 + q < hi ? a.runs[r0 + q] : ~0ull;
      const uint32_t nw = d[q] == ~0ull ? 0u : (uint32_t)(d[q] & 0xffffffu) + 1u;
      nwt += nw <= DD_LONG ? nw : 0u;
    }
    uint32_t total;
    const uint32_t o = dd_block_scan(nwt, &total, ws);
    const bool fit = o + nwt <= CAP;
    const int n_fit = __syncthreads_count(fit);
    // pass A: count the tile's records per bucket; long runs go straight out
    if (fit) {
#pragma unroll
      for (int q = 0; q < DD_RPT; q++) {
        if (d[q] == ~0ull) continue;
        const uint64_t s0 = d[q] >> 24;
        const uint32_t nw = (uint32_t)(d[q] & 0xffffffu) + 1u;
        const bool lng = nw > DD_LONG;
        const uint16_t ds = (a.with_ids && lng) ? ic.of(a, s0) : 0;
        R r;
        roll_set<K, R>(r, a.packed, s0, k);
        BaseStream bs;
        bs.init(a.packed, s0 + (uint64_t)k);
        for (uint32_t u = 0; u < nw; u++) {
          if (u > 0) r.push(bs.next());
          const uint32_t b = dd_level1(r, a.bits1);
          if (!lng) {
            atomicAdd(&tcnt[b], 1u);
          } else {
            const K key = r.canon();
            const uint32_t pos = atomicAdd(&gcur[b], 1u);
            kout[pos] = key;
            if (iout) iout[pos] = ds;
          }
        }
      }
    }
    __syncthreads();
    {
      const uint32_t v = tid < nb ? tcnt[tid] : 0u;
      uint32_t tt;
      const uint32_t pre = dd_block_scan(v, &tt, ws);
      if (tid < nb) {
        tstart[tid] = pre;
        tcnt[tid] = pre;  // the tile cursor of pass B
        gdst[tid] = gcur[tid];
        gcur[tid] += v;
      }
      total = tt;
    }
    __syncthreads();
    // pass B: place the records in bucket order
    if (fit) {
#pragma unroll
      for (int q = 0; q < DD_RPT; q++) {
        if (d[q] == ~0ull) continue;
        const uint64_t s0 = d[q] >> 24;
        const uint32_t nw = (uint32_t)(d[q] & 0xffffffu) + 1u;
        if (nw > DD_LONG) continue;
        const uint16_t ds = a.with_ids ? ic.of(a, s0) : 0;
        R r;
        roll_set<K, R>(r, a.packed, s0, k);
        BaseStream bs;
        bs.init(a.packed, s0 + (uint64_t)k);
        for (uint32_t u = 0; u < nw; u++) {
          if (u > 0) r.push(bs.next());
          const K key = r.canon();
          const uint32_t b = dd_level1(r, a.bits1);
          const uint32_t pos = atomicAdd(&tcnt[b], 1u);
          skey[pos] = key;
          sid[pos] = ds;
          sb[pos] = (uint8_t)b;
        }
      }
    }
    __syncthreads();
    for (uint32_t j = tid; j < total; j += DD_THREADS) {
      const uint32_t b = sb[j];
      const uint32_t g = gdst[b] + (j - tstart[b]);
      kout[g] = skey[j];
      if (iout) iout[g] = sid[j];
    }
    __syncthreads();
    for (int i = tid; i < nb; i += DD_THREADS) tcnt[i] = 0u;
    base += (uint64_t)n_fit * DD_RPT;
  }
}

// bucket offsets of level 1: off[b] = pre[b * DD_CTAS] (b <= 2^bits1)
__global__ void k_zi_off1(const uint32_t* __restrict__ pre, int nb, uint32_t* __restrict__ off) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= nb; i += gridDim.x * blockDim.x) off[i] = pre[(uint64_t)i * DD_CTAS];
}

struct SplitArgs {
  const void* keys_in;
  const uint16_t* ids_in;
  const uint32_t* off1;        // level-1 bucket b = [off1[b], off1[b + 1])
  int bits1, bits2;
  void* keys_out;
  uint16_t* ids_out;
  uint32_t* off2;              // final bucket b1 << bits2 | j, plus the total at the end
};

// one CTA per level-1 bucket: histogram by the next bits2 bits, scan, then
// tiles of DDK_THREADS x E records counting-sorted in shared memory and
// written out bucket by bucket
template <class K, int E>
__global__ void __launch_bounds__(DDK_THREADS) k_zi_split(SplitArgs a) {
  constexpr uint32_t T = (uint32_t)DDK_THREADS * E;
  static_assert(T <= DdTile<K>::CAP, "split tile larger than the shared-memory tile");
  extern __shared__ __align__(16) uint8_t smem[];
  K* skey = reinterpret_cast<K*>(smem);
  uint16_t* sid = reinterpret_cast<uint16_t*>(smem + (size_t)T * sizeof(K));
  uint16_t* sb = sid + T;
  __shared__ uint32_t gcur[DD_NB2], gdst[DD_NB2], tcnt[DD_NB2], tstart[DD_NB2];
  __shared__ uint32_t ws[32];
  const int nb2 = 1 << a.bits2;
  const int tid = threadIdx.x;
  const uint32_t b1 = blockIdx.x;
  const uint32_t lo = a.off1[b1], hi = a.off1[b1 + 1];
  const K* kin = reinterpret_cast<const K*>(a.keys_in);
  K* kout = reinterpret_cast<K*>(a.keys_out);
  for (int i = tid; i < nb2; i += DDK_THREADS) { gcur[i] = 0u; tcnt[i] = 0u; }
  __syncthreads();
  for (uint32_t j = lo + tid; j < hi; j += DDK_THREADS)
    atomicAdd(&gcur[dd_digit(key_hash(kin[j]), a.bits1, a.bits2)], 1u);
  __syncthreads();
  {
    const uint32_t v = tid < nb2 ? gcur[tid] : 0u;
    uint32_t tot;
    const uint32_t pre = dd_block_scan(v, &tot, ws);
    if (tid < nb2) {
      gcur[tid] = lo + pre;
      a.off2[(uint64_t)b1 * nb2 + tid] = lo + pre;
    }
  }
  if (b1 == gridDim.x - 1 && tid == 0) a.off2[(uint64_t)gridDim.x * nb2] = hi;
  __syncthreads();
  for (uint32_t t0 = lo; t0 < hi; t0 += T) {
    K key[E];
    uint16_t id[E];
    uint32_t bb[E], rk[E];
#pragma unroll
    for (int e = 0; e < E; e++) {
      const uint32_t j = t0 + (uint32_t)e * DDK_THREADS + tid;
      bb[e] = 0xffffffffu;
      if (j < hi) {
        key[e] = kin[j];
        id[e] = a.ids_in ? a.ids_in[j] : (uint16_t)0;
        bb[e] = dd_digit(key_hash(key[e]), a.bits1, a.bits2);
        rk[e] = atomicAdd(&tcnt[bb[e]], 1u);
      }
    }
    __syncthreads();
    uint32_t total;
    {
      const uint32_t v = tid < nb2 ? tcnt[tid] : 0u;
      const uint32_t pre = dd_block_scan(v, &total, ws);
      if (tid < nb2) {
        tstart[tid] = pre;
        gdst[tid] = gcur[tid];
        gcur[tid] += v;
        tcnt[tid] = 0u;
      }
    }
    __syncthreads();
#pragma unroll
    for (int e = 0; e < E; e++) {
      if (bb[e] == 0xffffffffu) continue;
      const uint32_t pos = tstart[bb[e]] + rk[e];
      skey[pos] = key[e];
      sid[pos] = id[e];
      sb[pos] = (uint16_t)bb[e];
    }
    __syncthreads();
    for (uint32_t j = tid; j < total; j += DDK_THREADS) {
      const uint32_t b = sb[j];
      const uint32_t g = gdst[b] + (j - tstart[b]);
      kout[g] = skey[j];
      if (a.ids_out) a.ids_out[g] = sid[j];
    }
    __syncthreads();
  }
}

struct BucketDedupArgs {
  const void* keys;
  const uint16_t* ids;
  const uint32_t* off;         // bucket b = records [off[b], off[b + 1])
  uint32_t n_buckets;
  int bits;                    // hash bits the buckets consumed
  int W;                       // mask words per slot (0: union, no masks)
  uint32_t slots;
  unsigned int* work;
  uint64_t* out_lo;
  uint64_t* out_hi;
  uint32_t* out_count;
  unsigned long long* out_mask;
  unsigned long long* n_out;
  uint64_t cap;
  uint32_t* status;
};

__device__ __forceinline__ bool dd_maybe_empty(K64 c) { return c.v == ~0ull; }
__device__ __forceinline__ bool dd_maybe_empty(K128 c) { return c.lo == ~0ull || c.hi == ~0ull; }
__device__ __forceinline__ K64 dd_cas(K64* p, K64 cmp, K64 val) {
  return K64{(uint64_t)atomicCAS(reinterpret_cast<unsigned long long*>(p), (unsigned long long)cmp.v,
                                 (unsigned long long)val.v)};
}
__device__ __forceinline__ K128 dd_cas(K128* p, K128 cmp, K128 val) { return atomicCAS(p, cmp, val); }

// Two CTAs per SM, so one CTA's barriers overlap the other's work.  CTA c
// takes buckets c, c + G, c + 2G, ...; a bucket's records (at most
// dd_e<K>() per thread, the bucket size the host plans for) stay in registers
// through its sub-rounds, and the next bucket's records are loaded while the
// last sub-round is emitted.  Larger buckets (more than 2^17 buckets would be
// needed) are read from global memory per sub-round.  The table starts empty
// and every emit (or overflow) leaves it empty.
constexpr int DDD_THREADS = 512;
template <class K> __host__ __device__ constexpr int dd_e() { return sizeof(K) == 8 ? 8 : 4; }
template <class K> __host__ __device__ constexpr size_t dd_keys_bytes(uint32_t slots) {
  return ((size_t)slots * sizeof(K) + 15) & ~(size_t)15;
}

template <class K>
__global__ void __launch_bounds__(DDD_THREADS, 2) k_zi_bucket_dedup(BucketDedupArgs a) {
  constexpr int E = dd_e<K>();
  extern __shared__ __align__(16) uint8_t smem[];
  const uint32_t S = a.slots;
  const int W = a.W;
  // table keys, W mask words per slot, and the list of occupied slots in
  // insertion order (the emit walks only these, and writes them densely)
  K* tk = reinterpret_cast<K*>(smem);
  unsigned long long* tm = reinterpret_cast<unsigned long long*>(smem + dd_keys_bytes<K>(S));
  uint16_t* list = reinterpret_cast<uint16_t*>(smem + dd_keys_bytes<K>(S) + (size_t)S * 8 * W);
  __shared__ uint32_t s_over, s_n;
  __shared__ unsigned long long s_base;
  const K EMPTY = key_empty<K>();
  const K* keys = reinterpret_cast<const K*>(a.keys);
  const int tid = threadIdx.x, nth = blockDim.x;
  const uint32_t in_regs = (uint32_t)E * (uint32_t)nth;
  K rk[E];
  uint16_t rd[E];
  auto load_regs = [&](uint32_t l, uint32_t h) {
#pragma unroll
    for (int e = 0; e < E; e++) {
      const uint32_t j = l + (uint32_t)e * nth + tid;
      if (j < h) {
        rk[e] = keys[j];
        rd[e] = W ? a.ids[j] : (uint16_t)0;
      }
    }
  };
  // insert one record; false when its probe sequence found no room
  auto insert = [&](const K& key, uint16_t ds, uint32_t sub_lo, uint32_t sub_hi) -> bool {
    const uint64_t h = key_hash(key);
    const uint32_t sub = dd_digit(h, a.bits, 20);
    if (sub < sub_lo || sub >= sub_hi) return true;
    uint32_t slot = (uint32_t)(((h & 0xffffffffull) * (uint64_t)S) >> 32);
    for (uint32_t probe = 0; probe < DD_PROBE_LIMIT; probe++) {
      K cur = tk[slot];
      if (dd_maybe_empty(cur)) {
        const K prev = dd_cas(&tk[slot], EMPTY, key);
        if (key_eq(prev, EMPTY)) {
          namespace cg = cooperative_groups;
          cg::coalesced_group g = cg::coalesced_threads();
          uint32_t at = 0;
          if (g.thread_rank() == 0) at = atomicAdd(&s_n, g.size());
          list[g.shfl(at, 0) + g.thread_rank()] = (uint16_t)slot;
          cur = key;
        } else {
          cur = prev;
        }
      }
      if (key_eq(cur, key)) {
        if (W) atomicOr(&tm[(size_t)slot * W + (ds >> 6)], 1ull << (ds & 63));
        return true;
      }
      slot = (slot + 1 == S) ? 0u : slot + 1;
    }
    return false;
  };
  for (uint32_t s = tid; s < S; s += nth) {
    tk[s] = EMPTY;
    for (int q = 0; q < W; q++) tm[(size_t)s * W + q] = 0ull;
  }
  if (tid == 0) s_n = 0;
  const uint32_t G = gridDim.x, NB = a.n_buckets;
  uint32_t b = blockIdx.x;
  uint32_t lo = 0, hi = 0;
  if (b < NB) {
    lo = a.off[b];
    hi = a.off[b + 1];
    if (hi - lo <= in_regs) load_regs(lo, hi);
  }
  __syncthreads();
  for (; b < NB; b += G) {
    uint32_t nlo = 0, nhi = 0;
    if (b + G < NB) {
      nlo = a.off[b + G];
      nhi = a.off[b + G + 1];
    }
    bool regs = hi - lo <= in_regs;
    // sub-rounds: at most half a table of records each (distinct <= records)
    uint32_t r = hi > lo ? (hi - lo + S / 2 - 1) / (S / 2) : 0u;
    uint32_t i = 0;
    while (i < r) {
      const uint32_t sub_lo = (uint32_t)(((uint64_t)i << 20) / r), sub_hi = (uint32_t)(((uint64_t)(i + 1) << 20) / r);
      if (tid == 0) s_over = 0;
      __syncthreads();
      if (regs) {
#pragma unroll
        for (int e = 0; e < E; e++) {
          const uint32_t j = lo + (uint32_t)e * nth + tid;
          if (j < hi && !insert(rk[e], rd[e], sub_lo, sub_hi)) s_over = 1;
        }
      } else {
        for (uint32_t j = lo + tid; j < hi; j += nth) {
          if (*(volatile uint32_t*)&s_over) break;
          if (!insert(keys[j], W ? a.ids[j] : (uint16_t)0, sub_lo, sub_hi)) { s_over = 1; break; }
        }
      }
      __syncthreads();
      const uint32_t n = s_n;
      if (s_over) {
        for (uint32_t s = tid; s < S; s += nth) {
          tk[s] = EMPTY;
          for (int q = 0; q < W; q++) tm[(size_t)s * W + q] = 0ull;
        }
        // this sub-range becomes two: sub-round i of r is sub-rounds 2i, 2i+1 of 2r
        if (r >= (1u << 20)) {
          if (tid == 0) set_status(a.status, ST_TABLE_STUCK);
          i = r;
        } else {
          r *= 2;
          i *= 2;
        }
        __syncthreads();
        if (tid == 0) s_n = 0;
        continue;
      }
      if (i + 1 == r) {  // this bucket's records are done with: load the next bucket's
        regs = false;
        if (nhi - nlo <= in_regs) load_regs(nlo, nhi);
      }
      // emit the listed slots densely (one global atomic per sub-round) and reset them
      if (tid == 0) s_base = atomicAdd(a.n_out, (unsigned long long)n);
      __syncthreads();
      const unsigned long long base = s_base;
      for (uint32_t t = tid; t < n; t += nth) {
        const uint32_t slot = list[t];
        const K key = tk[slot];
        tk[slot] = EMPTY;
        const unsigned long long o = base + t;
        uint32_t c = 1;
        if (W) {
          c = 0;
          for (int q = 0; q < W; q++) {
            const unsigned long long m = tm[(size_t)slot * W + q];
            tm[(size_t)slot * W + q] = 0ull;
            if (o < a.cap) a.out_mask[o * (uint64_t)W + q] = m;
            c += __popcll(m);
          }
        }
        if (o < a.cap) {
          if constexpr (sizeof(K) == 8) {
            a.out_lo[o] = reinterpret_cast<const K64&>(key).v;
          } else {
            a.out_lo[o] = reinterpret_cast<const K128&>(key).lo;
            a.out_hi[o] = reinterpret_cast<const K128&>(key).hi;
          }
          a.out_count[o] = c;
        } else {
          set_status(a.status, ST_OUT_OVERFLOW);
        }
      }
      if (tid == 0) s_n = 0;  // every thread read n before the barrier above
      __syncthreads();
      i++;
    }
    if (r == 0 && nhi - nlo <= in_regs) load_regs(nlo, nhi);
    lo = nlo;
    hi = nhi;
  }
}

// ---- per-input split of a batch result (records x masks -> per-input lists)
constexpr int SPLIT_CHUNK = 4096;
constexpr int SPLIT_MAX_INPUTS = 4096;

__global__ void __launch_bounds__(ZI_THREADS) k_zi_split_count(const unsigned long long* __restrict__ masks,
                                                               uint64_t n, int W, int n_inputs,
                                                               unsigned long long* __restrict__ cnt) {
  __shared__ uint32_t c[SPLIT_MAX_INPUTS];
  for (int i = threadIdx.x; i < n_inputs; i += blockDim.x) c[i] = 0;
  __syncthreads();
  const uint64_t c0 = (uint64_t)blockIdx.x * SPLIT_CHUNK;
  const uint64_t c1 = c0 + SPLIT_CHUNK < n ? c0 + SPLIT_CHUNK : n;
  for (uint64_t i = c0 + threadIdx.x; i < c1; i += blockDim.x)
    for (int q = 0; q < W; q++)
      for (unsigned long long m = masks[i * W + q]; m; m &= m - 1) atomicAdd(&c[q * 64 + __ffsll((long long)m) - 1], 1u);
  __syncthreads();
  for (int i = threadIdx.x; i < n_inputs; i += blockDim.x)
    if (c[i]) atomicAdd(&cnt[i], (unsigned long long)c[i]);
}

__global__ void __launch_bounds__(ZI_THREADS) k_zi_split_fill(const unsigned long long* __restrict__ masks,
                                                              const uint64_t* __restrict__ lo,
                                                              const uint64_t* __restrict__ hi, uint64_t n, int W,
                                                              int n_inputs, unsigned long long* __restrict__ cursor,
                                                              uint64_t* __restrict__ out_lo,
                                                              uint64_t* __restrict__ out_hi) {
  __shared__ uint32_t c[SPLIT_MAX_INPUTS];
  __shared__ unsigned long long base[SPLIT_MAX_INPUTS];
  for (int i = threadIdx.x; i < n_inputs; i += blockDim.x) c[i] = 0;
  __syncthreads();
  const uint64_t c0 = (uint64_t)blockIdx.x * SPLIT_CHUNK;
  const uint64_t c1 = c0 + SPLIT_CHUNK < n ? c0 + SPLIT_CHUNK : n;
  for (uint64_t i = c0 + threadIdx.x; i < c1; i += blockDim.x)
    for (int q = 0; q < W; q++)
      for (unsigned long long m = masks[i * W + q]; m; m &= m - 1) atomicAdd(&c[q * 64 + __ffsll((long long)m) - 1], 1u);
  __syncthreads();
  for (int i = threadIdx.x; i < n_inputs; i += blockDim.x) {
    base[i] = c[i] ? atomicAdd(&cursor[i], (unsigned long long)c[i]) : 0ull;
    c[i] = 0;
  }
  __syncthreads();
  for (uint64_t i = c0 + threadIdx.x; i < c1; i += blockDim.x)
    for (int q = 0; q < W; q++)
      for (unsigned long long m = masks[i * W + q]; m; m &= m - 1) {
        const int r = q * 64 + __ffsll((long long)m) - 1;
        const uint64_t o = base[r] + atomicAdd(&c[r], 1u);
        out_lo[o] = lo[i];
        if (out_hi) out_hi[o] = hi ? hi[i] : 0ull;
      }
}

int grid_for(mczi_ctx* ctx, uint64_t n) {
  const uint64_t g = (n + ZI_THREADS - 1) / ZI_THREADS;
  const uint64_t cap = (uint64_t)ctx->sm_count * 16;
  return (int)std::max<uint64_t>(1, std::min(g, cap));
}

struct SumU32 {
  static __device__ uint32_t identity() { return 0u; }
  static __device__ uint32_t combine(const uint32_t& a, const uint32_t& b) { return a + b; }
};

MphfView view_of(const ZiIndex& z) {
  MphfView v;
  v.bits = z.bits.as<unsigned long long>();
  v.rank = z.rank.as<uint32_t>();
  v.levels = z.levels;
  for (int l = 0; l < MPHF_MAX_LEVELS; l++) {
    v.off[l] = z.lvl_off[l];
    v.size[l] = z.lvl_size[l];
  }
  return v;
}

// ZI's validate_k (src/zi.rs:103-107) and minimizer bound (src/zi.rs:70-72)
int32_t zi_validate(mczi_ctx* ctx, uint32_t k, uint32_t m) {
  if (k < 3 || k > 63) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "k must be in [3, 63] for sshash-rs");
  if (k % 2 == 0) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "k must be odd for sshash-rs");
  if (m == 0 || m >= k) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "minimizer size must be > 0 and < k");
  return MCZI_OK;
}

int32_t zi_build_stream(mczi_ctx* ctx, Pipe& p, uint64_t nb, uint32_t k, uint32_t m, cudaEvent_t e0,
                        cudaEvent_t e1);

// k-mer records -> a 2-bit stream in which each k-mer is its own fragment
// (base b of the stream is base b mod k of k-mer b / k): one thread per
// packed word and per fragment-bit word, no atomics
__global__ void k_kmers_to_stream(const uint64_t* __restrict__ lo, const uint64_t* __restrict__ hi, uint64_t n,
                                  int k, uint32_t* __restrict__ packed, uint64_t pwords, uint32_t* __restrict__ fbits,
                                  uint64_t fwords) {
  const uint64_t nb = n * (uint64_t)k;
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < pwords; w += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t word = 0;
    for (uint32_t q = 0; q < 16; q++) {
      const uint64_t b = w * 16 + q;
      if (b >= nb) break;
      const uint64_t i = b / (uint64_t)k;
      const int sh = 2 * (k - 1 - (int)(b - i * (uint64_t)k));  // bit offset of the base in the k-mer value
      const uint64_t code = sh >= 64 ? (hi[i] >> (sh - 64)) & 3u : (lo[i] >> sh) & 3u;
      word |= (uint32_t)code << (30 - 2 * q);
    }
    packed[w] = word;
  }
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < fwords; w += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t word = 0;
    const uint64_t b0 = w * 32;
    // the first fragment start at or after b0
    uint64_t b = ((b0 + (uint64_t)k - 1) / (uint64_t)k) * (uint64_t)k;
    for (; b < b0 + 32 && b < nb; b += (uint64_t)k) word |= 1u << (b - b0);
    fbits[w] = word;
  }
}

int32_t zi_build(mczi_ctx* ctx, const uint8_t* fasta, uint64_t len, uint32_t k, uint32_t m) {
  int32_t rc = zi_validate(ctx, k, m);
  if (rc) return rc;
  ZiIndex& z = ctx->zi;
  z.built = false;
  mczi_input in{fasta, len};
  if ((rc = stage_inputs(ctx, &in, 1))) return rc;
  if (ctx->skipped) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "index FASTA does not start with a FASTA/FASTQ record");
  cudaStream_t s = ctx->stream;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaEventRecord(e0, s));
  Pipe p;
  if ((rc = pipe_pack(ctx, p))) return rc;
  uint64_t nb = 0;
  CK(cudaMemcpyAsync(&nb, p.d_nbases, 8, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (nb == 0)  // src/zi.rs:116-120
    return fail(ctx, MCZI_ERR_INVALID_CONFIG, "index FASTA did not contain any sequence of length >= k");
  return zi_build_stream(ctx, p, nb, k, m, e0, e1);
}

// The dictionary of the 2-bit stream in ctx->packed / ctx->fbits (nb bases;
// p.d_nbases on the device): superkmers, minimizer keys and filter, MPHF,
// buckets.  e0 was recorded at the start of the build.
int32_t zi_build_stream(mczi_ctx* ctx, Pipe& p, uint64_t nb, uint32_t k, uint32_t m, cudaEvent_t e0,
                        cudaEvent_t e1) {
  ZiIndex& z = ctx->zi;
  cudaStream_t s = ctx->stream;
  int32_t rc;
  if ((rc = pipe_scan(ctx, p, (int)k, (int)m))) return rc;
  const uint64_t n_desc = p.n_desc;
  uint64_t* sc = ctx->scalars.as<uint64_t>();
  // keep the index stream
  CKA(z.packed, p.pwords * 4);
  CK(cudaMemcpyAsync(z.packed.p, ctx->packed.p, p.pwords * 4, cudaMemcpyDeviceToDevice, s));
  z.pwords = p.pwords;
  z.n_bases = nb;
  z.k = (int)k;
  z.m = (int)m;
  z.n_sk = n_desc;
  // distinct minimizer keys
  uint64_t slots = 1024;
  while (slots < 2 * n_desc) slots <<= 1;
  CKA(ctx->zi_tmp0, slots * 8);
  CK(cudaMemsetAsync(ctx->zi_tmp0.p, 0, slots * 8, s));
  CK(cudaMemsetAsync(sc + SC_STATUS, 0, 8, s));
  CK(cudaMemsetAsync(sc + SC_NKEPT, 0, 8, s));
  const uint32_t* d_key = ctx->key.as<uint32_t>();
  if (n_desc) k_zi_key_set<<<grid_for(ctx, n_desc), ZI_THREADS, 0, s>>>(d_key, n_desc, ctx->zi_tmp0.as<unsigned long long>(),
                                                                       slots - 1, reinterpret_cast<uint32_t*>(sc + SC_STATUS));
  CKA(ctx->zi_tmp1, std::max<uint64_t>(n_desc, 1) * 4 * 2);  // two key lists (current, next level)
  uint32_t* keys_a = ctx->zi_tmp1.as<uint32_t>();
  uint32_t* keys_b = keys_a + std::max<uint64_t>(n_desc, 1);
  k_zi_key_compact<<<grid_for(ctx, slots), ZI_THREADS, 0, s>>>(ctx->zi_tmp0.as<unsigned long long>(), slots, keys_a,
                                                               reinterpret_cast<unsigned long long*>(sc + SC_NKEPT));
  CK(cudaGetLastError());
  uint64_t h[2];
  CK(cudaMemcpyAsync(h, sc + SC_NKEPT, 8, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(h + 1, sc + SC_STATUS, 8, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (h[1]) return fail(ctx, MCZI_ERR_DEVICE, "ZI key set overflow");
  const uint64_t n_keys = h[0];
  z.n_keys = n_keys;
  // the minimizer filter: a power of two of 64-bit words, >= n_keys / 2
  {
    uint64_t words = 1024;
    while (words * 2 < n_keys) words <<= 1;
    CKA(z.mfilter, words * 8);
    CK(cudaMemsetAsync(z.mfilter.p, 0, words * 8, s));
    z.mf_mask = words - 1;
    if (n_keys)
      k_zi_mfilter_set<<<grid_for(ctx, n_keys), ZI_THREADS, 0, s>>>(keys_a, n_keys,
                                                                     z.mfilter.as<unsigned long long>(), z.mf_mask);
    CK(cudaGetLastError());
  }
  // BBHash levels, gamma = 2
  const uint64_t max_bits = 4 * n_keys + 128ull * MPHF_MAX_LEVELS + 64;
  const uint64_t max_words = max_bits / 64 + 1;
  CKA(z.bits, max_words * 8);
  CK(cudaMemsetAsync(z.bits.p, 0, max_words * 8, s));
  CKA(ctx->zi_tmp2, max_words * 8);  // collision words of the current level
  uint64_t off = 0, rem = n_keys;
  int l = 0;
  while (rem > 0) {
    if (l >= MPHF_MAX_LEVELS) return fail(ctx, MCZI_ERR_DEVICE, "MPHF construction did not converge");
    const uint64_t size = ((std::max<uint64_t>(64, 2 * rem) + 63) / 64) * 64;
    if ((off + size) / 64 > max_words) return fail(ctx, MCZI_ERR_DEVICE, "MPHF bit vector overflow");
    unsigned long long* A = z.bits.as<unsigned long long>() + off / 64;
    unsigned long long* Cw = ctx->zi_tmp2.as<unsigned long long>();
    CK(cudaMemsetAsync(Cw, 0, size / 8, s));
    CK(cudaMemsetAsync(sc + SC_NKEPT, 0, 8, s));
    k_bb_mark<<<grid_for(ctx, rem), ZI_THREADS, 0, s>>>(keys_a, rem, l, size, A, Cw);
    k_bb_next<<<grid_for(ctx, rem), ZI_THREADS, 0, s>>>(keys_a, rem, l, size, Cw, keys_b,
                                                        reinterpret_cast<unsigned long long*>(sc + SC_NKEPT));
    k_bb_clear<<<grid_for(ctx, size / 64), ZI_THREADS, 0, s>>>(A, Cw, size / 64);
    CK(cudaGetLastError());
    uint64_t nn = 0;
    CK(cudaMemcpyAsync(&nn, sc + SC_NKEPT, 8, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    z.lvl_off[l] = off;
    z.lvl_size[l] = size;
    off += size;
    rem = nn;
    std::swap(keys_a, keys_b);
    l++;
  }
  z.levels = l;
  z.lvl_off[l] = off;
  z.n_words = off / 64 + 1;
  // rank: exclusive prefix of per-word popcounts
  CKA(z.rank, (z.n_words + 1) * 4);
  CKA(ctx->zi_tmp0, std::max<uint64_t>(slots * 8, (z.n_words + 1) * 4 + (z.n_words / SCAN_CHUNK + 2) * 4));
  uint32_t* pc = ctx->zi_tmp0.as<uint32_t>();
  uint32_t* tmp = pc + z.n_words + 1;
  k_bb_popc<<<grid_for(ctx, z.n_words), ZI_THREADS, 0, s>>>(z.bits.as<unsigned long long>(), z.n_words, pc);
  exclusive_scan<uint32_t, SumU32>(pc, z.rank.as<uint32_t>(), z.n_words, tmp, s);
  CK(cudaGetLastError());
  // buckets: CSR from MPHF index to superkmers
  const MphfView v = view_of(z);
  CKA(z.bucket_off, (n_keys + 2) * 4);
  CKA(z.bucket_key, std::max<uint64_t>(n_keys, 1) * 4);
  CKA(z.sk, std::max<uint64_t>(n_desc, 1) * 8);
  uint32_t* cnt = ctx->zi_tmp1.as<uint32_t>();  // reuse: n_keys + 1 <= 2 * n_desc words
  CKA(ctx->zi_tmp1, std::max<uint64_t>((n_keys + 2) * 4 * 2 + (n_keys / SCAN_CHUNK + 2) * 4, 16));
  cnt = ctx->zi_tmp1.as<uint32_t>();
  uint32_t* cursor = cnt + n_keys + 1;
  CK(cudaMemsetAsync(cnt, 0, (n_keys + 1) * 4, s));
  CK(cudaMemsetAsync(sc + SC_STATUS, 0, 8, s));
  if (n_desc) {
    k_zi_bucket_count<<<grid_for(ctx, n_desc), ZI_THREADS, 0, s>>>(d_key, n_desc, v, n_keys, cnt,
                                                                   reinterpret_cast<uint32_t*>(sc + SC_STATUS));
    exclusive_scan<uint32_t, SumU32>(cnt, z.bucket_off.as<uint32_t>(), n_keys, cursor + n_keys + 1, s);
    CK(cudaMemcpyAsync(cursor, z.bucket_off.p, (n_keys + 1) * 4, cudaMemcpyDeviceToDevice, s));
    k_zi_bucket_fill<<<grid_for(ctx, n_desc), ZI_THREADS, 0, s>>>(ctx->desc.as<uint64_t>(), d_key, n_desc, v, n_keys,
                                                                  cursor, z.sk.as<uint64_t>(),
                                                                  z.bucket_key.as<uint32_t>());
  } else {
    CK(cudaMemsetAsync(z.bucket_off.p, 0, 8, s));
  }
  CK(cudaGetLastError());
  CK(cudaEventRecord(e1, s));
  CK(cudaMemcpyAsync(h + 1, sc + SC_STATUS, 8, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (h[1] & ST_BAD_INDEX) return fail(ctx, MCZI_ERR_DEVICE, "MPHF missed an index key");
  CK(cudaEventElapsedTime(&z.build_ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  z.built = true;
  ctx->have_result = false;
  return MCZI_OK;
}

// absent k-mers of the staged queries; per_input: records carry input masks
// Absent runs (ctx->desc) -> deduplicated records (+ per-input masks).
// Records come out in bucket order; ZI's results are sets.
int32_t zi_dedup(mczi_ctx* ctx, Pipe& p, bool per_input, uint64_t absent_w, uint64_t* n_out) {
  ZiIndex& z = ctx->zi;
  cudaStream_t s = ctx->stream;
  uint64_t* sc = ctx->scalars.as<uint64_t>();
  const bool wide = z.k > 32;
  const int W = per_input ? (ctx->n_inputs + 63) / 64 : 0;
  if (absent_w >= 0xffffffffull) return fail(ctx, MCZI_ERR_TOO_LARGE, "more than 2^32 absent k-mers in one query");
  if (per_input && ctx->n_inputs > 65535) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "more than 65535 inputs in one batch");
  CK(cudaEventRecord(ctx->ev[2], s));
  const size_t keyb = wide ? 16 : 8;
  // dedup table: one CTA of 1024 threads per SM with the largest table that fits
  const size_t slotb = keyb + 8 * (size_t)W + 2;  // key, masks, list entry
  cudaFuncAttributes fa{};
  if (wide) cudaFuncGetAttributes(&fa, k_zi_bucket_dedup<K128>);
  else cudaFuncGetAttributes(&fa, k_zi_bucket_dedup<K64>);
  // two CTAs per SM
  const size_t per_cta = std::min((size_t)ctx->smem_optin, ctx->smem_per_sm / 2 - ctx->smem_reserved);
  const size_t budget = per_cta - fa.sharedSizeBytes - 64;
  // at most twice the records a CTA keeps in registers (the planned bucket size is half a table)
  const size_t reg_records = (size_t)DDD_THREADS * (wide ? dd_e<K128>() : dd_e<K64>());
  const uint32_t slots = (uint32_t)std::min<size_t>(std::min<size_t>((budget - 16) / slotb, 2 * reg_records), 1u << 20);
  if (slots < 2048) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "too many inputs for the ZI dedup table");
  const size_t smem = (((size_t)slots * keyb + 15) & ~(size_t)15) + (size_t)slots * 8 * W + (size_t)slots * 2;
  // final buckets of about half a table each, in one level (<= 8 bits) or two (<= 8 + 9)
  const uint64_t per_bucket = ctx->zi_bucket_records ? std::min<uint64_t>(ctx->zi_bucket_records, slots / 2) : slots / 2;
  int bits = 0;
  while (bits < DD_MAX_BITS && per_bucket << bits < absent_w) bits++;
  const int bits1 = std::min(bits, DD_MAX_BITS1), bits2 = bits - bits1;
  const uint32_t nb1 = 1u << bits1, nbf = 1u << bits;
  const uint64_t nh = (uint64_t)nb1 * DD_CTAS;
  const uint64_t ntmp = nh / SCAN_CHUNK + 2;
  const uint64_t cap = std::max<uint64_t>(absent_w, 1);
  CKA(ctx->zi_tmp0, (2 * nh + 2 + ntmp + (nb1 + 1) + (nbf + 1)) * 4);
  CKA(ctx->zi_tmp1, cap * keyb);
  if (W) CKA(ctx->zi_tmp2, cap * 2);
  if (bits2) {
    CKA(ctx->zi_tmp3, cap * keyb);
    if (W) CKA(ctx->zi_tmp4, cap * 2);
  }
  uint32_t* hist = ctx->zi_tmp0.as<uint32_t>();
  uint32_t* pre = hist + nh + 1;
  uint32_t* tmp = pre + nh + 1;
  uint32_t* off1 = tmp + ntmp;
  uint32_t* offf = off1 + nb1 + 1;
  CKA(ctx->out_lo, cap * 8);
  if (wide) CKA(ctx->out_hi, cap * 8);
  CKA(ctx->out_cnt, cap * 4);
  if (W) CKA(ctx->out_mask, cap * 8 * (uint64_t)W);
  CK(cudaMemsetAsync(sc + SC_NOUT, 0, 8, s));
  CK(cudaMemsetAsync(sc + SC_STATUS, 0, 8, s));
  CK(cudaMemsetAsync(sc + SC_WORK, 0, 8, s));
  ExpandArgs ea;
  ea.runs = ctx->desc.as<uint64_t>();
  ea.n_runs = p.n_desc;
  ea.packed = ctx->packed.as<uint32_t>();
  ea.input_base = ctx->input_base.as<uint64_t>();
  ea.n_inputs = ctx->n_inputs;
  ea.with_ids = W ? 1 : 0;
  ea.k = z.k;
  ea.bits1 = bits1;
  ea.hist = hist;
  ea.pre = pre;
  ea.keys_out = ctx->zi_tmp1.p;
  ea.ids_out = W ? ctx->zi_tmp2.as<uint16_t>() : nullptr;
  if (wide) k_zi_expand_count<K128, Roll128><<<DD_CTAS, DD_THREADS, 0, s>>>(ea);
  else k_zi_expand_count<K64, Roll64><<<DD_CTAS, DD_THREADS, 0, s>>>(ea);
  exclusive_scan<uint32_t, SumU32>(hist, pre, nh, tmp, s);
  if (wide) {
    CK(cudaFuncSetAttribute(k_zi_expand_scatter<K128, Roll128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)dd_tile_bytes<K128>()));
    k_zi_expand_scatter<K128, Roll128><<<DD_CTAS, DD_THREADS, dd_tile_bytes<K128>(), s>>>(ea);
  } else {
    CK(cudaFuncSetAttribute(k_zi_expand_scatter<K64, Roll64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)dd_tile_bytes<K64>()));
    k_zi_expand_scatter<K64, Roll64><<<DD_CTAS, DD_THREADS, dd_tile_bytes<K64>(), s>>>(ea);
  }
  k_zi_off1<<<1, 256, 0, s>>>(pre, (int)nb1, bits2 ? off1 : offf);
  const void* dkeys = ctx->zi_tmp1.p;
  const uint16_t* dids = W ? ctx->zi_tmp2.as<uint16_t>() : nullptr;
  p.launches += 6;
  if (bits2) {
    SplitArgs sa;
    sa.keys_in = ctx->zi_tmp1.p;
    sa.ids_in = dids;
    sa.off1 = off1;
    sa.bits1 = bits1;
    sa.bits2 = bits2;
    sa.keys_out = ctx->zi_tmp3.p;
    sa.ids_out = W ? ctx->zi_tmp4.as<uint16_t>() : nullptr;
    sa.off2 = offf;
    if (wide) {
      CK(cudaFuncSetAttribute(k_zi_split<K128, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)dd_split_tile_bytes<K128>()));
      k_zi_split<K128, 4><<<nb1, DDK_THREADS, dd_split_tile_bytes<K128>(), s>>>(sa);
    } else {
      CK(cudaFuncSetAttribute(k_zi_split<K64, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)dd_split_tile_bytes<K64>()));
      k_zi_split<K64, 8><<<nb1, DDK_THREADS, dd_split_tile_bytes<K64>(), s>>>(sa);
    }
    dkeys = ctx->zi_tmp3.p;
    dids = W ? ctx->zi_tmp4.as<uint16_t>() : nullptr;
    p.launches += 1;
  }
  CK(cudaGetLastError());
  CK(cudaEventRecord(ctx->ev[3], s));
  BucketDedupArgs da;
  da.keys = dkeys;
  da.ids = dids;
  da.off = offf;
  da.n_buckets = nbf;
  da.bits = bits;
  da.W = W;
  da.slots = slots;
  da.work = reinterpret_cast<unsigned int*>(sc + SC_WORK);
  da.out_lo = ctx->out_lo.as<uint64_t>();
  da.out_hi = wide ? ctx->out_hi.as<uint64_t>() : nullptr;
  da.out_count = ctx->out_cnt.as<uint32_t>();
  da.out_mask = W ? ctx->out_mask.as<unsigned long long>() : nullptr;
  da.n_out = reinterpret_cast<unsigned long long*>(sc + SC_NOUT);
  da.cap = cap;
  da.status = reinterpret_cast<uint32_t*>(sc + SC_STATUS);
  const unsigned grid = (unsigned)std::min<uint32_t>(nbf, (uint32_t)ctx->sm_count * 2);
  if (wide) {
    cudaFuncSetAttribute(k_zi_bucket_dedup<K128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_zi_bucket_dedup<K128><<<grid, DDD_THREADS, smem, s>>>(da);
  } else {
    cudaFuncSetAttribute(k_zi_bucket_dedup<K64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_zi_bucket_dedup<K64><<<grid, DDD_THREADS, smem, s>>>(da);
  }
  p.launches += 1;
  CK(cudaGetLastError());
  CK(cudaEventRecord(ctx->ev[4], s));
  uint64_t h[2];
  CK(cudaMemcpyAsync(h, sc + SC_NOUT, 8, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(h + 1, sc + SC_STATUS, 8, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (h[1] & (ST_TABLE_STUCK | ST_OUT_OVERFLOW)) return fail(ctx, MCZI_ERR_DEVICE, "ZI dedup could not place every k-mer");
  ctx->mask_words = W;
  ctx->cap_out = std::max(ctx->cap_out, cap);
  *n_out = h[0];
  return MCZI_OK;
}

int32_t zi_query(mczi_ctx* ctx, const mczi_input* q, size_t n, bool per_input, uint64_t* n_out) {
  ZiIndex& z = ctx->zi;
  if (!z.built) return fail(ctx, MCZI_ERR_STATE, "no ZI index: call mczi_zi_build first");
  int32_t rc;
  if (n == 0) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "at least one query FASTA is required");
  InputPlan pl;
  if ((rc = plan_inputs(ctx, q, n, pl))) return rc;
  if ((rc = stage_layout(ctx, pl, n))) return rc;
  ctx->have_result = false;
  ctx->mask_words = 0;
  for (int i = 0; i < N_PHASES; i++) ctx->phase_ms[i] = 0.f;
  std::memset(ctx->stats, 0, sizeof ctx->stats);
  cudaStream_t s = ctx->stream;
  Pipe p;
  if (streamed_worthwhile(ctx, pl)) {  // the copy overlaps the pack and the scan
    bool overflow = false;
    if ((rc = stream_pack_scan(ctx, q, n, pl, z.k, z.m, p, &overflow))) return rc;
    if (overflow && (rc = pipe_scan(ctx, p, z.k, z.m))) return rc;
  } else {
    if ((rc = copy_text_range(ctx, q, n, pl, 0, pl.text_len, s))) return rc;
    CK(cudaStreamSynchronize(s));
    ctx->staged = true;
    if ((rc = pipe_pack(ctx, p))) return rc;
    if ((rc = pipe_scan(ctx, p, z.k, z.m))) return rc;
  }
  const uint64_t n_query_sk = p.n_desc;
  uint64_t* sc = ctx->scalars.as<uint64_t>();
  // probe: absent-window runs into (desc2, key2)
  uint64_t cap = 2 * p.n_desc + 1024;
  uint64_t n_runs = 0, absent_w = 0;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaEventRecord(e0, s));
  for (int attempt = 0; attempt < 3 && p.n_desc; attempt++) {
    // (desc, key) hold the query superkmers being probed; the runs go to
    // (desc2, key2), which become the partition's input after the swap
    if (cap > p.desc_cap) p.desc_cap = cap;
    CKA(ctx->desc2, cap * 8);
    CKA(ctx->key2, cap * 4);
    CK(cudaMemsetAsync(sc + SC_NRUNS, 0, 8, s));
    CK(cudaMemsetAsync(sc + SC_NABSW, 0, 8, s));
    ProbeArgs pa;
    pa.qdesc = ctx->desc.as<uint64_t>();
    pa.qkey = ctx->key.as<uint32_t>();
    pa.n_q = reinterpret_cast<const unsigned long long*>(sc + SC_NDESC);
    pa.qpacked = ctx->packed.as<uint32_t>();
    pa.ipacked = z.packed.as<uint32_t>();
    pa.sk = z.sk.as<uint64_t>();
    pa.bucket_off = z.bucket_off.as<uint32_t>();
    pa.bucket_key = z.bucket_key.as<uint32_t>();
    pa.mfilter = z.mfilter.as<unsigned long long>();
    pa.mf_mask = z.mf_mask;
    pa.n_absent_windows = reinterpret_cast<unsigned long long*>(sc + SC_NABSW);
    pa.n_keys = z.n_keys;
    pa.v = view_of(z);
    pa.k = z.k;
    pa.out_desc = ctx->desc2.as<uint64_t>();
    pa.out_key = ctx->key2.as<uint32_t>();
    pa.n_runs = reinterpret_cast<unsigned long long*>(sc + SC_NRUNS);
    pa.cap = cap;
    const int grid = std::max<int>(1, std::min<int>(ctx->sm_count * 4, (int)((p.n_desc + PROBE_TILE - 1) / PROBE_TILE)));
    if (z.k <= 32) k_zi_probe<K64, Roll64><<<grid, ZI_THREADS, 0, s>>>(pa);
    else k_zi_probe<K128, Roll128><<<grid, ZI_THREADS, 0, s>>>(pa);
    p.launches += 1;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(&n_runs, sc + SC_NRUNS, 8, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(&absent_w, sc + SC_NABSW, 8, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (n_runs <= cap) break;
    cap = n_runs + 1024;
    if (attempt == 2) return fail(ctx, MCZI_ERR_DEVICE, "absent-run buffer overflow persisted");
  }
  CK(cudaEventRecord(e1, s));
  std::swap(ctx->desc, ctx->desc2);
  std::swap(ctx->key, ctx->key2);
  p.n_desc = n_runs;
  CK(cudaMemcpyAsync(sc + SC_NDESC, &p.n_desc, 8, cudaMemcpyHostToDevice, s));
  CK(cudaStreamSynchronize(s));
  float probe_ms = 0.f;
  CK(cudaEventElapsedTime(&probe_ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const int mode = per_input ? MCZI_MODE_PRESENCE : MCZI_MODE_ABUNDANCE;
  uint64_t out = 0;
  if ((rc = zi_dedup(ctx, p, per_input, absent_w, &out))) return rc;
  if ((rc = pipe_finish(ctx, p, mode, z.k, z.m, 0, out))) return rc;
  // phases for ZI: [0] pack, [1] scan, [2] expand into buckets, [3] bucket dedup, [4] probe
  ctx->phase_ms[1] -= probe_ms;
  ctx->phase_ms[4] = probe_ms;
  ctx->stats[1] = n_runs;
  ctx->stats[2] = n_query_sk;
  ctx->stats[6] = absent_w;
  if (n_out) *n_out = out;
  (void)p.n_desc_total;
  return MCZI_OK;
}

}  // namespace

}  // namespace mczi

using namespace mczi;

extern "C" {

int32_t mczi_zi_build(mczi_ctx* ctx, const uint8_t* index_fasta, uint64_t len, uint32_t k, uint32_t m) {
  if (!ctx) return MCZI_ERR_STATE;
  cudaSetDevice(ctx->device);
  return zi_build(ctx, index_fasta, len, k, m);
}

int32_t mczi_zi_query(mczi_ctx* ctx, const mczi_input* queries, size_t n, uint64_t* n_absent) {
  if (!ctx) return MCZI_ERR_STATE;
  cudaSetDevice(ctx->device);
  return zi_query(ctx, queries, n, false, n_absent);
}

int32_t mczi_zi_build_from_result(mczi_ctx* ctx, uint32_t m) {
  if (!ctx) return MCZI_ERR_STATE;
  if (!ctx->have_result) return fail(ctx, MCZI_ERR_STATE, "no result");
  const uint32_t k = (uint32_t)ctx->k;
  int32_t rc = zi_validate(ctx, k, m);
  if (rc) return rc;
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  const uint64_t n = ctx->n_out, nb = n * (uint64_t)k;
  if (n == 0) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "index FASTA did not contain any sequence of length >= k");
  ZiIndex& z = ctx->zi;
  z.built = false;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaEventRecord(e0, s));
  // the result's k-mers become the stream the dictionary is built from (the
  // staged inputs are replaced)
  const uint64_t pwords = nb / 16 + 8, fwords = nb / 32 + 8;
  CKA(ctx->packed, pwords * 4);
  CKA(ctx->fbits, fwords * 4);
  CKA(ctx->input_base, 16);
  const unsigned grid = (unsigned)std::min<uint64_t>((pwords + ZI_THREADS - 1) / ZI_THREADS, (uint64_t)ctx->sm_count * 16);
  k_kmers_to_stream<<<grid, ZI_THREADS, 0, s>>>(ctx->out_lo.as<uint64_t>(), k > 32 ? ctx->out_hi.as<uint64_t>() : nullptr,
                                                n, (int)k, ctx->packed.as<uint32_t>(), pwords, ctx->fbits.as<uint32_t>(),
                                                fwords);
  CK(cudaGetLastError());
  uint64_t* d_nb = ctx->input_base.as<uint64_t>();
  CK(cudaMemcpyAsync(d_nb, &nb, 8, cudaMemcpyHostToDevice, s));
  CK(cudaStreamSynchronize(s));
  ctx->staged = false;
  ctx->text_len = nb;
  ctx->have_result = false;
  Pipe p;
  p.d_nbases = d_nb;
  p.n_bases_host = nb;
  p.pwords = pwords;
  return zi_build_stream(ctx, p, nb, k, m, e0, e1);
}

int32_t mczi_zi_build_path(mczi_ctx* ctx, const char* index_path, uint32_t k, uint32_t m) {
  if (!ctx) return MCZI_ERR_STATE;
  if (!index_path) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "index path must not be NULL");
  std::vector<uint8_t> data;
  std::string e;
  // (a gzip file whose members carry their sizes stays compressed: decoded on the device)
  if (!read_input_file(index_path, &data, &e, true)) return fail(ctx, MCZI_ERR_IO, e);
  cudaSetDevice(ctx->device);
  return zi_build(ctx, data.data(), data.size(), k, m);
}

int32_t mczi_zi_query_paths(mczi_ctx* ctx, const char* const* query_paths, size_t n, uint64_t* n_absent) {
  if (!ctx) return MCZI_ERR_STATE;
  if (n == 0) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "at least one query FASTA is required");
  std::vector<std::vector<uint8_t>> data;
  std::string e;
  if (!read_input_files(query_paths, n, &data, &e, true)) return fail(ctx, MCZI_ERR_IO, e);
  std::vector<mczi_input> in(n);
  for (size_t i = 0; i < n; i++) in[i] = mczi_input{data[i].data(), data[i].size()};
  cudaSetDevice(ctx->device);
  return zi_query(ctx, in.data(), n, false, n_absent);
}

int32_t mczi_zi_query_per_input(mczi_ctx* ctx, const mczi_input* queries, size_t n, uint64_t* n_records) {
  if (!ctx) return MCZI_ERR_STATE;
  cudaSetDevice(ctx->device);
  return zi_query(ctx, queries, n, true, n_records);
}

int32_t mczi_zi_input_result(mczi_ctx* ctx, int32_t input, uint64_t* key_lo, uint64_t* key_hi, uint64_t cap,
                             uint64_t* n) {
  if (!ctx) return MCZI_ERR_STATE;
  if (!ctx->have_result || ctx->mask_words == 0) return fail(ctx, MCZI_ERR_STATE, "no per-input ZI result");
  if (input < 0 || input >= ctx->n_inputs) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "input index out of range");
  cudaSetDevice(ctx->device);
  const uint64_t nr = ctx->n_out;
  const int W = ctx->mask_words;
  std::vector<uint64_t> lo(nr), hi(ctx->k > 32 ? nr : 0), msk(nr * (uint64_t)W);
  if (nr) {
    CK(cudaMemcpyAsync(lo.data(), ctx->out_lo.p, nr * 8, cudaMemcpyDeviceToHost, ctx->stream));
    if (ctx->k > 32) CK(cudaMemcpyAsync(hi.data(), ctx->out_hi.p, nr * 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(msk.data(), ctx->out_mask.p, nr * 8 * W, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  std::vector<uint64_t> idx;
  for (uint64_t i = 0; i < nr; i++)
    if ((msk[i * W + (input >> 6)] >> (input & 63)) & 1ull) idx.push_back(i);
  if (ctx->k > 32)
    std::sort(idx.begin(), idx.end(), [&](uint64_t a, uint64_t b) { return hi[a] < hi[b] || (hi[a] == hi[b] && lo[a] < lo[b]); });
  else
    std::sort(idx.begin(), idx.end(), [&](uint64_t a, uint64_t b) { return lo[a] < lo[b]; });
  if (n) *n = idx.size();
  if (!key_lo) return MCZI_OK;
  if (cap < idx.size()) return fail(ctx, MCZI_ERR_STATE, "result buffer too small");
  for (size_t i = 0; i < idx.size(); i++) {
    key_lo[i] = lo[idx[i]];
    if (key_hi) key_hi[i] = ctx->k > 32 ? hi[idx[i]] : 0;
  }
  return MCZI_OK;
}

int32_t mczi_zi_result_masks(mczi_ctx* ctx, uint64_t* masks, uint64_t cap_words, int32_t* words_per_record) {
  if (!ctx) return MCZI_ERR_STATE;
  if (!ctx->have_result || ctx->mask_words == 0) return fail(ctx, MCZI_ERR_STATE, "no per-input ZI result");
  if (words_per_record) *words_per_record = ctx->mask_words;
  if (!masks) return MCZI_OK;
  const uint64_t need = ctx->n_out * (uint64_t)ctx->mask_words;
  if (cap_words < need) return fail(ctx, MCZI_ERR_STATE, "mask buffer too small");
  cudaSetDevice(ctx->device);
  if (need) {
    CK(cudaMemcpyAsync(masks, ctx->out_mask.p, need * 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  return MCZI_OK;
}

int32_t mczi_zi_batch_split(mczi_ctx* ctx, uint64_t* key_lo, uint64_t* key_hi, uint64_t* offsets, uint64_t cap,
                            uint64_t* total) {
  if (!ctx) return MCZI_ERR_STATE;
  if (!ctx->have_result || ctx->mask_words == 0) return fail(ctx, MCZI_ERR_STATE, "no per-input ZI result");
  const int ni = ctx->n_inputs;
  if (ni > SPLIT_MAX_INPUTS) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "more than 4096 inputs in one batch");
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  const uint64_t nr = ctx->n_out;
  const int W = ctx->mask_words;
  const bool wide = ctx->k > 32;
  // per-input sizes on the device (block-aggregated), offsets on the host
  CKA(ctx->zi_tmp0, ((size_t)ni + 1) * 8 * 2);
  unsigned long long* cnt = ctx->zi_tmp0.as<unsigned long long>();
  unsigned long long* cursor = cnt + ni + 1;
  CK(cudaMemsetAsync(cnt, 0, ((size_t)ni + 1) * 8, s));
  const unsigned blocks = (unsigned)((nr + SPLIT_CHUNK - 1) / SPLIT_CHUNK);
  if (nr) k_zi_split_count<<<blocks, ZI_THREADS, 0, s>>>(ctx->out_mask.as<unsigned long long>(), nr, W, ni, cnt);
  CK(cudaGetLastError());
  std::vector<uint64_t> off((size_t)ni + 1, 0);
  CK(cudaMemcpyAsync(off.data() + 1, cnt, (size_t)ni * 8, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  for (int i = 0; i < ni; i++) off[i + 1] += off[i];
  if (total) *total = off[ni];
  if (offsets) std::copy(off.begin(), off.end(), offsets);
  if (!key_lo) return MCZI_OK;
  if (cap < off[ni]) return fail(ctx, MCZI_ERR_STATE, "result buffer too small");
  if (off[ni] == 0) return MCZI_OK;
  CKA(ctx->zi_tmp1, off[ni] * 8 * (wide ? 2 : 1));
  uint64_t* dlo = ctx->zi_tmp1.as<uint64_t>();
  uint64_t* dhi = wide ? dlo + off[ni] : nullptr;
  CK(cudaMemcpyAsync(cursor, off.data(), (size_t)ni * 8, cudaMemcpyHostToDevice, s));
  k_zi_split_fill<<<blocks, ZI_THREADS, 0, s>>>(ctx->out_mask.as<unsigned long long>(), ctx->out_lo.as<uint64_t>(),
                                                wide ? ctx->out_hi.as<uint64_t>() : nullptr, nr, W, ni, cursor, dlo,
                                                dhi);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(key_lo, dlo, off[ni] * 8, cudaMemcpyDeviceToHost, s));
  if (key_hi) {
    if (wide) CK(cudaMemcpyAsync(key_hi, dhi, off[ni] * 8, cudaMemcpyDeviceToHost, s));
    else std::fill(key_hi, key_hi + off[ni], 0ull);
  }
  CK(cudaStreamSynchronize(s));
  return MCZI_OK;
}

int32_t mczi_zi_info(mczi_ctx* ctx, uint64_t* out, int32_t cap) {
  if (!ctx) return MCZI_ERR_STATE;
  const ZiIndex& z = ctx->zi;
  const uint64_t v[8] = {z.built ? 1ull : 0ull, (uint64_t)z.k, (uint64_t)z.m, z.n_bases, z.n_sk, z.n_keys,
                         (uint64_t)z.levels, (uint64_t)(z.build_ms * 1000.f)};
  const int32_t n = std::min<int32_t>(cap, 8);
  for (int32_t i = 0; i < n; i++) out[i] = v[i];
  return n;
}

}  // extern "C"
