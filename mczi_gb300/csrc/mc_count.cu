// mc_count.cu -- K5: per-partition canonical k-mer counting in shared memory
// with MC's strict `count > x` threshold.
//
// Replaces MC's phase-2/3 partition counters: the k <= 32 sort + run-length
// path (src/lib.rs:2512-2570), the u128 AHashMap path for k > 32
// (src/lib.rs:2400-2425, 3589-3614) and the fof per-dataset dedup + presence
// table (src/lib.rs:2213-2247, 4450-4522).
//
// A persistent CTA takes p1 buckets (4096) from a work counter; the last
// wave of buckets is handed out in parts by p2 bins.  For each bucket (or
// part) it histograms the window occupancy of the 2048 p2 bins, cuts its bins
// into rounds whose expected number of stored k-mers fits the shared-memory
// table (expected = occupancy x the distinct/occurrence ratio measured so far
// across the grid, at the target fill), and for every round: regenerates the
// canonical k-mers of the round's superkmers on chip (the k-mers never touch
// HBM), inserts them with shared-memory CAS, and emits the slots whose count
// passes the threshold, leaving the table empty.  A round in which a probe
// run exceeds PROBE_LIMIT slots is abandoned and split -- by bins while it
// spans several, then by k-mer hash range -- so the result never depends on
// the estimate.  Every k-mer of a bucket lands in exactly one round because
// the p2 bin and the hash range are functions of the canonical k-mer.
//
// Presence mode (fof): the table holds a bitmask of datasets per k-mer; the
// dataset of a superkmer is found from its base offset.  count = popcount.
#include "mczi_internal.h"
#include "mczi_common.cuh"

namespace mczi {

namespace {

constexpr int MAX_STACK = 48;
constexpr uint32_t PROBE_LIMIT = 256;
constexpr int MAX_THREADS = 1024;
constexpr uint32_t TAIL_PARTS = 4;  // parts of each bucket in the last wave (by p2 bins)
static_assert(NP2 % TAIL_PARTS == 0, "a part is a whole number of p2 bins");

// exclusive scan of one u32 per thread over the block (<= 1024 threads);
// `ws` is 32 words of shared scratch.  Ends with a barrier.
__device__ __forceinline__ uint32_t block_excl_scan_u32(uint32_t v, uint32_t* total, uint32_t* ws) {
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

template <class K>
struct KeyOps;

template <>
struct KeyOps<K64> {
  // 64-bit shared loads are single-copy atomic: only EMPTY needs the CAS
  static __device__ __forceinline__ bool maybe_partial(K64 c) { return c.v == ~0ull; }
  static __device__ __forceinline__ K64 cas(K64* p, K64 cmp, K64 val) {
    unsigned long long r = atomicCAS(reinterpret_cast<unsigned long long*>(p), (unsigned long long)cmp.v,
                                     (unsigned long long)val.v);
    return K64{(uint64_t)r};
  }
};

template <>
struct KeyOps<K128> {
  // a 16-byte load may observe half of a concurrent EMPTY -> key store; such
  // a value has an all-ones half, as EMPTY has
  static __device__ __forceinline__ bool maybe_partial(K128 c) { return c.lo == ~0ull || c.hi == ~0ull; }
  static __device__ __forceinline__ K128 cas(K128* p, K128 cmp, K128 val) { return atomicCAS(p, cmp, val); }
};

struct RoundRange {
  uint32_t bl, bh;   // p2 bins [bl, bh)
  uint32_t hlo, hhi; // k-mer hash range [hlo, hhi]
};

__device__ __forceinline__ uint32_t popc_words(const unsigned long long* m, int W) {
  uint32_t c = 0;
  for (int i = 0; i < W; i++) c += __popcll(m[i]);
  return c;
}

// Filtered rounds keep two bitmaps in shared memory.  The seen map is a
// blocked Bloom filter: a key sets two bits of one 32-bit word, and a window
// whose two bits were both set already is a repeat (or a collision).  Two
// bits per key cut the collision rate to about a third of one bit's at the
// densities the rounds run at.  The claimed map has one bit per 16-bit key
// code and is set for every key stored in the table, so that a first sight
// whose claimed bit is clear is known not to be stored.
//   seen map   : word from hash bits 20..51, bits from 52..56 and 57..61
//   key code   : hash bits 20..35, folded below 0xfffe (the per-window word
//                of fast rounds; 0xfffe and 0xffff mark repeats and done)
__device__ __forceinline__ bool seen_test_set(uint32_t* bmap, uint32_t bwords, uint64_t hv) {
  const uint32_t wi = (uint32_t)((((hv >> 20) & 0xffffffffull) * (uint64_t)bwords) >> 32);
  const uint32_t m = (1u << ((uint32_t)(hv >> 52) & 31u)) | (1u << ((uint32_t)(hv >> 57) & 31u));
  return (atomicOr(&bmap[wi], m) & m) == m;
}
__device__ __forceinline__ uint32_t key_code(uint64_t hv) {
  const uint32_t c = (uint32_t)(hv >> 20) & 0xffffu;
  return c >= 0xfffeu ? c - 2u : c;
}
__device__ __forceinline__ void claimed_set(uint32_t* cmap, uint32_t cbits, uint32_t code) {
  const uint32_t b = (code * cbits) >> 16;
  atomicOr(&cmap[b >> 5], 1u << (b & 31u));
}
__device__ __forceinline__ bool claimed_test(const uint32_t* cmap, uint32_t cbits, uint32_t code) {
  const uint32_t b = (code * cbits) >> 16;
  return (cmap[b >> 5] >> (b & 31u)) & 1u;
}

// per-window 16-bit word of the fast filtered rounds' scratch: the key code
// of a window seen for the first time in pass 1, W16_REPEAT for a repeat, or
// W16_DONE (outside the round's hash range, or past the end of its chunk)
constexpr uint32_t W16_DONE = 0xffffu;
constexpr uint32_t REP_LIST = 512;  // repeats a warp lists per round (more go through the records)
constexpr uint32_t W16_REPEAT = 0xfffeu;

// fast rounds' chunks: FAST_CH windows, one 16-bit word each in a record
constexpr uint32_t FAST_CH = COUNT_FAST_CHUNK;
constexpr uint32_t FAST_LOG = FAST_CH == 8 ? 3u : 2u;
struct __align__(2 * FAST_CH) ChunkWords {
  uint32_t w[FAST_CH / 2];
};

// chunk reference of the scratch: round-relative descriptor index << 10 |
// chunk within the descriptor (windows <= 4096, so < 1024 chunks)
__device__ __forceinline__ uint64_t chunk_pos(uint32_t ref, const uint64_t* rdesc) {
  return bd_start(rdesc[ref >> 10]) + (uint64_t)(ref & 1023u) * FAST_CH;
}

// dataset (input) of a base position: the largest i with dsbase[i] <= pos
__device__ __forceinline__ uint32_t dataset_of(const uint64_t* dsbase, int n, uint64_t pos) {
  int l = 0, h = n;
  while (h - l > 1) {
    const int mid = (l + h) >> 1;
    if (dsbase[mid] <= pos) l = mid;
    else h = mid;
  }
  return (uint32_t)l;
}

// the k-mer starting at base `pos` of the packed stream
template <class K, class R>
__device__ __forceinline__ void roll_at(R& roll, const uint32_t* __restrict__ packed, uint64_t pos, int k) {
  roll.init(k);
  if constexpr (sizeof(K) == 8) {
    roll.set(field64(packed, pos, k), k);
  } else {
    if (k > 32) roll.set(field64(packed, pos, k - 32), field64(packed, pos + (uint64_t)(k - 32), 32), k);
    else roll.set(0ull, field64(packed, pos, k), k);
  }
}

// looks key up from its home slot s: sub 1 counts it when stored (keys are
// final), sub 0 claims or counts it
template <class K, int MODE>
__device__ __forceinline__ void lookup_key(int sub, const K key, uint32_t s, uint32_t dset, K* keys, uint32_t* cnt,
                                           unsigned long long* msk, int W, uint32_t S, K EMPTY, uint32_t* s_over,
                                           uint32_t* claimed) {
  if (sub == 1) {
    // 2b: keys are final: plain loads, stop at EMPTY
    for (uint32_t probe = 0; probe < PROBE_LIMIT; probe++) {
      const K cur = keys[s];
      if (key_eq(cur, key)) {
        if (MODE == 0) atomicAdd(&cnt[s], 1u);
        else atomicOr(&msk[(size_t)s * W + (dset >> 6)], 1ull << (dset & 63));
        return;
      }
      if (key_eq(cur, EMPTY)) return;
      s = (s + 1 == S) ? 0u : s + 1;
    }
    return;
  }
  // 2a: claim-or-count, as the single pass (see k_count)
  for (uint32_t probe = 0; probe < PROBE_LIMIT; probe++) {
    K cur = keys[s];
    if (KeyOps<K>::maybe_partial(cur)) {
      const K prev = KeyOps<K>::cas(&keys[s], EMPTY, key);
      if (key_eq(prev, EMPTY)) {
        (*claimed)++;
        if (MODE == 1) atomicOr(&msk[(size_t)s * W + (dset >> 6)], 1ull << (dset & 63));
        return;
      }
      cur = prev;
    }
    if (key_eq(cur, key)) {
      if (MODE == 0) atomicAdd(&cnt[s], 1u);
      else atomicOr(&msk[(size_t)s * W + (dset >> 6)], 1ull << (dset & 63));
      return;
    }
    s = (s + 1 == S) ? 0u : s + 1;
  }
  *s_over = 1;  // table far past its target fill: the round is split
}

// the window whose k-mer starts at base `pos`, re-extracted from the stream
template <class K, class R, int MODE>
__device__ __forceinline__ void lookup_window(int sub, uint64_t pos, uint32_t dset,
                                              const uint32_t* __restrict__ packed, int k, K* keys, uint32_t* cnt,
                                              unsigned long long* msk, int W, uint32_t S, K EMPTY, uint32_t* s_over,
                                              uint32_t* claimed) {
  R roll;
  roll_at<K, R>(roll, packed, pos, k);
  const uint64_t hv = sym_hash(roll);
  const uint32_t s = (uint32_t)(((hv & 0xffffffffull) * (uint64_t)S) >> 32);
  lookup_key<K, MODE>(sub, roll.canon(), s, dset, keys, cnt, msk, W, S, EMPTY, s_over, claimed);
}

// exclusive prefix over the warp of a per-lane n < 2^NB, and the warp's
// total, from one ballot per bit of n (no chain of shuffles)
template <int NB>
__device__ __forceinline__ uint32_t warp_prefix_small(uint32_t n, uint32_t* total) {
  const uint32_t lt = (1u << (threadIdx.x & 31)) - 1u;
  uint32_t ex = 0, tot = 0;
#pragma unroll
  for (int b = 0; b < NB; b++) {
    const uint32_t bal = __ballot_sync(0xffffffffu, (n >> b) & 1u);
    ex += (uint32_t)__popc(bal & lt) << b;
    tot += (uint32_t)__popc(bal) << b;
  }
  *total = tot;
  return ex;
}

// Passes 2 and 3 of a fast filtered round.  Pass 2 stores or counts every
// repeat (claim-or-count; the claiming occurrence is implicit): first the
// warp's own list of repeats that pass 1 appended with their keys (no
// re-extraction, fast_claims), then the repeats whose list was full, found in
// the chunk records (fast_scan); the same scan lists the first sights whose
// claimed bit is set.  Pass 3 (fast_pass3), once every key is stored, counts
// each listed first sight whose key is in the table.  The scan reads 32
// consecutive records at a time (the next 32 already in flight) and gathers
// the record repeats into a register queue (two entries per lane); whenever
// 32 are queued all lanes look one up, so the rare lookups run with full
// warps instead of one or two lanes each.  Only windows looked up from the
// records are re-extracted from the packed stream.  Each warp keeps its own
// lists, so no shared counter is touched.  (Looking the first sights up
// inside the scan, when no list was full, measured slower: the lookups'
// dependent loads stall the scan.  So did taking two list entries per lane
// at a time.)
template <class K, int MODE>
__device__ __forceinline__ void fast_claims(const K* rl_keys, const uint32_t* rl_info, uint32_t nrep, K* keys,
                                            uint32_t* cnt, unsigned long long* msk, int W, uint32_t S, K EMPTY,
                                            uint32_t* s_over, uint32_t* claimed) {
  // the repeats pass 1 listed with their keys (slot | dataset << 16)
  for (uint32_t i = (uint32_t)(threadIdx.x & 31); i < nrep; i += 32) {
    const uint32_t inf = rl_info[i];
    lookup_key<K, MODE>(0, rl_keys[i], inf & 0xffffu, inf >> 16, keys, cnt, msk, W, S, EMPTY, s_over, claimed);
  }
}

template <class K, class R, int MODE>
__device__ __forceinline__ uint32_t fast_scan(const ChunkWords* words, const uint32_t* refs, uint32_t* list,
                                              uint32_t nchunks, const uint64_t* rdesc, const uint64_t* dsbase,
                                              int n_datasets, const uint32_t* __restrict__ packed, int k, K* keys,
                                              uint32_t* cnt, unsigned long long* msk, int W, uint32_t S,
                                              const uint32_t* cmap, uint32_t cbits, K EMPTY, uint32_t* s_over,
                                              uint32_t* claimed) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const uint32_t stride = (uint32_t)nw * 32u;
  uint64_t q0 = 0, q1 = 0;  // queued window positions: entries lane and 32 + lane
  uint32_t qn = 0;          // queued entries (warp-uniform)
  uint32_t ln = 0;          // entries in this warp's first-sight list (warp-uniform)
  uint32_t g = (uint32_t)wid * 32u;
  ChunkWords v;
#pragma unroll
  for (int i = 0; i < (int)FAST_CH / 2; i++) v.w[i] = 0xffffffffu;
  uint32_t ref = 0;
  if (g + (uint32_t)lane < nchunks) {
    v = words[g + lane];
    ref = refs[g + lane];
  }
  for (; g < nchunks; g += stride) {
    // the next group's records, in flight while this one is processed
    ChunkWords vn;
#pragma unroll
    for (int i = 0; i < (int)FAST_CH / 2; i++) vn.w[i] = 0xffffffffu;
    uint32_t rn = 0;
    if (g + stride + (uint32_t)lane < nchunks) {
      vn = words[g + stride + lane];
      rn = refs[g + stride + lane];
    }
    uint32_t m = 0, f = 0;  // record repeats; first sights whose claimed bit is set
#pragma unroll
    for (int j = 0; j < (int)FAST_CH; j++) {
      const uint32_t wj = (v.w[j >> 1] >> (16 * (j & 1))) & 0xffffu;
      m |= (wj == W16_REPEAT) ? (1u << j) : 0u;
      f |= (wj < W16_REPEAT && claimed_test(cmap, cbits, wj)) ? (1u << j) : 0u;
    }
    // the first sights to the warp's list
    {
      uint32_t nf;
      uint32_t at = ln + warp_prefix_small<FAST_LOG + 1>(__popc(f), &nf);
      for (uint32_t ff = f; ff; ff &= ff - 1) list[at++] = ((g + (uint32_t)lane) << FAST_LOG) | (uint32_t)(__ffs(ff) - 1);
      ln += nf;
    }
    // repeats that found their warp's list full, through the queue 32 at a
    // time (rare: most rounds have none)
    uint32_t total = 0, excl = 0, incl = 0;
    uint64_t base = 0;
    if (__any_sync(0xffffffffu, m != 0)) {
      base = m ? chunk_pos(ref, rdesc) : 0ull;
      excl = warp_prefix_small<FAST_LOG + 1>(__popc(m), &total);
      incl = excl + __popc(m);
    }
    for (uint32_t b0 = 0; b0 < total; b0 += 32) {
      const uint32_t t = b0 + (uint32_t)lane;
      // source lane of candidate t: the first lane whose inclusive count exceeds t
      int src = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const uint32_t x = __shfl_sync(0xffffffffu, incl, src + step - 1);
        if (x <= t) src += step;
      }
      const uint32_t ms = __shfl_sync(0xffffffffu, m, src & 31);
      const uint32_t es = __shfl_sync(0xffffffffu, excl, src & 31);
      const uint64_t bs = __shfl_sync(0xffffffffu, base, src & 31);
      const uint32_t gsz = min(32u, total - b0);
      uint64_t e = 0;
      if (t < total) e = bs + (uint64_t)(__fns(ms, 0, (int)(t - es) + 1));
      // entry i of this gather goes to queue position qn + i
      const uint64_t er = __shfl_sync(0xffffffffu, e, (lane - (int)qn) & 31);
      const uint32_t i = (uint32_t)((lane - (int)qn) & 31);
      if (i < gsz) {
        if ((uint32_t)lane >= qn) q0 = er;
        else q1 = er;
      }
      if (qn + gsz >= 32) {
        const uint32_t ds = MODE == 1 ? dataset_of(dsbase, n_datasets, q0) : 0u;
        lookup_window<K, R, MODE>(0, q0, ds, packed, k, keys, cnt, msk, W, S, EMPTY, s_over, claimed);
        q0 = q1;
        qn = qn + gsz - 32;
      } else {
        qn += gsz;
      }
    }
    v = vn;
    ref = rn;
  }
  if ((uint32_t)lane < qn) {
    const uint32_t ds = MODE == 1 ? dataset_of(dsbase, n_datasets, q0) : 0u;
    lookup_window<K, R, MODE>(0, q0, ds, packed, k, keys, cnt, msk, W, S, EMPTY, s_over, claimed);
  }
  return ln;
}

// pass 3: this warp's listed first sights, 32 lookups at a time
template <class K, class R, int MODE>
__device__ __forceinline__ void fast_pass3(const uint32_t* refs, const uint32_t* list, uint32_t ln,
                                           const uint64_t* rdesc, const uint64_t* dsbase,
                                           int n_datasets, const uint32_t* __restrict__ packed, int k, K* keys,
                                           uint32_t* cnt, unsigned long long* msk, int W, uint32_t S, K EMPTY,
                                           uint32_t* s_over, uint32_t* claimed) {
  const int lane = threadIdx.x & 31;
  for (uint32_t i = (uint32_t)lane; i < ln; i += 32) {
    const uint32_t e = list[i];
    const uint64_t pos = chunk_pos(refs[e >> FAST_LOG], rdesc) + (e & (FAST_CH - 1));
    const uint32_t ds = MODE == 1 ? dataset_of(dsbase, n_datasets, pos) : 0u;
    lookup_window<K, R, MODE>(1, pos, ds, packed, k, keys, cnt, msk, W, S, EMPTY, s_over, claimed);
  }
}

}  // namespace

size_t count_slot_bytes(int k, int mode, int n_datasets) {
  const size_t keyb = k <= 32 ? 8 : 16;
  const size_t valb = mode == 0 ? 4 : 8 * (size_t)((n_datasets + 63) / 64);
  return keyb + valb;
}

size_t count_fixed_smem_bytes(int mode, int n_datasets) {
  const size_t hist = 2 * (NP2 + 1) * sizeof(uint32_t) + (NP2 + 1) * sizeof(uint16_t);
  const size_t dsb = mode == 0 ? 0 : ((size_t)n_datasets + 1) * sizeof(uint64_t);
  return hist + dsb + 96;
}

size_t count_smem_bytes(int k, int mode, int n_datasets, uint32_t table_slots, uint32_t filter_words) {
  const size_t S = table_slots;
  const size_t keyb = k <= 32 ? 8 : 16;
  size_t b = S * keyb;
  b = (b + 15) & ~(size_t)15;
  b += S * (count_slot_bytes(k, mode, n_datasets) - keyb);
  b = (b + 15) & ~(size_t)15;
  b += (size_t)filter_words * 4;
  b = (b + 15) & ~(size_t)15;
  return b + count_fixed_smem_bytes(mode, n_datasets);
}

// KC > 0 compiles the kernel for one k (the shifts and masks of the rolling
// k-mer become constants); KC == 0 takes k from the arguments
template <class K, class R, int MODE, int KC>
__global__ void __launch_bounds__(MAX_THREADS, 1) k_count(CountArgs a) {
  extern __shared__ __align__(16) uint8_t smem[];
  const uint32_t S = a.table_slots;
  const int W = MODE == 0 ? 1 : (a.n_datasets + 63) / 64;
  K* keys = reinterpret_cast<K*>(smem);
  size_t off = ((size_t)S * sizeof(K) + 15) & ~(size_t)15;
  uint32_t* cnt = reinterpret_cast<uint32_t*>(smem + off);                     // MODE 0
  unsigned long long* msk = reinterpret_cast<unsigned long long*>(smem + off);  // MODE 1
  off += MODE == 0 ? (size_t)S * 4 : (size_t)S * 8 * W;
  off = (off + 15) & ~(size_t)15;
  const uint32_t fwords = a.filter_words;  // 0: single-pass rounds
  const bool filtered = fwords > 0;
  // filtered rounds: the seen-once bitmap (7/8 of the words) and a coarser
  // claimed-key bitmap (1/8) that lets pass 2 skip the table for keys pass 1
  // never stored (both indexed by the same 32 hash bits)
  const uint32_t cwords = filtered ? min(2048u, (fwords / 4) & ~31u) : 0u;
  const uint32_t cbits = cwords * 32u;
  const uint32_t bwords = fwords - cwords;
  const uint64_t fbits = (uint64_t)bwords * 32;
  uint32_t* bmap = reinterpret_cast<uint32_t*>(smem + off);
  uint32_t* cmap = bmap + bwords;
  // this CTA's per-window scratch of fast filtered rounds (L2-resident: a
  // round writes and re-reads only its own windows' words)
  // layout per CTA: per warp a list of REP_LIST repeats (keys, then u32
  // slot | dataset << 16), then per chunk of FAST_CH windows a record of
  // 16-bit window words (scr_chunks ChunkWords) and a u32 chunk reference
  // (scr_chunks of them, see chunk_pos), then one first-sight list of
  // scr_lcap u32 entries per warp (chunk << FAST_LOG | window)
  uint32_t* scr0 = (filtered && a.win_scratch) ? a.win_scratch + (size_t)blockIdx.x * a.scratch_words : nullptr;
  const uint32_t scr_nw = blockDim.x >> 5;
  const uint64_t rl_words = (uint64_t)scr_nw * REP_LIST * (sizeof(K) / 4 + 1);
  K* rl_keys = scr0 ? reinterpret_cast<K*>(scr0) + (size_t)(threadIdx.x >> 5) * REP_LIST : nullptr;
  uint32_t* rl_info =
      scr0 ? scr0 + (size_t)scr_nw * REP_LIST * (sizeof(K) / 4) + (size_t)(threadIdx.x >> 5) * REP_LIST : nullptr;
  uint32_t* scr = scr0 && a.scratch_words > rl_words + 4096ull * scr_nw + 64 ? scr0 + rl_words : nullptr;
  // words per chunk: its record, its reference and FAST_CH list entries (the
  // lists' rounding up to whole groups of 32 chunks per warp stays inside
  // the 4096 words per warp kept apart)
  constexpr uint32_t chunk_words = FAST_CH / 2 + 1 + FAST_CH;
  const uint32_t scr_chunks =
      scr ? (uint32_t)(((a.scratch_words - rl_words - 4096ull * scr_nw) / chunk_words) & ~3ull) : 0u;
  const uint32_t scr_lcap = ((scr_chunks + 32u * scr_nw - 1) / (32u * scr_nw)) * 32u * FAST_CH;
  ChunkWords* scr_words = reinterpret_cast<ChunkWords*>(scr);
  uint32_t* scr_refs = scr ? scr + (size_t)scr_chunks * (FAST_CH / 2) : nullptr;
  uint32_t* scr_list = scr ? scr + (size_t)scr_chunks * (FAST_CH / 2 + 1) : nullptr;
  off += (size_t)fwords * 4;
  off = (off + 15) & ~(size_t)15;
  uint32_t* occ = reinterpret_cast<uint32_t*>(smem + off);   // NP2 + 1, becomes occupancy prefix
  off += (NP2 + 1) * sizeof(uint32_t);
  uint32_t* dst = reinterpret_cast<uint32_t*>(smem + off);   // NP2 + 1, descriptor prefix
  off += (NP2 + 1) * sizeof(uint32_t);
  uint16_t* rstart = reinterpret_cast<uint16_t*>(smem + off);  // round start bins
  off += (NP2 + 1) * sizeof(uint16_t);
  off = (off + 7) & ~(size_t)7;
  uint64_t* dsbase = reinterpret_cast<uint64_t*>(smem + off);  // MODE 1

  __shared__ uint32_t s_bucket, s_nused, s_over, s_nrounds, s_sp;
  __shared__ unsigned long long s_bwin;
  __shared__ RoundRange stack[MAX_STACK];
  __shared__ uint32_t warp_tmp[32];
  __shared__ float s_rho;
  __shared__ uint32_t sh_cpre[MAX_THREADS + 1];
  __shared__ uint32_t sh_cpre32[MAX_THREADS / 32];
  __shared__ uint32_t s_cbase;  // chunks of the round's earlier batches
  __shared__ uint64_t sh_desc[MAX_THREADS];
  __shared__ uint16_t sh_dset[MODE == 1 ? MAX_THREADS : 1];
  const uint32_t chunk = a.chunk;

  const int tid = threadIdx.x, nth = blockDim.x;
  const int lane = tid & 31;
  const int k = KC > 0 ? KC : a.k;
  const K EMPTY = key_empty<K>();

  if (MODE == 1) {
    for (int i = tid; i <= a.n_datasets; i += nth) dsbase[i] = a.dataset_base[i];
  }
  // the table (keys and counts or masks) holds stale slots: true until a
  // round's emission has cleared every slot it visited, and again after a
  // round that overflowed (uniform over the CTA)
  bool table_dirty = true;

  for (;;) {
    __syncthreads();
    if (tid == 0) {
      s_bucket = atomicAdd(a.work_counter, 1u);
      const unsigned long long o = a.stats[0], d = a.stats[1];
      float rho = 1.0f;
      if (o > 200000ull) rho = fminf(1.0f, 1.3f * (float)d / (float)o + 0.02f);
      s_rho = rho;
    }
    __syncthreads();
    // Work units: buckets in order, except that the last gridDim.x buckets
    // are handed out as TAIL_PARTS parts each, part p taking the bucket's p2
    // bins [p, p + 1) * NP2 / TAIL_PARTS.  Buckets take about equal times,
    // so whole buckets to the end would leave part of the CTAs idle for up
    // to one bucket's time while the last wave finishes.
    const uint32_t tail_from = (uint32_t)NP1 > gridDim.x ? (uint32_t)NP1 - gridDim.x : 0u;
    const uint32_t unit = s_bucket;
    if (unit >= tail_from + ((uint32_t)NP1 - tail_from) * TAIL_PARTS) break;
    const bool whole = unit < tail_from;
    const uint32_t b = whole ? unit : tail_from + (unit - tail_from) / TAIL_PARTS;
    const int jlo = whole ? 0 : (int)((unit - tail_from) % TAIL_PARTS) * (NP2 / TAIL_PARTS);
    const int jhi = whole ? NP2 : jlo + NP2 / TAIL_PARTS;
    const uint64_t lo = a.bucket_off[b], hi = a.bucket_off[b + 1];
    if (hi <= lo) continue;
    // Descriptors of a batch are loaded ahead of their use: a round's next
    // batch while the current one's steps run, the next round's first batch
    // before this round's emission (otherwise every batch starts with the
    // full latency of its loads in front of a block scan).  pf_base is the
    // index in desc of the prefetched batch's first descriptor (uniform).
    uint64_t pf_base = ~0ull, pf_dsc = 0;
    auto prefetch = [&](uint64_t base) {
      pf_base = base;
      pf_dsc = base + (uint64_t)tid < hi ? a.desc[base + (uint64_t)tid] : 0ull;
    };

    // ---- per-bin occupancy and descriptor counts, and the bucket's total
    // windows in 64 bits: every 32-bit counter below (bin occupancy, its
    // prefix, a slot's count) is bounded by that total
    const uint64_t* src = a.desc_unsorted ? a.desc_unsorted : a.desc;
    for (int i = tid; i <= NP2; i += nth) { occ[i] = 0; dst[i] = 0; }
    if (tid == 0) s_bwin = 0;
    __syncthreads();
    uint64_t my_win = 0;
    for (uint64_t i = lo + tid; i < hi; i += nth) {
      const uint64_t bd = src[i];
      const uint32_t bin = bd_p2(bd);
      const uint32_t len = bd_windows(bd);
      atomicAdd(&occ[bin], len);
      atomicAdd(&dst[bin], 1u);
      my_win += len;
    }
    for (int o = 16; o > 0; o >>= 1) my_win += __shfl_xor_sync(0xffffffffu, my_win, o);
    if (lane == 0 && my_win) atomicAdd(&s_bwin, (unsigned long long)my_win);
    __syncthreads();
    if (s_bwin > a.max_bucket_windows) {
      if (tid == 0) set_status(a.status, ST_COUNT_WIDTH);
      continue;  // uniform: every thread read the same s_bwin
    }
    // exclusive prefix of both arrays (sequential chunks + warp scan)
    {
      const int per = (NP2 + nth - 1) / nth;
      const int base = tid * per;
      uint32_t so = 0, sd = 0;
      for (int i = 0; i < per; i++) {
        const int j = base + i;
        if (j < NP2) { so += occ[j]; sd += dst[j]; }
      }
      // block scan of (so, sd) via two passes of warp scans
      uint32_t vo = so, vd = sd;
      for (int o = 1; o < 32; o <<= 1) {
        uint32_t yo = __shfl_up_sync(0xffffffffu, vo, o);
        uint32_t yd = __shfl_up_sync(0xffffffffu, vd, o);
        if (lane >= o) { vo += yo; vd += yd; }
      }
      __shared__ uint32_t wo[32], wd[32];
      if (lane == 31) { wo[tid >> 5] = vo; wd[tid >> 5] = vd; }
      __syncthreads();
      if (tid < 32) {
        const int nw = nth / 32;
        uint32_t to = tid < nw ? wo[tid] : 0u, td = tid < nw ? wd[tid] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
          uint32_t yo = __shfl_up_sync(0xffffffffu, to, o);
          uint32_t yd = __shfl_up_sync(0xffffffffu, td, o);
          if (tid >= o) { to += yo; td += yd; }
        }
        wo[tid] = to;
        wd[tid] = td;
      }
      __syncthreads();
      uint32_t ro = vo - so + ((tid >> 5) ? wo[(tid >> 5) - 1] : 0u);
      uint32_t rd = vd - sd + ((tid >> 5) ? wd[(tid >> 5) - 1] : 0u);
      for (int i = 0; i < per; i++) {
        const int j = base + i;
        if (j < NP2) {
          const uint32_t co = occ[j], cd = dst[j];
          occ[j] = ro;
          dst[j] = rd;
          ro += co;
          rd += cd;
        }
      }
      __syncthreads();
      if (tid == nth - 1) { occ[NP2] = ro; dst[NP2] = rd; }
      __syncthreads();
    }
    if (a.desc_unsorted) {
      // partition pass 2 of this bucket: p2 order into `desc`, the bin starts
      // as cursors (afterwards dst[b] holds the start of bin b + 1)
      // (a part of a bucket writes only its own bins; every descriptor still
      // advances its bin's cursor, so the cursors end as in a whole bucket)
      uint64_t* out = const_cast<uint64_t*>(a.desc);
      for (uint64_t i = lo + tid; i < hi; i += nth) {
        const uint64_t bd = src[i];
        const uint32_t bin = bd_p2(bd);
        const uint32_t at = atomicAdd(&dst[bin], 1u);
        if ((int)bin >= jlo && (int)bin < jhi) out[lo + at] = bd;
      }
      __syncthreads();
      // shift back by one bin, top chunk first: a chunk reads only entries
      // below itself, which later (lower) chunks have not rewritten yet
      for (int top = NP2; top >= 0; top -= nth) {
        const int i = top - tid;
        const uint32_t v = (i > 0) ? dst[i - 1] : 0u;
        __syncthreads();
        if (i >= 0) dst[i] = v;
        __syncthreads();
      }
    }

    // ---- cut bins into rounds: round id of a bin = floor(occ_prefix / budget)
    // single pass: distinct keys of a round must fit the table; filtered:
    // only repeated keys are stored, and the bitmap holds >= 8 bits per window
    float budget_f = a.fill * (float)S / s_rho;
    if (filtered) budget_f = fminf(budget_f, (float)fbits / 8.0f);
    const uint32_t budget = budget_f < 1.0f ? 1u : (uint32_t)budget_f;
    if (tid == 0) s_nrounds = 0;
    __syncthreads();
    {
      // compaction of round starts, in bin order: warp ballots, chunked (a
      // part of a bucket plans its own bins only)
      for (int base = jlo; base < jhi; base += nth) {
        const int j = base + tid;
        bool st = false;
        if (j < jhi) st = (j == jlo) || (occ[j] / budget != occ[j - 1] / budget);
        const unsigned bal = __ballot_sync(0xffffffffu, st);
        if (lane == 0) warp_tmp[tid >> 5] = __popc(bal);
        __syncthreads();
        if (tid == 0) {
          uint32_t run = s_nrounds;
          for (int w2 = 0; w2 < nth / 32; w2++) { const uint32_t c = warp_tmp[w2]; warp_tmp[w2] = run; run += c; }
          s_nrounds = run;
        }
        __syncthreads();
        if (st) rstart[warp_tmp[tid >> 5] + __popc(bal & ((1u << lane) - 1u))] = (uint16_t)j;
        __syncthreads();
      }
    }
    const uint32_t nrounds = s_nrounds;

    for (uint32_t r = 0; r < nrounds; r++) {
      __syncthreads();
      if (tid == 0) {
        const uint32_t bl = rstart[r];
        const uint32_t bh = (r + 1 < nrounds) ? rstart[r + 1] : (uint32_t)jhi;
        stack[0] = RoundRange{bl, bh, 0u, 0xffffffffu};
        s_sp = 1;
      }
      __syncthreads();
      while (s_sp > 0) {
        __syncthreads();
        const RoundRange rr = stack[s_sp - 1];
        __syncthreads();
        if (tid == 0) { s_sp--; s_nused = 0; s_over = 0; }
        const uint32_t dlo = dst[rr.bl], dhi = dst[rr.bh];
        if (dhi == dlo) { __syncthreads(); continue; }
        // clear the table unless the last emission left it empty, and the
        // filter bitmaps (fwords is a multiple of 32 and bmap 16-byte aligned)
        if (table_dirty) {
          for (uint32_t i = tid; i < S; i += nth) {
            keys[i] = EMPTY;
            if (MODE == 0) cnt[i] = 0;
            else for (int q = 0; q < W; q++) msk[(size_t)i * W + q] = 0ull;
          }
        }
        for (uint32_t i = tid; i < fwords / 4; i += nth) reinterpret_cast<uint4*>(bmap)[i] = make_uint4(0u, 0u, 0u, 0u);
        __syncthreads();
        table_dirty = true;
        const bool full_range = (rr.hlo == 0u && rr.hhi == 0xffffffffu);
        uint32_t claimed = 0;  // slots this thread claimed in this round
        // ---- insert.  The round's superkmers are taken in batches of up to
        // blockDim descriptors; each is cut into chunks of `chunk` windows and
        // the chunks are spread over all threads, so long and short superkmers
        // keep every lane busy.  A chunk extracts its first k-mer from the
        // packed stream and rolls through the rest.
        //   single pass (ph 0): claim-or-count every window;
        //   filtered (ph 1, 2): pass 1 sets a window's two seen bits and
        //   claims a slot only when both were already set (a repeat -- or a
        //   collision, harmless).  A k-mer seen once is never stored, one seen
        //   twice or more always is, so for x >= 1 the emitted set and counts
        //   equal the single pass'.  Two ways to count the claimed keys:
        //   - fast (the round's chunks fit the CTA's scratch): pass 1 touches
        //     no table; it writes a 16-bit word per window (the key code of a
        //     first sight, W16_REPEAT for a repeat) and a reference per chunk
        //     to the scratch.  Pass 2 reads those records (no rolling), stores
        //     or counts every repeat and lists the first sights whose claimed
        //     bit is set; pass 3 counts the listed first sights whose key is
        //     stored.  Only the looked-up windows' k-mers are re-extracted,
        //     and the lookups run in full warps (fast_claims, fast_scan).  Every
        //     occurrence of a stored key is counted once: its claiming repeat
        //     implicitly, the other repeats in pass 2, the first sight in 3.
        //   - otherwise pass 1 claims the repeats and pass 2 re-rolls every
        //     window and counts every occurrence of the claimed keys.
        // a round of one batch keeps that batch's descriptors and chunk
        // prefixes in shared memory from pass 1 to pass 2
        const bool one_batch = dhi - dlo <= (uint64_t)nth;
        // chunks of the round <= (windows + descriptors * (chunk - 1)) / chunk
        const uint64_t round_windows = (uint64_t)(occ[rr.bh] - occ[rr.bl]);
        const bool fast = scr != nullptr && chunk == FAST_CH &&
                          (round_windows + (uint64_t)(dhi - dlo) * (FAST_CH - 1)) / FAST_CH <= scr_chunks &&
                          dhi - dlo < (1u << 22);  // chunk references: 22-bit descriptor index
        uint32_t total = 0;
        uint32_t rl_n = 0;  // repeats this warp appended to its list in pass 1 (warp-uniform)
        for (int ph = filtered ? 1 : 0; ph <= (filtered ? 2 : 0); ph++) {
          if (ph == 2 && fast) {
            // ---- passes 2 and 3 of a fast round, over its chunk records
            __syncthreads();
            const uint32_t nchunks = s_cbase;
            uint32_t* list = scr_list + (size_t)(tid >> 5) * scr_lcap;
            // a round of one batch still has its descriptors in shared memory
            const uint64_t* rdesc = one_batch ? sh_desc : a.desc + lo + dlo;
            fast_claims<K, MODE>(rl_keys, rl_info, min(rl_n, REP_LIST), keys, cnt, msk, W, S, EMPTY, &s_over,
                                 &claimed);
            const uint32_t ln = fast_scan<K, R, MODE>(scr_words, scr_refs, list, nchunks, rdesc, dsbase, a.n_datasets,
                                                      a.packed, k, keys, cnt, msk, W, S, cmap, cbits, EMPTY, &s_over,
                                                      &claimed);
            __syncthreads();
            if (!s_over)
              fast_pass3<K, R, MODE>(scr_refs, list, ln, rdesc, dsbase, a.n_datasets, a.packed, k, keys, cnt, msk, W,
                                     S, EMPTY, &s_over, &claimed);
            break;
          }
          if (tid == 0) s_cbase = 0;
          __syncthreads();
          for (uint64_t bb = dlo; bb < dhi; bb += (uint64_t)nth) {
            if (!(ph == 2 && one_batch)) {
              const bool has = bb + (uint64_t)tid < dhi;
              uint64_t dsc = 0;
              uint32_t nch = 0;
              if (has) {
                dsc = pf_base == lo + bb ? pf_dsc : a.desc[lo + bb + (uint64_t)tid];
                const uint32_t len = bd_windows(dsc);
                nch = (len + chunk - 1) / chunk;
                if (MODE == 1) {
                  const uint64_t s0 = bd_start(dsc);
                  int l2 = 0, h2 = a.n_datasets;  // largest i with dsbase[i] <= s0
                  while (h2 - l2 > 1) { const int mid = (l2 + h2) >> 1; if (dsbase[mid] <= s0) l2 = mid; else h2 = mid; }
                  sh_dset[tid] = (uint16_t)l2;
                }
              }
              sh_desc[tid] = dsc;
              const uint32_t cp = block_excl_scan_u32(nch, &total, warp_tmp);
              sh_cpre[tid] = cp;
              if (lane == 0) sh_cpre32[tid >> 5] = cp;
              if (tid == 0) sh_cpre[nth] = total;
              // the round's next batch is loaded while this one's steps run
              if (bb + (uint64_t)nth < dhi) prefetch(lo + bb + (uint64_t)nth);
              __syncthreads();
            }
            const int nd = (int)min((uint64_t)nth, dhi - bb);
            const uint32_t cbase = s_cbase;
            // Warps take steps of 32 chunks (one per lane) round-robin: step
            // t goes to warp t mod (warps), so a batch ends with at most one
            // step of imbalance.  (Handing steps out from a shared counter
            // serialised every step on one shared-memory address.)  The
            // descriptor of the step's first chunk comes from a two-level
            // 32-ary search (every 32nd prefix is kept apart, conflict-free);
            // every descriptor holds >= 1 chunk, so at most 32 descriptor
            // starts fall inside a step and a lane's descriptor is jw + (starts
            // at or before its chunk).
            for (uint32_t c0 = (uint32_t)(tid >> 5) * 32u;; c0 += (uint32_t)nth) {
              if (c0 >= total || __any_sync(0xffffffffu, *(volatile uint32_t*)&s_over)) break;
              const int i1 = lane << 5;
              const unsigned b1 = __ballot_sync(0xffffffffu, i1 < nd && sh_cpre32[lane] <= c0);
              const int seg = (31 - __clz(b1)) << 5;
              const int i2 = seg + lane;
              const unsigned b2 = __ballot_sync(0xffffffffu, i2 < nd && sh_cpre[i2] <= c0);
              const int jw = seg + 31 - __clz(b2);
              const int bi = jw + 1 + lane;
              const uint32_t rel = bi < nd ? sh_cpre[bi] - c0 : 0xffffffffu;  // >= 1
              const uint32_t starts = __reduce_or_sync(0xffffffffu, rel < 32u ? (1u << rel) : 0u);
              const int lo2 = jw + __popc(starts & (0xffffffffu >> (31 - lane)));
              const uint32_t cend = total;
              const uint32_t c = c0 + (uint32_t)lane;
              if (ph == 1 && fast) {
                // pass 1 of a fast round, in step for the whole warp (the
                // repeats are appended to the warp's list with one ballot per
                // window position): the windows' seen bits, a 16-bit word
                // per window and a reference per chunk in the scratch
                const bool has = c < cend;
                uint32_t nwin = 0, w0 = 0, dset = 0, q = 0, word = 0;
                uint64_t s0 = 0;
                const uint32_t* wp = a.packed;
                R roll;
                if (has) {
                  const uint64_t d2 = sh_desc[lo2];
                  w0 = (c - sh_cpre[lo2]) * FAST_CH;
                  nwin = min(FAST_CH, bd_windows(d2) - w0);
                  dset = MODE == 1 ? (uint32_t)sh_dset[lo2] : 0u;
                  s0 = bd_start(d2) + w0;
                  roll_at<K, R>(roll, a.packed, s0, k);
                  const uint64_t p = s0 + (uint64_t)k;
                  wp = a.packed + (p >> 4);
                  q = (uint32_t)(p & 15);
                  word = *wp << (2 * q);
                }
                uint32_t rw[FAST_CH / 2];  // the record's words, two windows each
#pragma unroll
                for (uint32_t jj = 0; jj < FAST_CH; jj++) {
                  bool repeat = false;
                  uint32_t v = W16_DONE, slot = 0;
                  K key = EMPTY;
                  if (jj < nwin) {
                    if (jj > 0) {
                      roll.push(word >> 30);
                      word <<= 2;
                      if (++q == 16) { q = 0; word = *++wp; }
                    }
                    const uint64_t hv = sym_hash(roll);
                    const uint32_t hk = (uint32_t)(hv >> 32);
                    if (full_range || (hk >= rr.hlo && hk <= rr.hhi)) {
                      const uint32_t hb = key_code(hv);
                      repeat = seen_test_set(bmap, bwords, hv);
                      v = hb;
                      if (repeat) {
                        claimed_set(cmap, cbits, hb);
                        key = roll.canon();
                        slot = (uint32_t)(((hv & 0xffffffffull) * (uint64_t)S) >> 32);
                        v = W16_REPEAT;
                      }
                    }
                  }
                  const unsigned bal = __ballot_sync(0xffffffffu, repeat);
                  if (bal) {
                    const uint32_t idx = rl_n + (uint32_t)__popc(bal & ((1u << lane) - 1u));
                    if (repeat && idx < REP_LIST) {
                      rl_keys[idx] = key;
                      rl_info[idx] = slot | (dset << 16);
                      v = W16_DONE;  // counted from the list in pass 2
                    }
                    rl_n += (uint32_t)__popc(bal);
                  }
                  if (jj & 1) rw[jj >> 1] |= v << 16;
                  else rw[jj >> 1] = v;
                }
                if (has) {
                  const uint32_t ci = cbase + c;
                  ChunkWords rec;
#pragma unroll
                  for (int i = 0; i < (int)FAST_CH / 2; i++) rec.w[i] = rw[i];
                  scr_words[ci] = rec;
                  scr_refs[ci] = ((uint32_t)(bb - dlo + (uint64_t)lo2) << 10) | (w0 >> FAST_LOG);
                }
                continue;
              }
              if (c >= cend) continue;
              const uint64_t d2 = sh_desc[lo2];
              const uint32_t len = bd_windows(d2);
              const uint32_t w0 = (c - sh_cpre[lo2]) * chunk;
              const uint32_t w1 = min(w0 + chunk, len);
              const uint32_t dset = MODE == 1 ? (uint32_t)sh_dset[lo2] : 0u;
              const uint64_t s0 = bd_start(d2) + w0;
              R roll;
              roll_at<K, R>(roll, a.packed, s0, k);
              // next base: the top two bits of `word` (pre-shifted), q = its
              // index inside the packed word at wp
              const uint64_t p = s0 + (uint64_t)k;
              const uint32_t* wp = a.packed + (p >> 4);
              uint32_t q = (uint32_t)(p & 15);
              uint32_t word = *wp << (2 * q);
              for (uint32_t j = w0; j < w1; j++) {
                if (j > w0) {
                  roll.push(word >> 30);
                  word <<= 2;
                  if (++q == 16) { q = 0; word = *++wp; }
                }
                // slot, filter bits and range come from the strand-symmetric
                // hash; the canonical key is formed only where the table is touched
                const uint64_t hv = sym_hash(roll);
                if (!full_range) {
                  const uint32_t hk = (uint32_t)(hv >> 32);
                  if (hk < rr.hlo || hk > rr.hhi) continue;  // its word stays W16_DONE
                }
                const uint32_t hb = key_code(hv);
                if (ph == 2) {
                  // slow pass 2: a key pass 1 never stored has its claimed bits clear
                  if (!claimed_test(cmap, cbits, hb)) continue;
                  const K key = roll.canon();
                  uint32_t s = (uint32_t)(((hv & 0xffffffffull) * (uint64_t)S) >> 32);
                  // keys are final during pass 2: plain loads, stop at EMPTY
                  for (uint32_t probe = 0; probe < PROBE_LIMIT; probe++) {
                    const K cur = keys[s];
                    if (key_eq(cur, key)) {
                      if (MODE == 0) atomicAdd(&cnt[s], 1u);
                      else atomicOr(&msk[(size_t)s * W + (dset >> 6)], 1ull << (dset & 63));
                      break;
                    }
                    if (key_eq(cur, EMPTY)) break;
                    s = (s + 1 == S) ? 0u : s + 1;
                  }
                  continue;
                }
                if (ph == 1) {
                  const bool repeat = seen_test_set(bmap, bwords, hv);
                  if (repeat) claimed_set(cmap, cbits, hb);  // stored below, or in pass 2
                  if (!repeat) continue;  // first sight: not stored
                }
                const bool count_here = ph == 0;
                const K key = roll.canon();
                uint32_t s = (uint32_t)(((hv & 0xffffffffull) * (uint64_t)S) >> 32);
                bool done = false;
                // Probe with plain loads; CAS only on a slot that looks empty.
                // A slot goes from EMPTY to a key exactly once, so a load that
                // shows a complete key (no all-ones half) is final; anything
                // else is resolved by the CAS's atomic snapshot.  The claiming
                // thread's own occurrence is implicit: a slot's stored count is
                // (occurrences counted here - 1).  A probe run longer than
                // PROBE_LIMIT means the table is far past its target fill: the
                // round is split.
                for (uint32_t probe = 0; probe < PROBE_LIMIT; probe++) {
                  K cur = keys[s];
                  if (KeyOps<K>::maybe_partial(cur)) {
                    const K prev = KeyOps<K>::cas(&keys[s], EMPTY, key);
                    if (key_eq(prev, EMPTY)) {
                      claimed++;
                      if (MODE == 1 && count_here) atomicOr(&msk[(size_t)s * W + (dset >> 6)], 1ull << (dset & 63));
                      done = true;
                      break;
                    }
                    cur = prev;
                  }
                  if (key_eq(cur, key)) {
                    if (count_here) {
                      if (MODE == 0) atomicAdd(&cnt[s], 1u);
                      else atomicOr(&msk[(size_t)s * W + (dset >> 6)], 1ull << (dset & 63));
                    }
                    done = true;
                    break;
                  }
                  s = (s + 1 == S) ? 0u : s + 1;
                }
                if (!done) { s_over = 1; break; }
              }
            }
            __syncthreads();
            if (tid == 0) s_cbase = cbase + total;
            if (s_over) break;
          }
          if (s_over) break;
        }
        // distinct keys of the round (for the distinct/occurrence estimate)
        for (int o = 16; o > 0; o >>= 1) claimed += __shfl_down_sync(0xffffffffu, claimed, o);
        if (lane == 0 && claimed) atomicAdd(&s_nused, claimed);
        __syncthreads();
        if (s_over) {
          if (tid == 0) {
            if (rr.bh - rr.bl > 1) {
              // split bins by occupancy midpoint
              const uint32_t target = (occ[rr.bl] + occ[rr.bh]) / 2;
              uint32_t mid = rr.bl + 1;
              while (mid < rr.bh - 1 && occ[mid + 1] <= target) mid++;
              if (s_sp + 2 <= MAX_STACK) {
                stack[s_sp++] = RoundRange{mid, rr.bh, rr.hlo, rr.hhi};
                stack[s_sp++] = RoundRange{rr.bl, mid, rr.hlo, rr.hhi};
              } else set_status(a.status, ST_TABLE_STUCK);
            } else if (rr.hhi > rr.hlo) {
              const uint32_t hm = rr.hlo + (rr.hhi - rr.hlo) / 2;
              if (s_sp + 2 <= MAX_STACK) {
                stack[s_sp++] = RoundRange{rr.bl, rr.bh, hm + 1, rr.hhi};
                stack[s_sp++] = RoundRange{rr.bl, rr.bh, rr.hlo, hm};
              } else set_status(a.status, ST_TABLE_STUCK);
            } else {
              set_status(a.status, ST_TABLE_STUCK);
            }
            atomicAdd(&a.stats[3], 1ull);
          }
          __syncthreads();
          continue;
        }
        // the next round's first batch (a split sub-round of this range, or
        // the next planned round), loaded while this round emits
        {
          const uint32_t nsp = s_sp;
          if (nsp > 0) prefetch(lo + dst[stack[nsp - 1].bl]);
          else if (r + 1 < nrounds) prefetch(lo + dst[rstart[r + 1]]);
        }
        // ---- emit slots with count > threshold, and empty the table.  A
        // thread owns slots tid, tid + nth, ... (as in the clear above).  Pass
        // A tests up to 32 of them, remembers the kept ones in a bit mask and
        // clears the others; each warp reserves its kept slots with one atomic
        // (whose latency is paid once per warp and group, not once per 32
        // slots); pass B writes the kept slots and clears them.
        {
          // the claiming occurrence is implicit except in slow filtered
          // rounds, whose pass 2 counts every occurrence
          const uint32_t implicit = (filtered && !fast) ? 0u : 1u;
          auto slot_count = [&](uint32_t s) -> uint32_t {
            return MODE == 0 ? cnt[s] + implicit : popc_words(&msk[(size_t)s * W], W);
          };
          auto slot_clear = [&](uint32_t s) {
            keys[s] = EMPTY;
            if (MODE == 0) cnt[s] = 0;
            else for (int q = 0; q < W; q++) msk[(size_t)s * W + q] = 0ull;
          };
          const uint32_t group = 32u * (uint32_t)nth;
          for (uint32_t g0 = 0; g0 < S; g0 += group) {
            uint32_t kept = 0;  // bit i: slot g0 + i * nth + tid is emitted
            for (uint32_t i = 0; i < 32u; i++) {
              const uint32_t s = g0 + i * (uint32_t)nth + (uint32_t)tid;
              if (g0 + i * (uint32_t)nth >= S) break;  // uniform
              if (s < S) {
                const K key = keys[s];
                if (!key_eq(key, EMPTY)) {
                  if ((uint64_t)slot_count(s) > a.threshold) kept |= 1u << i;
                  else slot_clear(s);
                }
              }
            }
            // this warp's emissions in the group, and the positions i at
            // which any of its lanes emits (both warp-uniform)
            const uint32_t mine = __reduce_add_sync(0xffffffffu, (uint32_t)__popc(kept));
            if (!mine) continue;
            uint32_t todo = __reduce_or_sync(0xffffffffu, kept);
            unsigned long long ob = 0;
            if (lane == 0) ob = atomicAdd(a.n_out, (unsigned long long)mine);
            ob = __shfl_sync(0xffffffffu, ob, 0);
            while (todo) {
              const uint32_t i = (uint32_t)__ffs(todo) - 1u;
              todo &= todo - 1u;
              const bool emit = (kept >> i) & 1u;
              const unsigned bal = __ballot_sync(0xffffffffu, emit);
              if (emit) {
                const uint32_t s = g0 + i * (uint32_t)nth + (uint32_t)tid;
                const K key = keys[s];
                const uint32_t c = slot_count(s);
                const unsigned long long idx = ob + __popc(bal & ((1u << lane) - 1u));
                if (idx < a.out_cap) {
                  if constexpr (sizeof(K) == 8) {
                    a.out_lo[idx] = reinterpret_cast<const K64&>(key).v;
                  } else {
                    a.out_lo[idx] = reinterpret_cast<const K128&>(key).lo;
                    a.out_hi[idx] = reinterpret_cast<const K128&>(key).hi;
                  }
                  a.out_count[idx] = c;
                  if (MODE == 1 && a.out_mask)
                    for (int q = 0; q < W; q++) a.out_mask[idx * W + q] = msk[(size_t)s * W + q];
                } else {
                  set_status(a.status, ST_OUT_OVERFLOW);
                }
                slot_clear(s);
              }
              ob += __popc(bal);
            }
          }
          table_dirty = false;
        }
        if (tid == 0) {
          // the round's windows times the share of the key hash range it
          // covered (span / 2^32; integer arithmetic: FP64 is slow here and
          // the whole CTA waits for this thread at the next barrier)
          const uint64_t span = (uint64_t)(rr.hhi - rr.hlo) + 1ull;  // <= 2^32
          atomicAdd(&a.stats[0], (unsigned long long)(((uint64_t)(occ[rr.bh] - occ[rr.bl]) * span) >> 32));
          atomicAdd(&a.stats[1], (unsigned long long)s_nused);
          atomicAdd(&a.stats[2], 1ull);
        }
        __syncthreads();
      }
    }
  }
}

template <class K, class R, int MODE, int KC>
static void launch_one(const CountArgs& a, cudaStream_t s) {
  const size_t smem = count_smem_bytes(a.k, a.mode, a.n_datasets, a.table_slots, a.filter_words);
  cudaFuncSetAttribute(k_count<K, R, MODE, KC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_count<K, R, MODE, KC><<<a.ctas, a.threads, smem, s>>>(a);
}

size_t count_static_smem(int k, int mode) {
  cudaFuncAttributes fa{};
  cudaError_t e;
  // every instantiation of a (key width, mode) has the same static shared memory
  if (k <= 32) e = mode == 0 ? cudaFuncGetAttributes(&fa, k_count<K64, Roll64, 0, 0>) : cudaFuncGetAttributes(&fa, k_count<K64, Roll64, 1, 0>);
  else e = mode == 0 ? cudaFuncGetAttributes(&fa, k_count<K128, Roll128, 0, 0>) : cudaFuncGetAttributes(&fa, k_count<K128, Roll128, 1, 0>);
  return e == cudaSuccess ? fa.sharedSizeBytes : 4096;
}

void launch_count(const CountArgs& a, cudaStream_t s) {
  if (a.k <= 32) {
    if (a.mode == 0) {
      if (a.k == 31) launch_one<K64, Roll64, 0, 31>(a, s);
      else launch_one<K64, Roll64, 0, 0>(a, s);
    } else {
      if (a.k == 31) launch_one<K64, Roll64, 1, 31>(a, s);
      else launch_one<K64, Roll64, 1, 0>(a, s);
    }
  } else {
    if (a.mode == 0) {
      if (a.k == 63) launch_one<K128, Roll128, 0, 63>(a, s);
      else launch_one<K128, Roll128, 0, 0>(a, s);
    } else {
      launch_one<K128, Roll128, 1, 0>(a, s);
    }
  }
}

}  // namespace mczi
