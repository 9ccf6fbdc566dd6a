// mc_count.cu -- K5: per-partition canonical k-mer counting in shared memory
// with MC's strict `count > x` threshold.
//
// Replaces MC's phase-2/3 partition counters: the k <= 32 sort + run-length
// path (src/lib.rs:2512-2570), the u128 AHashMap path for k > 32
// (src/lib.rs:2400-2425, 3589-3614) and the fof per-dataset dedup + presence
// table (src/lib.rs:2213-2247, 4450-4522).
//
// A persistent CTA takes p1 buckets from a work counter.  For each bucket it
// histograms the window occupancy of the 4096 p2 bins, cuts the bins into
// rounds whose expected number of distinct k-mers fits the shared-memory
// table (expected = occupancy x the distinct/occurrence ratio measured so far
// across the grid), and for every round: clears the table, regenerates the
// canonical k-mers of the round's superkmers on chip (the k-mers never touch
// HBM), inserts them with shared-memory CAS, and emits the slots whose count
// passes the threshold.  A round whose table fills past 85 % is abandoned and
// split -- by bins while it spans several, then by k-mer hash range -- so the
// result never depends on the estimate.  Every k-mer of a bucket lands in
// exactly one round because the p2 bin and the hash range are functions of
// the canonical k-mer.
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
__global__ void k_count(CountArgs a) {
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
  const uint32_t cwords = filtered ? ((fwords / 8) & ~31u) : 0u;
  const uint64_t fbits = (uint64_t)(fwords - cwords) * 32, cbits = (uint64_t)cwords * 32;
  uint32_t* bmap = reinterpret_cast<uint32_t*>(smem + off);
  uint32_t* cmap = bmap + (fwords - cwords);
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
  __shared__ uint32_t s_step;
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
    const uint32_t b = s_bucket;
    if (b >= (uint32_t)NP1) break;
    const uint64_t lo = a.bucket_off[b], hi = a.bucket_off[b + 1];
    if (hi <= lo) continue;

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
      uint64_t* out = const_cast<uint64_t*>(a.desc);
      for (uint64_t i = lo + tid; i < hi; i += nth) {
        const uint64_t bd = src[i];
        out[lo + atomicAdd(&dst[bd_p2(bd)], 1u)] = bd;
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
      // compaction of round starts, in bin order: warp ballots, chunked
      for (int base = 0; base < NP2; base += nth) {
        const int j = base + tid;
        bool st = false;
        if (j < NP2) st = (j == 0) || (occ[j] / budget != occ[j - 1] / budget);
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
        const uint32_t bh = (r + 1 < nrounds) ? rstart[r + 1] : (uint32_t)NP2;
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
        // clear the table (and the filter bitmap)
        for (uint32_t i = tid; i < S; i += nth) {
          keys[i] = EMPTY;
          if (MODE == 0) cnt[i] = 0;
          else for (int q = 0; q < W; q++) msk[(size_t)i * W + q] = 0ull;
        }
        for (uint32_t i = tid; i < fwords; i += nth) bmap[i] = 0u;
        __syncthreads();
        const bool full_range = (rr.hlo == 0u && rr.hhi == 0xffffffffu);
        uint32_t claimed = 0;  // slots this thread claimed in this round
        // ---- insert.  The round's superkmers are taken in batches of up to
        // blockDim descriptors; each is cut into chunks of `chunk` windows and
        // the chunks are spread over all threads, so long and short superkmers
        // keep every lane busy.  A chunk extracts its first k-mer from the
        // packed stream and rolls through the rest.
        //   single pass (ph 0): claim-or-count every window;
        //   filtered (ph 1, 2): pass 1 sets one bitmap bit per window and claims
        //   a slot only when the bit was already set (a repeat -- or a bitmap
        //   collision, harmless); pass 2 counts every occurrence of the claimed
        //   keys with plain-load lookups.  A k-mer seen once is never stored,
        //   and a k-mer seen twice or more always is, so for x >= 1 the
        //   emitted set and counts are the same as the single pass.
        // a round of one batch keeps that batch's descriptors and chunk
        // prefixes in shared memory from pass 1 to pass 2
        const bool one_batch = dhi - dlo <= (uint64_t)nth;
        uint32_t total = 0;
        for (int ph = filtered ? 1 : 0; ph <= (filtered ? 2 : 0); ph++) {
          if (ph == 2) {
            if (one_batch && tid == 0) s_step = 0;
            __syncthreads();
          }
          for (uint64_t bb = dlo; bb < dhi; bb += (uint64_t)nth) {
            if (!(ph == 2 && one_batch)) {
              const bool has = bb + (uint64_t)tid < dhi;
              uint64_t dsc = 0;
              uint32_t nch = 0;
              if (has) {
                dsc = a.desc[lo + bb + (uint64_t)tid];
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
              if (tid == 0) s_step = 0;  // the previous batch's steps all ended before its closing barrier
              const uint32_t cp = block_excl_scan_u32(nch, &total, warp_tmp);
              sh_cpre[tid] = cp;
              if (lane == 0) sh_cpre32[tid >> 5] = cp;
              if (tid == 0) sh_cpre[nth] = total;
              __syncthreads();
            }
            const int nd = (int)min((uint64_t)nth, dhi - bb);
            // Warps take steps of 32 chunks (one per lane) from a shared
            // counter, so a batch ends with at most one step of imbalance.  The
            // descriptor of the step's first chunk comes from a two-level
            // 32-ary search (every 32nd prefix is kept apart, conflict-free);
            // every descriptor holds >= 1 chunk, so at most 32 descriptor
            // starts fall inside a step and a lane's descriptor is jw + (starts
            // at or before its chunk).
            for (;;) {
              uint32_t c0 = 0;
              if (lane == 0) c0 = atomicAdd(&s_step, 32u);
              c0 = __shfl_sync(0xffffffffu, c0, 0);
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
              if (c >= cend) continue;
              const uint64_t d2 = sh_desc[lo2];
              const uint32_t len = bd_windows(d2);
              const uint32_t w0 = (c - sh_cpre[lo2]) * chunk;
              const uint32_t w1 = min(w0 + chunk, len);
              const uint32_t dset = MODE == 1 ? (uint32_t)sh_dset[lo2] : 0u;
              const uint64_t s0 = bd_start(d2) + w0;
              R roll;
              roll.init(k);
              if constexpr (sizeof(K) == 8) {
                roll.set(field64(a.packed, s0, k), k);
              } else {
                if (k > 32) roll.set(field64(a.packed, s0, k - 32), field64(a.packed, s0 + (uint64_t)(k - 32), 32), k);
                else roll.set(0ull, field64(a.packed, s0, k), k);
              }
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
                // slot, bitmap position and range come from the strand-symmetric
                // hash; the canonical key is formed only where the table is touched
                const uint64_t hv = sym_hash(roll);
                if (!full_range) {
                  const uint32_t hk = (uint32_t)(hv >> 32);
                  if (hk < rr.hlo || hk > rr.hhi) continue;
                }
                // bitmap positions from hash bits 20..51 (the slot uses the low
                // 32 bits, range splits bits 32..63)
                const uint64_t hb = (hv >> 20) & 0xffffffffull;
                if (ph == 2) {
                  // a key pass 1 never stored has its claimed bit clear
                  const uint32_t cp = (uint32_t)((hb * cbits) >> 32);
                  if (!((cmap[cp >> 5] >> (cp & 31)) & 1u)) continue;
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
                  const uint32_t bp = (uint32_t)((hb * fbits) >> 32);
                  const uint32_t bit = 1u << (bp & 31);
                  if (!(atomicOr(&bmap[bp >> 5], bit) & bit)) continue;  // first sight: not stored
                  const uint32_t cp = (uint32_t)((hb * cbits) >> 32);
                  atomicOr(&cmap[cp >> 5], 1u << (cp & 31));  // stored (below) or already stored
                }
                const K key = roll.canon();
                uint32_t s = (uint32_t)(((hv & 0xffffffffull) * (uint64_t)S) >> 32);
                bool done = false;
                // Probe with plain loads; CAS only on a slot that looks empty.
                // A slot goes from EMPTY to a key exactly once, so a load that
                // shows a complete key (no all-ones half) is final; anything
                // else is resolved by the CAS's atomic snapshot.  In the single
                // pass the claiming thread's own occurrence is implicit: a
                // slot's stored count is (occurrences - 1).  A probe run longer
                // than PROBE_LIMIT means the table is far past its target
                // fill: the round is split.
                for (uint32_t probe = 0; probe < PROBE_LIMIT; probe++) {
                  K cur = keys[s];
                  if (KeyOps<K>::maybe_partial(cur)) {
                    const K prev = KeyOps<K>::cas(&keys[s], EMPTY, key);
                    if (key_eq(prev, EMPTY)) {
                      claimed++;
                      if (MODE == 1 && ph == 0) atomicOr(&msk[(size_t)s * W + (dset >> 6)], 1ull << (dset & 63));
                      done = true;
                      break;
                    }
                    cur = prev;
                  }
                  if (key_eq(cur, key)) {
                    if (ph == 0) {
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
        // ---- emit slots with count > threshold
        for (uint32_t base = 0; base < S; base += nth) {
          const uint32_t s = base + tid;
          bool emit = false;
          uint32_t c = 0;
          K key = EMPTY;
          if (s < S) {
            key = keys[s];
            if (!key_eq(key, EMPTY)) {
              c = MODE == 0 ? cnt[s] + (filtered ? 0u : 1u) : popc_words(&msk[(size_t)s * W], W);
              emit = (uint64_t)c > a.threshold;
            }
          }
          const unsigned bal = __ballot_sync(0xffffffffu, emit);
          if (bal) {
            unsigned long long ob = 0;
            const int leader = __ffs(bal) - 1;
            if (lane == leader) ob = atomicAdd(a.n_out, (unsigned long long)__popc(bal));
            ob = __shfl_sync(0xffffffffu, ob, leader);
            if (emit) {
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
            }
          }
        }
        if (tid == 0) {
          const double frac = ((double)rr.hhi - (double)rr.hlo + 1.0) / 4294967296.0;
          atomicAdd(&a.stats[0], (unsigned long long)((double)(occ[rr.bh] - occ[rr.bl]) * frac));
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
