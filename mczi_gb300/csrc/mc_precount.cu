// mc_precount.cu -- K4: the pass-1 minimizer-count table and the superkmer
// filter it drives.
//
// Replaces MC's CompactMinimizerTable / ShardedMinimizerCounts
// (src/lib.rs:4171-4251, 4524-4564; filter MinimizerCounts::is_above_threshold
// :4625-4629) and, in fof mode, DatasetMinimizerTable (:4253-4370) with its
// once-per-dataset increments.  A superkmer is kept iff its minimizer's
// count is > x, where the count is the number of windows of all superkmers
// with that minimizer (abundance) or the number of datasets containing it
// (fof).  Every k-mer's own count is <= its minimizer's count, so the filter
// never removes a k-mer that passes the threshold; collisions of the 32-bit
// key only merge counts upwards.
//
// The table lives in HBM: open addressing over u64 slots holding
// key << 32 | value (0 = empty; a stored value is never 0).  Threads of a
// warp that carry the same key (or key+dataset pair) are merged with
// __match_any_sync first, so one atomic is issued per distinct key per warp.
#include "mczi_internal.h"
#include "mczi_common.cuh"

namespace mczi {

namespace {

constexpr int PC_THREADS = 256;

__device__ __forceinline__ uint64_t slot_of(uint64_t h, uint64_t mask) { return h & mask; }

// adds `delta` to key's counter (claims a slot on first sight); returns false
// if the table is full along the probe run
__device__ bool table_add(unsigned long long* tab, uint64_t mask, uint32_t key, uint32_t delta, bool* fresh) {
  uint64_t s = slot_of(mix64(key ^ 0x51ed270b27d0b5c1ull), mask);
  for (uint64_t probe = 0; probe <= mask; probe++) {
    unsigned long long cur = tab[s];
    if (cur == 0ull) {
      const unsigned long long want = ((unsigned long long)key << 32) | delta;
      const unsigned long long prev = atomicCAS(&tab[s], 0ull, want);
      if (prev == 0ull) { if (fresh) *fresh = true; return true; }
      cur = prev;
    }
    if ((uint32_t)(cur >> 32) == key) {
      atomicAdd(&tab[s], (unsigned long long)delta);
      if (fresh) *fresh = false;
      return true;
    }
    s = (s + 1) & mask;
  }
  return false;
}

__device__ uint32_t table_get(const unsigned long long* tab, uint64_t mask, uint32_t key) {
  uint64_t s = slot_of(mix64(key ^ 0x51ed270b27d0b5c1ull), mask);
  for (uint64_t probe = 0; probe <= mask; probe++) {
    const unsigned long long cur = tab[s];
    if (cur == 0ull) return 0;
    if ((uint32_t)(cur >> 32) == key) return (uint32_t)cur;
    s = (s + 1) & mask;
  }
  return 0;
}

__device__ __forceinline__ uint32_t dataset_of(const uint64_t* dsbase, int n, uint64_t s0) {
  int lo = 0, hi = n;  // largest i with dsbase[i] <= s0
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (dsbase[mid] <= s0) lo = mid;
    else hi = mid;
  }
  return (uint32_t)lo;
}

}  // namespace

// abundance: count[key] += windows, merged per warp
__global__ void __launch_bounds__(PC_THREADS) k_precount_abundance(PrecountArgs a) {
  const uint64_t n = *a.n_desc;
  for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < n; base += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = base + threadIdx.x;
    const bool has = i < n;
    const unsigned act = __ballot_sync(0xffffffffu, has);
    if (!has) continue;
    const uint32_t key = a.key[i];
    const uint32_t len = (uint32_t)(a.desc[i] & 0xffffffu) + 1u;
    const unsigned peers = __match_any_sync(act, key);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    uint32_t sum = 0;
    for (unsigned p = peers; p; p &= p - 1) sum += __shfl_sync(peers, len, __ffs(p) - 1);
    if (lane == leader && !table_add(a.table, a.mask, key, sum, nullptr)) set_status(a.status, ST_MINTAB_FULL);
  }
}

// fof: a (key, dataset) pair set gives the dataset-once flag; each fresh pair
// adds 1 to the key's dataset count
__global__ void __launch_bounds__(PC_THREADS) k_precount_presence(PrecountArgs a) {
  const uint64_t n = *a.n_desc;
  for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < n; base += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = base + threadIdx.x;
    const bool has = i < n;
    const unsigned act = __ballot_sync(0xffffffffu, has);
    if (!has) continue;
    const uint32_t key = a.key[i];
    const uint32_t ds = dataset_of(a.dataset_base, a.n_datasets, a.desc[i] >> 24);
    const unsigned long long pair = ((unsigned long long)key << 32) | ds;
    const unsigned peers = __match_any_sync(act, pair);
    if ((threadIdx.x & 31) != __ffs(peers) - 1) continue;
    // pair table slots hold key << 32 | (dataset + 1): a match needs both
    bool fresh = false;
    uint64_t s = mix64(((uint64_t)key << 32) | ds) & a.pair_mask;
    bool done = false;
    for (uint64_t probe = 0; probe <= a.pair_mask; probe++) {
      unsigned long long cur = a.pairs[s];
      const unsigned long long want = ((unsigned long long)key << 32) | (ds + 1u);
      if (cur == 0ull) {
        const unsigned long long prev = atomicCAS(&a.pairs[s], 0ull, want);
        if (prev == 0ull) { fresh = true; done = true; break; }
        cur = prev;
      }
      if (cur == want) { done = true; break; }
      s = (s + 1) & a.pair_mask;
    }
    if (!done) { set_status(a.status, ST_MINTAB_FULL); continue; }
    if (fresh && !table_add(a.table, a.mask, key, 1u, nullptr)) set_status(a.status, ST_MINTAB_FULL);
  }
}

// keep superkmers whose minimizer count > x: block-local compaction, one
// global atomic per CTA
__global__ void __launch_bounds__(PC_THREADS) k_precount_filter(PrecountArgs a) {
  __shared__ uint32_t warp_cnt[PC_THREADS / 32];
  __shared__ unsigned long long s_base;
  const uint64_t n = *a.n_desc;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < n; base += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = base + threadIdx.x;
    bool keep = false;
    uint64_t d = 0;
    uint32_t key = 0;
    if (i < n) {
      key = a.key[i];
      d = a.desc[i];
      keep = (uint64_t)table_get(a.table, a.mask, key) > a.threshold;
    }
    const unsigned bal = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) warp_cnt[wid] = __popc(bal);
    __syncthreads();
    if (threadIdx.x == 0) {
      uint32_t run = 0;
      for (int w = 0; w < PC_THREADS / 32; w++) { const uint32_t c = warp_cnt[w]; warp_cnt[w] = run; run += c; }
      s_base = atomicAdd(a.n_kept, (unsigned long long)run);
    }
    __syncthreads();
    if (keep) {
      const uint64_t o = s_base + warp_cnt[wid] + __popc(bal & ((1u << lane) - 1u));
      a.desc_out[o] = d;
      a.key_out[o] = key;
    }
    __syncthreads();
  }
}

void launch_precount(const PrecountArgs& a, int sm_count, cudaStream_t s) {
  const int grid = sm_count * 8;
  if (a.mode == 0) k_precount_abundance<<<grid, PC_THREADS, 0, s>>>(a);
  else k_precount_presence<<<grid, PC_THREADS, 0, s>>>(a);
  k_precount_filter<<<grid, PC_THREADS, 0, s>>>(a);
}

}  // namespace mczi
