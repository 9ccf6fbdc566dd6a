// mc_partition.cu -- K3: radix partition of superkmer descriptors into
// device buckets by their minimizer key.
//
// Replaces MC's superkmer partition writers (src/lib.rs:3483-3560,
// 4821-4925: partition = spread_hash_u32(minimizer) % P, one temp file per
// partition).  Here the buckets stay in HBM.  The key (mix32 of the minimizer
// value) is consumed as two digits (12 + 11 bits):
//   pass 1 (global): p1 = key >> 20.  A fixed grid of PART_CTAS CTAs each owns a
//           contiguous slice; per-CTA shared-memory histograms are written as
//           hist[p1][cta], scanned, and each CTA scatters its slice with
//           shared-memory cursors (no global atomics on the data path).
//   pass 2 (per bucket): p2 = the next 11 key bits, one CTA per p1 bucket,
//           histogram + scan + scatter inside the bucket's range, back into
//           the original buffers.
// The descriptors end up grouped by (p1, p2); the counting kernel carves
// each p1 bucket into rounds of consecutive p2 bins.  Pass 1 drops the key:
// each superkmer becomes one u64 (start, windows, p2) -- see bd_make.
#include "mczi_internal.h"
#include "mczi_common.cuh"
#include "scan.cuh"

namespace mczi {

namespace {

constexpr int PART_U = 8;  // elements per thread per step

struct SumU32 {
  static __device__ uint32_t identity() { return 0u; }
  static __device__ uint32_t combine(const uint32_t& a, const uint32_t& b) { return a + b; }
};

__device__ __forceinline__ void slice(uint64_t n, uint64_t& lo, uint64_t& hi) {
  const uint64_t per = (n + PART_CTAS - 1) / PART_CTAS;
  lo = per * blockIdx.x;
  hi = lo + per < n ? lo + per : n;
  if (lo > n) lo = n;
}

// exclusive scan of NB (multiple of blockDim) u32 bins in shared memory
template <int NB>
__device__ void smem_exclusive_scan(uint32_t* bins, uint32_t* total) {
  __shared__ uint32_t warp_tot[32];
  const int per = NB / PART_THREADS;
  const int base = threadIdx.x * per;
  uint32_t s = 0;
  for (int i = 0; i < per; i++) s += bins[base + i];
  // block exclusive scan of s
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t v = s;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += y;
  }
  if (lane == 31) warp_tot[wid] = v;
  __syncthreads();
  if (wid == 0) {
    uint32_t t = lane < PART_THREADS / 32 ? warp_tot[lane] : 0u;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    warp_tot[lane] = t;  // inclusive
  }
  __syncthreads();
  uint32_t run = v - s + (wid > 0 ? warp_tot[wid - 1] : 0u);
  if (total && threadIdx.x == PART_THREADS - 1) *total = run + s;
  for (int i = 0; i < per; i++) {
    uint32_t c = bins[base + i];
    bins[base + i] = run;
    run += c;
  }
  __syncthreads();
}

}  // namespace

__global__ void __launch_bounds__(PART_THREADS) k_part1_hist(PartArgs a) {
  __shared__ uint32_t h[NP1];
  for (int i = threadIdx.x; i < NP1; i += PART_THREADS) h[i] = 0;
  __syncthreads();
  uint64_t n = *a.n_desc;
  if (n > a.desc_cap) n = a.desc_cap;
  uint64_t lo, hi;
  slice(n, lo, hi);
  // U independent loads in flight per thread (the loop is latency-bound otherwise)
  for (uint64_t i0 = lo; i0 < hi; i0 += (uint64_t)PART_THREADS * PART_U) {
    uint32_t kk[PART_U];
#pragma unroll
    for (int u = 0; u < PART_U; u++) {
      const uint64_t i = i0 + (uint64_t)u * PART_THREADS + threadIdx.x;
      kk[u] = i < hi ? a.key_in[i] : 0u;
    }
#pragma unroll
    for (int u = 0; u < PART_U; u++) {
      const uint64_t i = i0 + (uint64_t)u * PART_THREADS + threadIdx.x;
      if (i < hi) atomicAdd(&h[kk[u] >> (32 - P1_BITS)], 1u);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < NP1; i += PART_THREADS) a.hist[(uint64_t)i * PART_CTAS + blockIdx.x] = h[i];
}

__global__ void k_part1_offsets(const uint32_t* __restrict__ pre, uint64_t* __restrict__ bucket_off) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= NP1; i += gridDim.x * blockDim.x)
    bucket_off[i] = pre[(uint64_t)i * PART_CTAS];  // pre[NP1 * PART_CTAS] is the total
}

__global__ void __launch_bounds__(PART_THREADS) k_part1_scatter(PartArgs a, const uint32_t* __restrict__ pre) {
  __shared__ uint32_t cur[NP1];
  for (int i = threadIdx.x; i < NP1; i += PART_THREADS) cur[i] = pre[(uint64_t)i * PART_CTAS + blockIdx.x];
  __syncthreads();
  uint64_t n = *a.n_desc;
  if (n > a.desc_cap) n = a.desc_cap;
  uint64_t lo, hi;
  slice(n, lo, hi);
  for (uint64_t i0 = lo; i0 < hi; i0 += (uint64_t)PART_THREADS * PART_U) {
    uint32_t kk[PART_U];
    uint64_t dd[PART_U];
#pragma unroll
    for (int u = 0; u < PART_U; u++) {
      const uint64_t i = i0 + (uint64_t)u * PART_THREADS + threadIdx.x;
      kk[u] = i < hi ? a.key_in[i] : 0u;
      dd[u] = i < hi ? a.desc_in[i] : 0ull;
    }
#pragma unroll
    for (int u = 0; u < PART_U; u++) {
      const uint64_t i = i0 + (uint64_t)u * PART_THREADS + threadIdx.x;
      if (i < hi) {
        const uint32_t pos = atomicAdd(&cur[kk[u] >> (32 - P1_BITS)], 1u);
        // one u64 per superkmer from here on: the p1 digit is the bucket
        a.desc_out[pos] = bd_make(dd[u] >> 24, (uint32_t)(dd[u] & 0xffffffu) + 1u,
                                  (kk[u] >> (32 - P1_BITS - P2_BITS)) & (NP2 - 1));
      }
    }
  }
}

// pass 2: one CTA per p1 bucket, from desc_out back to desc_in (u64 records)
__global__ void __launch_bounds__(PART_THREADS) k_part2(PartArgs a) {
  __shared__ uint32_t h[NP2];
  const int b = blockIdx.x;
  const uint64_t lo = a.bucket_off[b], hi = a.bucket_off[b + 1];
  if (hi <= lo) return;
  for (int i = threadIdx.x; i < NP2; i += PART_THREADS) h[i] = 0;
  __syncthreads();
  for (uint64_t i0 = lo; i0 < hi; i0 += (uint64_t)PART_THREADS * PART_U) {
    uint64_t dd[PART_U];
#pragma unroll
    for (int u = 0; u < PART_U; u++) {
      const uint64_t i = i0 + (uint64_t)u * PART_THREADS + threadIdx.x;
      dd[u] = i < hi ? a.desc_out[i] : 0ull;
    }
#pragma unroll
    for (int u = 0; u < PART_U; u++) {
      const uint64_t i = i0 + (uint64_t)u * PART_THREADS + threadIdx.x;
      if (i < hi) atomicAdd(&h[bd_p2(dd[u])], 1u);
    }
  }
  __syncthreads();
  smem_exclusive_scan<NP2>(h, nullptr);
  for (uint64_t i0 = lo; i0 < hi; i0 += (uint64_t)PART_THREADS * PART_U) {
    uint64_t dd[PART_U];
#pragma unroll
    for (int u = 0; u < PART_U; u++) {
      const uint64_t i = i0 + (uint64_t)u * PART_THREADS + threadIdx.x;
      dd[u] = i < hi ? a.desc_out[i] : 0ull;
    }
#pragma unroll
    for (int u = 0; u < PART_U; u++) {
      const uint64_t i = i0 + (uint64_t)u * PART_THREADS + threadIdx.x;
      if (i < hi) {
        const uint32_t pos = atomicAdd(&h[bd_p2(dd[u])], 1u);
        const_cast<uint64_t*>(a.desc_in)[lo + pos] = dd[u];
      }
    }
  }
}

void launch_partition(const PartArgs& a, cudaStream_t s, bool with_pass2) {
  k_part1_hist<<<PART_CTAS, PART_THREADS, 0, s>>>(a);
  const uint64_t nh = (uint64_t)NP1 * PART_CTAS;
  // scanned hist goes to hist + nh + 1 .. (exclusive; entry nh is the total)
  uint32_t* pre = a.hist + nh;
  exclusive_scan<uint32_t, SumU32>(a.hist, pre, nh, a.hist_tmp, s);
  k_part1_offsets<<<16, 256, 0, s>>>(pre, a.bucket_off);
  k_part1_scatter<<<PART_CTAS, PART_THREADS, 0, s>>>(a, pre);
  if (with_pass2) k_part2<<<NP1, PART_THREADS, 0, s>>>(a);
}

}  // namespace mczi
