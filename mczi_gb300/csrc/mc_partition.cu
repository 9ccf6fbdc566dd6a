// mc_partition.cu -- K3: radix partition of superkmer descriptors into
// device buckets by their minimizer key.
//
// Replaces MC's superkmer partition writers (src/lib.rs:3483-3560,
// 4821-4925: partition = spread_hash_u32(minimizer) % P, one temp file per
// partition).  Here the buckets stay in HBM.  The key (mix32 of the minimizer
// value) is consumed as two digits (12 + 11 bits): this file groups the
// descriptors by p1 = key >> 20 (4096 buckets); the counting kernel groups
// each bucket by the next 11 bits (p2) itself before counting it, and carves
// the bucket into rounds of consecutive p2 bins.  Each superkmer becomes one
// u64 (start, windows, p2) here -- see bd_make.
#include "mczi_internal.h"
#include "mczi_common.cuh"

namespace mczi {

namespace {

constexpr int PART_U = 8;  // elements per thread per step

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

// ---- p1 in two tile-sorted levels.  Scattering every descriptor on its own into 4096
// buckets from 152 CTAs made 600 K write streams of single 8-byte stores; the
// store count, not DRAM, bounded it.  Instead: level A groups tiles of
// PT_TILE descriptors by the top PA_BITS of p1 in shared memory and writes
// each group as one piece (about 128 descriptors); level B does the same by
// the full p1 within those groups.  Each tile reserves its pieces from
// per-bucket cursors (global atomics, one per non-empty bin per tile), so
// no per-CTA offsets are needed; order inside a bucket does not matter.
constexpr int PA_BITS = 6;
constexpr int NPA = 1 << PA_BITS;
constexpr uint32_t PT_TILE = 8192;
constexpr int PT_E = (int)PT_TILE / PART_THREADS;
constexpr size_t PT_SMEM = (size_t)PT_TILE * (8 + 2);  // descriptor + p1 per element

__global__ void __launch_bounds__(PART_THREADS) k_part_hist_global(PartArgs a, uint32_t* __restrict__ ghist) {
  __shared__ uint32_t h[NP1];
  for (int i = threadIdx.x; i < NP1; i += PART_THREADS) h[i] = 0;
  __syncthreads();
  uint64_t n = *a.n_desc;
  if (n > a.desc_cap) n = a.desc_cap;
  uint64_t lo, hi;
  slice(n, lo, hi);
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
  for (int i = threadIdx.x; i < NP1; i += PART_THREADS)
    if (h[i]) atomicAdd(&ghist[i], h[i]);
}

// one CTA: bucket offsets (u64, NP1 + 1) and the cursors of both levels
__global__ void __launch_bounds__(PART_THREADS) k_part_bins(const uint32_t* __restrict__ ghist,
                                                            uint64_t* __restrict__ bucket_off,
                                                            uint32_t* __restrict__ cur_a, uint32_t* __restrict__ cur_b) {
  __shared__ uint32_t bins[NP1];
  __shared__ uint32_t total;
  for (int i = threadIdx.x; i < NP1; i += PART_THREADS) bins[i] = ghist[i];
  __syncthreads();
  smem_exclusive_scan<NP1>(bins, &total);
  for (int i = threadIdx.x; i < NP1; i += PART_THREADS) {
    bucket_off[i] = bins[i];
    cur_b[i] = bins[i];
    if ((i & (NPA - 1)) == 0) cur_a[i >> PA_BITS] = bins[i];
  }
  if (threadIdx.x == 0) bucket_off[NP1] = total;
}

// level A: descriptors of this CTA's slice -> (descriptor, p1) grouped by the
// top PA_BITS of p1
__global__ void __launch_bounds__(PART_THREADS) k_part_level_a(PartArgs a, uint32_t* __restrict__ cur_a,
                                                               uint16_t* __restrict__ tmp_p1) {
  extern __shared__ __align__(16) uint8_t smem[];
  uint64_t* sbd = reinterpret_cast<uint64_t*>(smem);
  uint16_t* sp1 = reinterpret_cast<uint16_t*>(sbd + PT_TILE);
  __shared__ uint32_t tcnt[NPA], tstart[NPA], gdst[NPA];
  const int tid = threadIdx.x;
  uint64_t n = *a.n_desc;
  if (n > a.desc_cap) n = a.desc_cap;
  uint64_t lo, hi;
  slice(n, lo, hi);
  if (tid < NPA) tcnt[tid] = 0;
  __syncthreads();
  for (uint64_t t0 = lo; t0 < hi; t0 += PT_TILE) {
    uint64_t bd[PT_E];
    uint16_t p1[PT_E];
    uint32_t rk[PT_E];
#pragma unroll
    for (int e = 0; e < PT_E; e++) {
      const uint64_t i = t0 + (uint64_t)e * PART_THREADS + tid;
      if (i < hi) {
        const uint64_t d = a.desc_in[i];
        const uint32_t key = a.key_in[i];
        p1[e] = (uint16_t)(key >> (32 - P1_BITS));
        // one u64 per superkmer from here on: the p1 digit is the bucket
        bd[e] = bd_make(d >> 24, (uint32_t)(d & 0xffffffu) + 1u, (key >> (32 - P1_BITS - P2_BITS)) & (NP2 - 1));
        rk[e] = atomicAdd(&tcnt[p1[e] >> (P1_BITS - PA_BITS)], 1u);
      }
    }
    __syncthreads();
    if (tid < 32) {  // 64 bins: two per lane, one warp scan
      const uint32_t c0 = tcnt[2 * tid], c1 = tcnt[2 * tid + 1];
      uint32_t x = c0 + c1;
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (tid >= o) x += y;
      }
      const uint32_t ex = x - c0 - c1;
      tstart[2 * tid] = ex;
      tstart[2 * tid + 1] = ex + c0;
      gdst[2 * tid] = c0 ? atomicAdd(&cur_a[2 * tid], c0) : 0u;
      gdst[2 * tid + 1] = c1 ? atomicAdd(&cur_a[2 * tid + 1], c1) : 0u;
    }
    __syncthreads();
#pragma unroll
    for (int e = 0; e < PT_E; e++) {
      const uint64_t i = t0 + (uint64_t)e * PART_THREADS + tid;
      if (i < hi) {
        const uint32_t pos = tstart[p1[e] >> (P1_BITS - PA_BITS)] + rk[e];
        sbd[pos] = bd[e];
        sp1[pos] = p1[e];
      }
    }
    __syncthreads();
    const uint32_t total = (uint32_t)(hi - t0 < PT_TILE ? hi - t0 : PT_TILE);
    for (uint32_t j = tid; j < total; j += PART_THREADS) {
      const uint32_t b = (uint32_t)sp1[j] >> (P1_BITS - PA_BITS);
      const uint32_t g = gdst[b] + (j - tstart[b]);
      a.desc_out[g] = sbd[j];
      tmp_p1[g] = sp1[j];
    }
    __syncthreads();
    if (tid < NPA) tcnt[tid] = 0;
    __syncthreads();
  }
}

// level B: (descriptor, p1) grouped by the top bits -> descriptors grouped by
// p1 at the bucket offsets
__global__ void __launch_bounds__(PART_THREADS) k_part_level_b(const uint64_t* __restrict__ tmp_bd,
                                                               const uint16_t* __restrict__ tmp_p1,
                                                               const unsigned long long* __restrict__ n_desc,
                                                               uint64_t desc_cap, uint32_t* __restrict__ cur_b,
                                                               uint64_t* __restrict__ out) {
  extern __shared__ __align__(16) uint8_t smem[];
  uint64_t* sbd = reinterpret_cast<uint64_t*>(smem);
  uint16_t* sp1 = reinterpret_cast<uint16_t*>(sbd + PT_TILE);
  __shared__ uint32_t tcnt[NP1], tstart[NP1], gdst[NP1];
  const int tid = threadIdx.x;
  uint64_t n = *n_desc;
  if (n > desc_cap) n = desc_cap;
  uint64_t lo, hi;
  slice(n, lo, hi);
  for (int b = tid; b < NP1; b += PART_THREADS) tcnt[b] = 0;
  __syncthreads();
  for (uint64_t t0 = lo; t0 < hi; t0 += PT_TILE) {
    uint64_t bd[PT_E];
    uint16_t p1[PT_E];
    uint32_t rk[PT_E];
#pragma unroll
    for (int e = 0; e < PT_E; e++) {
      const uint64_t i = t0 + (uint64_t)e * PART_THREADS + tid;
      if (i < hi) {
        bd[e] = tmp_bd[i];
        p1[e] = tmp_p1[i];
        rk[e] = atomicAdd(&tcnt[p1[e]], 1u);
      }
    }
    __syncthreads();
    for (int b = tid; b < NP1; b += PART_THREADS) tstart[b] = tcnt[b];
    __syncthreads();
    smem_exclusive_scan<NP1>(tstart, nullptr);
    for (int b = tid; b < NP1; b += PART_THREADS) {
      const uint32_t c = tcnt[b];
      gdst[b] = c ? atomicAdd(&cur_b[b], c) : 0u;
      tcnt[b] = 0;
    }
    __syncthreads();
#pragma unroll
    for (int e = 0; e < PT_E; e++) {
      const uint64_t i = t0 + (uint64_t)e * PART_THREADS + tid;
      if (i < hi) {
        const uint32_t pos = tstart[p1[e]] + rk[e];
        sbd[pos] = bd[e];
        sp1[pos] = p1[e];
      }
    }
    __syncthreads();
    const uint32_t total = (uint32_t)(hi - t0 < PT_TILE ? hi - t0 : PT_TILE);
    for (uint32_t j = tid; j < total; j += PART_THREADS) {
      const uint32_t b = sp1[j];
      out[gdst[b] + (j - tstart[b])] = sbd[j];
    }
    __syncthreads();
  }
}

void launch_partition_tiled(const PartArgs& a, uint32_t* scratch, uint16_t* tmp_p1, uint64_t* final_out,
                            cudaStream_t s) {
  uint32_t* ghist = scratch;
  uint32_t* cur_a = scratch + NP1;
  uint32_t* cur_b = cur_a + NPA;
  cudaMemsetAsync(ghist, 0, NP1 * sizeof(uint32_t), s);
  k_part_hist_global<<<PART_CTAS, PART_THREADS, 0, s>>>(a, ghist);
  k_part_bins<<<1, PART_THREADS, 0, s>>>(ghist, a.bucket_off, cur_a, cur_b);
  cudaFuncSetAttribute(k_part_level_a, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)PT_SMEM);
  k_part_level_a<<<PART_CTAS, PART_THREADS, PT_SMEM, s>>>(a, cur_a, tmp_p1);
  cudaFuncSetAttribute(k_part_level_b, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)PT_SMEM);
  k_part_level_b<<<PART_CTAS, PART_THREADS, PT_SMEM, s>>>(a.desc_out, tmp_p1, a.n_desc, a.desc_cap, cur_b, final_out);
}

}  // namespace mczi
