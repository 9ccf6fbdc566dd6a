// simplitig.cu -- the device half of the simplitig FASTA writer.
//
// MC's simplitig output (src/lib.rs:1478-1613) is a greedy walk: seeds in
// ascending canonical order; from each unused seed extend to the right by
// the first of A, C, G, T whose canonical k-mer is still unused, then
// reverse-complement the path and extend again.  The walk is sequential and
// its output is defined by that order, so it stays on the host.  What made
// it slow is that every candidate was rebuilt from the path string and looked
// up in a host hash set.  Here the device computes, once and in parallel, for
// every kept k-mer (by rank in ascending order) and both of its orientations,
// the rank and orientation of each of its four right extensions that are in
// the set; the host walk then only follows these entries.
//
// Entry (i, o, b), o = 0 for the canonical string and 1 for its reverse
// complement, b the appended base (A0 C1 G2 T3): (j << 1 | o') where k-mer j
// in orientation o' is the extended string, or SIMPLITIG_NO_EXT
// (SIMPLITIG_STRIDE words per key).
#include "api_internal.h"
#include "host_io.h"
#include "mczi_common.cuh"

#include <algorithm>

namespace mczi {

namespace {

typedef unsigned __int128 u128;

constexpr int SX_THREADS = 256;

__device__ __forceinline__ u128 make128(uint64_t hi, uint64_t lo) { return ((u128)hi << 64) | lo; }

// reverse complement of a right-aligned 2k-bit value
__device__ __forceinline__ u128 rc_k(u128 x, int k) {
  const u128 full = make128(rc64_full((uint64_t)x), rc64_full((uint64_t)(x >> 64)));
  return full >> (128 - 2 * k);
}

__global__ void __launch_bounds__(SX_THREADS) k_sx_insert(const uint64_t* __restrict__ lo, const uint64_t* __restrict__ hi,
                                                         uint64_t n, K128* tab, uint32_t* rank, uint64_t mask,
                                                         uint32_t* status) {
  const K128 EMPTY = key_empty<K128>();
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const K128 key{lo[i], hi[i]};
    uint64_t s = key_hash(key) & mask;
    bool done = false;
    for (uint64_t probe = 0; probe <= mask; probe++) {
      const K128 prev = atomicCAS(&tab[s], EMPTY, key);
      if (key_eq(prev, EMPTY)) {
        rank[s] = (uint32_t)i;
        done = true;
        break;
      }
      if (key_eq(prev, key)) { done = true; break; }  // keys are distinct; defensive
      s = (s + 1) & mask;
    }
    if (!done) set_status(status, ST_TABLE_STUCK);
  }
}

__device__ __forceinline__ uint32_t sx_find(const K128* tab, const uint32_t* rank, uint64_t mask, u128 v) {
  const K128 key{(uint64_t)v, (uint64_t)(v >> 64)};
  uint64_t s = key_hash(key) & mask;
  for (uint64_t probe = 0; probe <= mask; probe++) {
    const K128 cur = tab[s];
    if (key_eq(cur, key)) return rank[s];
    if (key_eq(cur, key_empty<K128>())) return 0xffffffffu;
    s = (s + 1) & mask;
  }
  return 0xffffffffu;
}

__global__ void __launch_bounds__(SX_THREADS) k_sx_extensions(const uint64_t* __restrict__ lo,
                                                             const uint64_t* __restrict__ hi, uint64_t n, int k,
                                                             const K128* __restrict__ tab,
                                                             const uint32_t* __restrict__ rank, uint64_t mask,
                                                             uint32_t* __restrict__ ext) {
  const u128 kmask = k == 64 ? ~(u128)0 : (((u128)1 << (2 * k)) - 1);
  const int hs = 2 * (k - 1);
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < 2 * n; t += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = t >> 1;
    const int o = (int)(t & 1);
    const u128 key = make128(hi[i], lo[i]);
    const u128 rk = rc_k(key, k);
    const u128 S = o ? rk : key, R = o ? key : rk;  // the oriented string and its reverse complement
#pragma unroll
    for (int b = 0; b < 4; b++) {
      const u128 f = ((S << 2) | (u128)b) & kmask;
      const u128 r = (R >> 2) | ((u128)(3 - b) << hs);
      const u128 c = f < r ? f : r;
      const uint32_t j = sx_find(tab, rank, mask, c);
      ext[i * SIMPLITIG_STRIDE + (uint64_t)o * 4 + (uint64_t)b] =
          j == 0xffffffffu ? SIMPLITIG_NO_EXT : ((j << 1) | (c == f ? 0u : 1u));
    }
  }
}

}  // namespace

int32_t simplitig_extensions(mczi_ctx* ctx, const uint64_t* lo, const uint64_t* hi, uint64_t n, int k,
                             uint32_t* ext_host) {
  if (n == 0) return MCZI_OK;
  cudaStream_t s = ctx->stream;
  uint64_t slots = 1024;
  while (slots < 2 * n) slots <<= 1;
  CKA(ctx->sx_keys, n * 16);
  CKA(ctx->sx_tab, slots * 16);
  CKA(ctx->sx_rank, slots * 4);
  CKA(ctx->sx_ext, n * SIMPLITIG_STRIDE * 4);
  CKA(ctx->scalars, SC_COUNT * sizeof(uint64_t));
  uint64_t* dlo = ctx->sx_keys.as<uint64_t>();
  uint64_t* dhi = dlo + n;
  uint64_t* sc = ctx->scalars.as<uint64_t>();
  CK(cudaMemcpyAsync(dlo, lo, n * 8, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(dhi, hi, n * 8, cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(ctx->sx_tab.p, 0xff, slots * 16, s));
  CK(cudaMemsetAsync(sc + SC_STATUS, 0, 8, s));
  const unsigned grid = (unsigned)std::min<uint64_t>((2 * n + SX_THREADS - 1) / SX_THREADS, (uint64_t)ctx->sm_count * 16);
  k_sx_insert<<<grid, SX_THREADS, 0, s>>>(dlo, dhi, n, ctx->sx_tab.as<K128>(), ctx->sx_rank.as<uint32_t>(), slots - 1,
                                           reinterpret_cast<uint32_t*>(sc + SC_STATUS));
  k_sx_extensions<<<grid, SX_THREADS, 0, s>>>(dlo, dhi, n, k, ctx->sx_tab.as<K128>(), ctx->sx_rank.as<uint32_t>(),
                                               slots - 1, ctx->sx_ext.as<uint32_t>());
  CK(cudaGetLastError());
  uint64_t st = 0;
  CK(cudaMemcpyAsync(&st, sc + SC_STATUS, 8, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(ext_host, ctx->sx_ext.p, n * SIMPLITIG_STRIDE * 4, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (st & ST_TABLE_STUCK) return fail(ctx, MCZI_ERR_DEVICE, "simplitig key table full");
  return MCZI_OK;
}

}  // namespace mczi
