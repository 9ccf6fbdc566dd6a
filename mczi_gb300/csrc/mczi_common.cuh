// mczi_common.cuh -- shared device helpers for the MC/ZI k-mer kernels.
//
// Base code: A0 C1 G2 T3 (MC's `base_bits`, src/lib.rs:3030-3038).  A k-mer
// value is MSB-first, 2 bits per base, right-aligned (src/lib.rs:3056-3069);
// canonical = min(forward, reverse complement) (src/lib.rs:3589-3614).
//
// Packed base stream in HBM: u32 words, base b in word b >> 4 at bits
// [31 - 2(b & 15) - 1, 31 - 2(b & 15)], i.e. MSB-first, so a run of bases is a
// contiguous big-endian bit field.  Fragment starts are one bit per base, LSB
// first in u32 words.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace mczi {

// status bits written by kernels (never trap a shared GPU: record and return)
enum : uint32_t {
  ST_OK = 0,
  ST_DESC_OVERFLOW = 1u << 0,    // descriptor buffer too small
  ST_OUT_OVERFLOW = 1u << 1,     // result buffer too small
  ST_SPIN_TIMEOUT = 1u << 2,     // a bounded wait gave up
  ST_TABLE_STUCK = 1u << 3,      // a round could not be split further
  ST_BAD_INDEX = 1u << 4,        // an index check failed (kernel skipped the access)
  ST_MINTAB_FULL = 1u << 5,      // minimizer table full
  ST_ZI_OVERFLOW = 1u << 6,      // ZI absent buffer too small
  ST_COUNT_WIDTH = 1u << 7,      // a bucket holds more k-mer windows than its 32-bit counters take
  ST_GZ_CORRUPT = 1u << 8,       // a gzip member failed to decode, or decoded to another length or CRC
};

__device__ __forceinline__ void set_status(uint32_t* st, uint32_t bit) { atomicOr(st, bit); }

// ---------------------------------------------------------------- keys
struct K64 {
  uint64_t v;
};
struct __align__(16) K128 {
  uint64_t lo, hi;
};

__host__ __device__ __forceinline__ bool key_lt(K64 a, K64 b) { return a.v < b.v; }
__host__ __device__ __forceinline__ bool key_lt(K128 a, K128 b) {
  return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}
__host__ __device__ __forceinline__ bool key_eq(K64 a, K64 b) { return a.v == b.v; }
__host__ __device__ __forceinline__ bool key_eq(K128 a, K128 b) { return a.hi == b.hi && a.lo == b.lo; }

template <class K> __host__ __device__ __forceinline__ K key_empty();
template <> __host__ __device__ __forceinline__ K64 key_empty<K64>() { return K64{~0ull}; }
template <> __host__ __device__ __forceinline__ K128 key_empty<K128>() { return K128{~0ull, ~0ull}; }

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ull;
  return x ^ (x >> 33);
}
__device__ __forceinline__ uint32_t mix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  return x ^ (x >> 16);
}

__device__ __forceinline__ uint64_t key_hash(K64 k) { return mix64(k.v); }
// 128-bit keys: fold of the 128-bit product of the two (offset) halves --
// one wide multiply on the FMA pipe instead of two rounds of shifts and xors
// on the integer ALU, which bounds the counting kernel
__device__ __forceinline__ uint64_t key_hash(K128 k) {
  const uint64_t a = k.lo ^ 0x2d358dccaa6c78a5ull, b = k.hi ^ 0x8bb84b93962eacc9ull;
  return (a * b) ^ __umul64hi(a, b);
}

// reverse the order of 2-bit groups and complement (x ^ 3 per base)
__device__ __forceinline__ uint64_t rc64_full(uint64_t x) {
  x = ~x;
  x = __brevll(x);
  // brev reversed bits inside each 2-bit group too: swap them back
  return ((x >> 1) & 0x5555555555555555ull) | ((x & 0x5555555555555555ull) << 1);
}

// ------------------------------------------------------------- rolling k-mers
// Forward/reverse state for a k-mer of length k (k <= 32 for K64, <= 64 for K128)
struct Roll64 {
  uint64_t fwd, rev, mask;
  int hs;
  __device__ __forceinline__ void init(int k) {
    mask = (k == 32) ? ~0ull : ((1ull << (2 * k)) - 1);
    hs = 2 * (k - 1);
    fwd = rev = 0;
  }
  __device__ __forceinline__ void push(uint32_t b) {
    fwd = ((fwd << 2) | b) & mask;
    rev = (rev >> 2) | ((uint64_t)(b ^ 3u) << hs);
  }
  // set from a right-aligned forward value
  __device__ __forceinline__ void set(uint64_t f, int k) {
    fwd = f;
    rev = rc64_full(f) >> (64 - 2 * k);
  }
  __device__ __forceinline__ K64 canon() const { return K64{fwd < rev ? fwd : rev}; }
};

struct Roll128 {
  uint64_t flo, fhi, rlo, rhi, mlo, mhi;
  int k;
  __device__ __forceinline__ void init(int kk) {
    k = kk;
    if (k == 64) { mlo = mhi = ~0ull; }
    else if (k >= 32) { mlo = ~0ull; mhi = (k == 32) ? 0 : ((1ull << (2 * (k - 32))) - 1); }
    else { mlo = (1ull << (2 * k)) - 1; mhi = 0; }
    flo = fhi = rlo = rhi = 0;
  }
  __device__ __forceinline__ void push(uint32_t b) {
    fhi = ((fhi << 2) | (flo >> 62)) & mhi;
    flo = ((flo << 2) | b) & mlo;
    // rev = (rev >> 2) | ((b^3) << 2(k-1))
    rlo = (rlo >> 2) | (rhi << 62);
    rhi = rhi >> 2;
    const int hs = 2 * (k - 1);
    const uint64_t c = (uint64_t)(b ^ 3u);
    if (hs >= 64) rhi |= c << (hs - 64);
    else rlo |= c << hs;
  }
  // set from right-aligned forward (hi, lo)
  __device__ __forceinline__ void set(uint64_t hi, uint64_t lo, int kk) {
    k = kk;
    flo = lo;
    fhi = hi;
    // full 128-bit reverse complement, then shift right by 128 - 2k
    uint64_t r_hi = rc64_full(lo), r_lo = rc64_full(hi);
    const int sh = 128 - 2 * k;
    if (sh == 0) { rlo = r_lo; rhi = r_hi; }
    else if (sh < 64) { rlo = (r_lo >> sh) | (r_hi << (64 - sh)); rhi = r_hi >> sh; }
    else if (sh == 64) { rlo = r_hi; rhi = 0; }
    else { rlo = r_hi >> (sh - 64); rhi = 0; }
  }
  __device__ __forceinline__ K128 canon() const {
    bool f = (fhi < rhi) || (fhi == rhi && flo < rlo);
    return f ? K128{flo, fhi} : K128{rlo, rhi};
  }
};

// Strand-symmetric hash of a rolling k-mer: forward XOR reverse complement is
// the same for both strands, so the hash is a function of the canonical k-mer
// without forming it (the 128-bit compare and select of canon()).
__device__ __forceinline__ uint64_t sym_hash(const Roll64& r) { return mix64(r.fwd ^ r.rev); }
__device__ __forceinline__ uint64_t sym_hash(const Roll128& r) {
  const uint64_t a = r.flo ^ r.rlo ^ 0x2d358dccaa6c78a5ull, b = r.fhi ^ r.rhi ^ 0x8bb84b93962eacc9ull;
  return (a * b) ^ __umul64hi(a, b);
}

// ------------------------------------------------------------- packed stream
__device__ __forceinline__ uint32_t base_at(const uint32_t* __restrict__ packed, uint64_t p) {
  return (packed[p >> 4] >> (30 - 2 * (uint32_t)(p & 15))) & 3u;
}

// Right-aligned 2n-bit field (n <= 32) of bases [p, p + n) from the packed
// stream; reads three words (callers guarantee two words of slack).
__device__ __forceinline__ uint64_t field64(const uint32_t* __restrict__ w, uint64_t p, int n) {
  const uint64_t wi = p >> 4;
  const uint32_t off = 2 * (uint32_t)(p & 15);
  const uint64_t a = ((uint64_t)w[wi] << 32) | w[wi + 1];
  const uint64_t b = (uint64_t)w[wi + 2];
  uint64_t top = off ? ((a << off) | (b >> (32 - off))) : a;  // bases p .. p+31
  return n == 32 ? top : (top >> (64 - 2 * n));
}

// Same from a shared-memory copy whose word 0 holds base `base0` (multiple of 16)
__device__ __forceinline__ uint64_t field64_s(const uint32_t* w, uint32_t rel, int n) {
  const uint32_t wi = rel >> 4;
  const uint32_t off = 2 * (rel & 15);
  const uint64_t a = ((uint64_t)w[wi] << 32) | w[wi + 1];
  const uint64_t b = (uint64_t)w[wi + 2];
  uint64_t top = off ? ((a << off) | (b >> (32 - off))) : a;
  return n == 32 ? top : (top >> (64 - 2 * n));
}

// Superkmer descriptors.  Before the partition: u64 start << 24 | (windows-1)
// plus a u32 key.  From partition pass 1 on, the bucket (p1 digit) is implicit
// and one u64 carries start << 23 | (windows-1) << 11 | p2 (windows <= 4096,
// p2 < 2048, start < 2^41).
__host__ __device__ __forceinline__ uint64_t bd_make(uint64_t start, uint32_t windows, uint32_t p2) {
  return (start << 23) | ((uint64_t)(windows - 1) << 11) | (uint64_t)p2;
}
__host__ __device__ __forceinline__ uint64_t bd_start(uint64_t bd) { return bd >> 23; }
__host__ __device__ __forceinline__ uint32_t bd_windows(uint64_t bd) { return (uint32_t)((bd >> 11) & 0xfffu) + 1u; }
__host__ __device__ __forceinline__ uint32_t bd_p2(uint64_t bd) { return (uint32_t)(bd & 0x7ffu); }

// m-mer hash of the minimizer order, multiplicative (Knuth): the top half of
// the 64-bit product with an odd constant, one multiply and no shifts of the
// integer pipe, which bounds the scan.  The scan applies it to both strands of
// an m-mer and keeps the smaller, so the order is strand-symmetric.
__device__ __forceinline__ uint32_t mmer_hash64(uint64_t v) {
  return (uint32_t)((v * 0x9E3779B97F4A7C15ull) >> 32);
}

}  // namespace mczi
