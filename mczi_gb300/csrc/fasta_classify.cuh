// fasta_classify.cuh -- the FASTA byte rules of the packer (K1), usable on
// the device and, for tests, in host C++.
//
// MC parses FASTA with helicase's split_non_actg (src/lib.rs:3264-3308):
// headers are dropped, line breaks inside a record are transparent, any byte
// other than A/C/G/T (either case) ends the current fragment, and so does the
// start of a new record.  step_fasta applies that to one byte; fasta32 to 32
// bytes at once with byte masks (same answers); fasta32_runs walks the base
// runs of a classified chunk in order.
#pragma once
#include <stdint.h>

#ifndef __CUDACC__
#define __host__
#define __device__
#define __forceinline__ inline
#endif

namespace mczi {
namespace fasta {

enum : uint32_t { LS = 0, HDR = 1, SEQ = 2 };

__host__ __device__ __forceinline__ int ffs32(uint32_t x) {
#ifdef __CUDA_ARCH__
  return __ffs((int)x);
#else
  return __builtin_ffs((int)x);
#endif
}
__host__ __device__ __forceinline__ int popc32(uint32_t x) {
#ifdef __CUDA_ARCH__
  return __popc(x);
#else
  return __builtin_popcount(x);
#endif
}
__host__ __device__ __forceinline__ int clz32(uint32_t x) {
#ifdef __CUDA_ARCH__
  return __clz((int)x);
#else
  return x ? __builtin_clz(x) : 32;
#endif
}

__host__ __device__ __forceinline__ int8_t code_of(uint32_t c) {
  // A/a 0, C/c 1, G/g 2, T/t 3, else -1
  switch (c | 0x20u) {
    case 'a': return 0;
    case 'c': return 1;
    case 'g': return 2;
    case 't': return 3;
    default: return -1;
  }
}

// exact per-byte zero test: high bit of each byte set where the byte is 0
__host__ __device__ __forceinline__ uint32_t zero_bytes(uint32_t x) {
  const uint32_t y = ((x & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | x;
  return ~y & 0x80808080u;
}

// the four 0x80 flags of zero_bytes as 4 bits (the products do not overlap)
__host__ __device__ __forceinline__ uint32_t gather4(uint32_t z) { return (((z >> 7) * 0x00204081u) >> 21) & 0xFu; }

// Classify one byte.  Returns 0..3 for a base, 4 for a break, 5 for skip.
__host__ __device__ __forceinline__ uint32_t step_fasta(uint32_t c, uint32_t& st) {
  if (c == '\n') { st = LS; return 5; }
  if (st == LS) {
    if (c == '>') { st = HDR; return 4; }
    st = SEQ;
  }
  if (st == HDR) return 4;
  if (c == '\r') return 5;
  const int8_t code = code_of(c);
  return code < 0 ? 4u : (uint32_t)code;
}

// 32 bytes classified from the line state before them.  base: bit i = byte i
// is a base (not in a header); brk: bit i = byte i ends the current fragment
// (any other byte except '\n' and a '\r' outside a header); codes: MC codes
// MSB-first (byte 0 in bits 63-62), meaningful where base is set.  st is
// updated as step_fasta would leave it.  src: 16-byte aligned.
struct Fasta32 {
  uint32_t base, brk;
  uint64_t codes;
};

__host__ __device__ __forceinline__ Fasta32 fasta32(const uint8_t* src, uint32_t& st) {
  uint32_t w[8];
#ifdef __CUDA_ARCH__
  const uint4 v0 = *reinterpret_cast<const uint4*>(src);
  const uint4 v1 = *reinterpret_cast<const uint4*>(src + 16);
  w[0] = v0.x; w[1] = v0.y; w[2] = v0.z; w[3] = v0.w;
  w[4] = v1.x; w[5] = v1.y; w[6] = v1.z; w[7] = v1.w;
#else
  for (int j = 0; j < 8; j++)
    w[j] = (uint32_t)src[4 * j] | ((uint32_t)src[4 * j + 1] << 8) | ((uint32_t)src[4 * j + 2] << 16) |
           ((uint32_t)src[4 * j + 3] << 24);
#endif
  uint32_t nl = 0, cr = 0, gt = 0, acgt = 0;
  uint64_t codes = 0;
#pragma unroll
  for (int j = 0; j < 8; j++) {
    const uint32_t l = w[j] | 0x20202020u;
    nl |= gather4(zero_bytes(w[j] ^ 0x0a0a0a0au)) << (4 * j);
    cr |= gather4(zero_bytes(w[j] ^ 0x0d0d0d0du)) << (4 * j);
    gt |= gather4(zero_bytes(w[j] ^ 0x3e3e3e3eu)) << (4 * j);
    acgt |= gather4(zero_bytes(l ^ 0x61616161u) | zero_bytes(l ^ 0x63636363u) | zero_bytes(l ^ 0x67676767u) |
                    zero_bytes(l ^ 0x74747474u)) << (4 * j);
    // a0 c1 g3 t2 from bits 1-2, then MC's A0 C1 G2 T3 by x ^ (x >> 1)
    const uint32_t t = (w[j] >> 1) & 0x03030303u;
    const uint32_t mc = t ^ ((t >> 1) & 0x01010101u);
    const uint32_t v8 = ((mc & 3u) << 6) | (((mc >> 8) & 3u) << 4) | (((mc >> 16) & 3u) << 2) | ((mc >> 24) & 3u);
    codes |= (uint64_t)v8 << (56 - 8 * j);
  }
  // header lines: from a '>' at a line start (or an open header) to the next '\n'
  const uint32_t ls = (nl << 1) | (st == LS ? 1u : 0u);
  uint32_t starts = (ls & gt) | (st == HDR ? 1u : 0u);
  uint32_t hdr = 0;
  while (starts) {
    const int s0 = ffs32(starts) - 1;
    const uint32_t after = nl & (0xffffffffu << s0);
    const uint32_t upto = after ? ((1u << (ffs32(after) - 1)) - 1u) : 0xffffffffu;
    hdr |= upto & (0xffffffffu << s0);
    starts &= ~(upto | (1u << s0));
  }
  Fasta32 c;
  c.base = acgt & ~hdr;
  c.brk = ~(c.base | nl | (cr & ~hdr));
  c.codes = codes;
  st = (nl >> 31) ? (uint32_t)LS : ((hdr >> 31) ? (uint32_t)HDR : (uint32_t)SEQ);
  return c;
}

// bases of a chunk, and whether a break comes before the first / after the
// last base (both mean "any break" when there is no base)
__host__ __device__ __forceinline__ void fasta32_counts(const Fasta32& f, uint32_t* nb, uint32_t* fb, uint32_t* lb) {
  *nb = (uint32_t)popc32(f.base);
  if (*nb == 0) {
    *fb = *lb = f.brk ? 1u : 0u;
  } else {
    const int a = ffs32(f.base) - 1, b = 31 - clz32(f.base);
    *fb = (f.brk & ((1u << a) - 1u)) ? 1u : 0u;
    *lb = ((f.brk >> b) >> 1) ? 1u : 0u;
  }
}

// The runs of consecutive bases in order: emit(len, codes top-aligned in a
// u64, fragment_start).  pending carries "a break since the last base" in
// and out, as the byte loop's state does.
template <class F>
__host__ __device__ __forceinline__ void fasta32_runs(const Fasta32& fc, uint32_t& pending, F&& emit) {
  uint32_t m = fc.base;
  int done = 0;  // bytes [0, done) handled
  while (m) {
    const int a = ffs32(m) - 1;
    const uint32_t rest = ~(m >> a);
    const int len = rest ? ffs32(rest) - 1 : 32 - a;
    if (fc.brk & ((1u << a) - 1u) & (0xffffffffu << done)) pending = 1;
    const uint64_t run = (fc.codes << (2 * a)) & (len >= 32 ? ~0ull : ~(~0ull >> (2 * len)));
    emit(len, run, pending != 0);
    pending = 0;
    done = a + len;
    m = done >= 32 ? 0u : (m & (0xffffffffu << done));
  }
  if (done < 32 && (fc.brk & (0xffffffffu << done))) pending = 1;
}

}  // namespace fasta
}  // namespace mczi
