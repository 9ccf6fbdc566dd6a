// mc_pack.cu -- K1: FASTA/FASTQ bytes -> 2-bit packed base stream + fragment
// start bits, on the device.
//
// Replaces helicase's `dna_packed().split_non_actg()` parse as MC uses it
// (src/lib.rs:3264-3308): headers and quality lines are dropped, line breaks
// inside a FASTA record are transparent, any byte other than A/C/G/T (either
// case) ends the current fragment, and so does the start of a new record.
// Fragments shorter than k are not removed here: the window scan never emits
// a window that crosses a fragment start, so they simply contribute nothing.
//
// Layout: inputs are copied to HBM at offsets aligned to PACK_TILE bytes (the
// gaps are filled with '\n').  Three passes over 8 KiB tiles:
//   1. k_pack_lines : newline count and last newline per tile
//   2. k_pack_count : bases and fragment-break summary per tile, given the
//                     line state from the scan of pass 1
//   3. k_pack_write : 2-bit codes and fragment-start bits, staged in shared
//                     memory, interior words stored, edge words OR-ed.
#include <algorithm>

#include "fasta_classify.cuh"
#include "mczi_internal.h"
#include "scan.cuh"

namespace mczi {

namespace {

using namespace fasta;

struct LineOp {
  static __device__ LineSum identity() { return LineSum{-1, 0, 0, 0}; }
  static __device__ LineSum combine(const LineSum& a, const LineSum& b) {
    if (b.reset) return b;
    return LineSum{a.last > b.last ? a.last : b.last, a.nl + b.nl, a.reset, 0};
  }
};

struct BaseOp {
  static __device__ BaseSum identity() { return BaseSum{0, 0, 0, 0}; }
  static __device__ BaseSum combine(const BaseSum& a, const BaseSum& b) {
    if (a.nb == 0 && b.nb == 0) return BaseSum{0, 0, a.lb | b.lb, 0};
    if (a.nb == 0) return BaseSum{b.nb, a.lb | b.fb, b.lb, 0};
    if (b.nb == 0) return BaseSum{a.nb, a.fb, a.lb | b.lb, 0};
    return BaseSum{a.nb + b.nb, a.fb, b.lb, 0};
  }
};

// per-thread newline summary, in-tile positions
struct NlSum {
  int32_t last;
  uint32_t nl;
};
struct NlOp {
  static __device__ NlSum identity() { return NlSum{-1, 0}; }
  static __device__ NlSum combine(const NlSum& a, const NlSum& b) {
    return NlSum{a.last > b.last ? a.last : b.last, a.nl + b.nl};
  }
};

__device__ __forceinline__ void load_tile(const uint8_t* __restrict__ text, uint64_t tile, uint8_t* sb) {
  const uint4* src = reinterpret_cast<const uint4*>(text + tile * PACK_TILE);
  uint4* dst = reinterpret_cast<uint4*>(sb);
#pragma unroll
  for (int i = 0; i < PACK_TILE / 16 / PACK_THREADS; i++)
    dst[threadIdx.x + i * PACK_THREADS] = src[threadIdx.x + i * PACK_THREADS];
}

// Line state at this thread's first byte.
// FASTA: returns LS/HDR/SEQ.  FASTQ: returns the line index mod 4.
__device__ __forceinline__ uint32_t thread_state(const uint8_t* sb, bool fastq, uint32_t tile_state,
                                                 uint32_t tile_line4, int first) {
  __shared__ NlSum sh[PACK_THREADS / 32 + 1];
  NlSum mine{-1, 0};
#pragma unroll
  for (int q = 0; q < PACK_PER_THREAD / 16; q++) {
    // newlines of this thread's bytes, four at a time
    const uint4 v = *reinterpret_cast<const uint4*>(sb + first + 16 * q);
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const uint32_t z = zero_bytes(w[j] ^ 0x0a0a0a0au);
      if (z) {
        mine.nl += __popc(z);
        mine.last = first + 16 * q + 4 * j + (31 - __clz(z)) / 8;
      }
    }
  }
  NlSum tot;
  NlSum pre = block_exclusive_scan<NlSum, NlOp, PACK_THREADS>(mine, &tot, sh);
  if (fastq) return (tile_line4 + pre.nl) & 3u;
  if (pre.last >= 0) {
    const int ls = pre.last + 1;
    if (ls == first) return LS;
    return sb[ls] == '>' ? HDR : SEQ;
  }
  if (tile_state == LS) {
    if (first == 0) return LS;
    return sb[0] == '>' ? HDR : SEQ;
  }
  return tile_state;
}

__device__ __forceinline__ uint32_t step_fastq(uint32_t c, uint32_t& line) {
  if (c == '\n') {
    uint32_t r = ((line & 3u) == 1u) ? 4u : 5u;  // end of a sequence line ends the fragment
    line++;
    return r;
  }
  if ((line & 3u) != 1u) return 4;
  if (c == '\r') return 5;
  int8_t code = code_of(c);
  return code < 0 ? 4u : (uint32_t)code;
}

// Fast path for 32 bytes that are all A/C/G/T (either case): returns true and
// the 32 MC codes MSB-first in *codes.  One u32 holds 4 bytes, first byte in
// the low bits.  Bits 1-2 of A, C, T, G (either case) are t = 0, 1, 2, 3: a
// byte is one of the eight letters iff it equals, up to the case bit, the
// upper-case letter t names ('A' + {0, 2, 0x13, 6}[t], computed for four
// bytes at once), and MC's code (A0 C1 G2 T3) is t ^ (t >> 1).  One multiply
// gathers a word's four 2-bit codes into its top byte, first byte's highest.
__device__ __forceinline__ bool acgt32(const uint8_t* src, uint64_t* codes) {
  const uint4 v0 = *reinterpret_cast<const uint4*>(src);
  const uint4 v1 = *reinterpret_cast<const uint4*>(src + 16);
  const uint32_t w[8] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z, v1.w};
  bool ok = true;
  uint32_t p[8];
#pragma unroll
  for (int j = 0; j < 8; j++) {
    const uint32_t t = (w[j] >> 1) & 0x03030303u;
    const uint32_t t1 = (t >> 1) & 0x01010101u;
    const uint32_t expect = 0x41414141u + 2u * t + 15u * (t1 & ~t);  // + 0x13 where t == 2
    ok &= (w[j] | 0x20202020u) == (expect | 0x20202020u);
    p[j] = (t ^ t1) * 0x40100401u;  // bits 24-31: codes of bytes 0, 1, 2, 3 from the top
  }
  // the eight top bytes in order: byte 0 of the chunk at the top of *codes
  const uint32_t hi = __byte_perm(__byte_perm(p[3], p[2], 0x0073), __byte_perm(p[1], p[0], 0x7300), 0x7610);
  const uint32_t lo = __byte_perm(__byte_perm(p[7], p[6], 0x0073), __byte_perm(p[5], p[4], 0x7300), 0x7610);
  *codes = ((uint64_t)hi << 32) | lo;
  return ok;
}

// a chunk's base count and breaks as one BaseSum term
__device__ __forceinline__ BaseSum fasta32_sum(const Fasta32& f) {
  uint32_t nb, fb, lb;
  fasta32_counts(f, &nb, &fb, &lb);
  return BaseSum{nb, fb, lb, 0};
}

// OR 2*len code bits (top-aligned in v) into the staging words at base p
__device__ __forceinline__ void stage_codes(uint32_t* spk, uint64_t p, uint64_t w0, uint64_t v) {
  const uint64_t q = (p >> 4) - w0;
  const uint32_t r2 = 2 * (uint32_t)(p & 15);
  const uint32_t a = (uint32_t)(v >> (32 + r2)), b = (uint32_t)(v >> r2);
  if (a) atomicOr(&spk[q], a);
  if (b) atomicOr(&spk[q + 1], b);
  if (r2) {
    const uint32_t c = (uint32_t)(v << (32 - r2));
    if (c) atomicOr(&spk[q + 2], c);
  }
}

__device__ __forceinline__ void tile_line_state(const uint8_t* __restrict__ text, const uint32_t* __restrict__ tile_info,
                                                const uint64_t* __restrict__ input_tile0, const LineSum* __restrict__ line_pre,
                                                uint64_t tile, bool& fastq, uint32_t& st, uint32_t& line4) {
  const uint32_t info = tile_info[tile];
  fastq = (info >> 1) & 1u;
  if (info & 1u) {  // input starts here
    st = LS;
    line4 = 0;
    return;
  }
  const LineSum e = line_pre[tile];
  line4 = (uint32_t)(e.nl & 3u);
  const uint64_t p0 = tile * PACK_TILE;
  uint64_t ls;
  if (e.last >= 0) ls = (uint64_t)e.last + 1;
  else ls = input_tile0[info >> 2] * PACK_TILE;
  if (ls == p0) st = LS;
  else st = (text[ls] == '>') ? HDR : SEQ;
}

}  // namespace

__global__ void __launch_bounds__(PACK_THREADS) k_pack_lines(const uint8_t* __restrict__ text,
                                                             const uint32_t* __restrict__ tile_info,
                                                             uint64_t tile_lo, uint64_t tile_hi,
                                                             LineSum* __restrict__ out) {
  const uint64_t tile = tile_lo + blockIdx.x;
  if (tile >= tile_hi) return;
  const uint4* src = reinterpret_cast<const uint4*>(text + tile * PACK_TILE);
  int32_t last = -1;
  uint32_t nl = 0;
#pragma unroll
  for (int i = 0; i < PACK_TILE / 16 / PACK_THREADS; i++) {
    const int vi = threadIdx.x + i * PACK_THREADS;
    uint4 v = src[vi];
    uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int j = 0; j < 4; j++) {
#pragma unroll
      for (int b = 0; b < 4; b++) {
        if (((w[j] >> (8 * b)) & 0xffu) == '\n') {
          nl++;
          last = vi * 16 + j * 4 + b;
        }
      }
    }
  }
  // block reduce
  for (int o = 16; o > 0; o >>= 1) {
    nl += __shfl_down_sync(0xffffffffu, nl, o);
    int32_t l2 = __shfl_down_sync(0xffffffffu, last, o);
    last = l2 > last ? l2 : last;
  }
  __shared__ uint32_t snl[PACK_THREADS / 32];
  __shared__ int32_t slast[PACK_THREADS / 32];
  if ((threadIdx.x & 31) == 0) {
    snl[threadIdx.x >> 5] = nl;
    slast[threadIdx.x >> 5] = last;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t n = 0;
    int32_t l = -1;
    for (int i = 0; i < PACK_THREADS / 32; i++) {
      n += snl[i];
      l = slast[i] > l ? slast[i] : l;
    }
    LineSum s;
    s.last = l >= 0 ? (int64_t)(tile * PACK_TILE + (uint64_t)l) : -1;
    s.nl = n;
    s.reset = tile_info[tile] & 1u;
    s.pad = 0;
    out[tile] = s;
  }
}

__global__ void __launch_bounds__(PACK_THREADS) k_pack_count(const uint8_t* __restrict__ text,
                                                             const uint32_t* __restrict__ tile_info,
                                                             const uint64_t* __restrict__ input_tile0,
                                                             const LineSum* __restrict__ line_pre, uint64_t tile_lo,
                                                             uint64_t tile_hi, BaseSum* __restrict__ out) {
  __shared__ __align__(16) uint8_t sb[PACK_TILE];
  __shared__ BaseSum shs[PACK_THREADS / 32 + 1];
  const uint64_t tile = tile_lo + blockIdx.x;
  if (tile >= tile_hi) return;
  load_tile(text, tile, sb);
  bool fastq;
  uint32_t tst, tl4;
  tile_line_state(text, tile_info, input_tile0, line_pre, tile, fastq, tst, tl4);
  __syncthreads();
  const int first = threadIdx.x * PACK_PER_THREAD;
  uint32_t st = thread_state(sb, fastq, tst, tl4, first);
  BaseSum s{0, 0, 0, 0};
  // 32-byte chunks in order; an all-ACGT chunk on a sequence line leaves the
  // line state as it is
#pragma unroll
  for (int h = 0; h < PACK_PER_THREAD / 32; h++) {
    const int f = first + 32 * h;
    BaseSum c{0, 0, 0, 0};
    uint64_t codes;
    const bool seq_line = fastq ? ((st & 3u) == 1u) : (st != HDR);
    if (seq_line && acgt32(sb + f, &codes)) {
      c.nb = 32;  // 32 bases, no break; a FASTA line that started here is now mid-sequence
      if (!fastq) st = SEQ;
    } else if (!fastq) {
      c = fasta32_sum(fasta32(sb + f, st));
    } else {
      for (int i = 0; i < 32; i++) {
        const uint32_t r = step_fastq(sb[f + i], st);
        if (r < 4) { c.nb++; c.lb = 0; }
        else if (r == 4) { if (c.nb == 0) c.fb = 1; c.lb = 1; }
      }
    }
    s = BaseOp::combine(s, c);
  }
  // for nb == 0 lb means "any break"; for nb > 0 fb is a break before the first base
  BaseSum tot;
  block_exclusive_scan<BaseSum, BaseOp, PACK_THREADS>(s, &tot, shs);
  if (threadIdx.x == 0) out[tile] = tot;
}

__global__ void __launch_bounds__(PACK_THREADS) k_pack_write(const uint8_t* __restrict__ text,
                                                             const uint32_t* __restrict__ tile_info,
                                                             const uint64_t* __restrict__ input_tile0,
                                                             const LineSum* __restrict__ line_pre,
                                                             const BaseSum* __restrict__ base_pre, uint64_t tile_lo,
                                                             uint64_t tile_hi, uint32_t* __restrict__ packed,
                                                             uint32_t* __restrict__ fbits,
                                                             uint64_t* __restrict__ input_base) {
  __shared__ __align__(16) uint8_t sb[PACK_TILE];
  __shared__ BaseSum shs[PACK_THREADS / 32 + 1];
  __shared__ uint32_t spk[PACK_TILE / 16 + 3];
  __shared__ uint32_t sfb[PACK_TILE / 32 + 2];
  const uint64_t tile = tile_lo + blockIdx.x;
  if (tile >= tile_hi) return;
  // the tile's base prefix is needed after pass A: its load is issued first,
  // so its latency overlaps the tile load and pass A
  const BaseSum tile_pre = base_pre[tile];
  load_tile(text, tile, sb);
  for (int i = threadIdx.x; i < PACK_TILE / 16 + 2; i += PACK_THREADS) spk[i] = 0;
  for (int i = threadIdx.x; i < PACK_TILE / 32 + 2; i += PACK_THREADS) sfb[i] = 0;
  bool fastq;
  uint32_t tst, tl4;
  tile_line_state(text, tile_info, input_tile0, line_pre, tile, fastq, tst, tl4);
  __syncthreads();
  const int first = threadIdx.x * PACK_PER_THREAD;
  constexpr int NCH = PACK_PER_THREAD / 32;
  const uint32_t st0 = thread_state(sb, fastq, tst, tl4, first);
  // pass A: this thread's summary, 32-byte chunks in order (all-ACGT chunks
  // on a sequence line take the fast path and leave the line state as it is)
  uint32_t st = st0;
  BaseSum s{0, 0, 0, 0};
  uint64_t codes[NCH];
  bool fast[NCH];
#pragma unroll
  for (int h = 0; h < NCH; h++) {
    const int f = first + 32 * h;
    BaseSum c{0, 0, 0, 0};
    codes[h] = 0;
    const bool seq_line = fastq ? ((st & 3u) == 1u) : (st != HDR);
    fast[h] = seq_line && acgt32(sb + f, &codes[h]);
    if (fast[h]) {
      c.nb = 32;
      if (!fastq) st = SEQ;  // 32 letters: a FASTA line that started here is now mid-sequence
    } else if (!fastq) {
      c = fasta32_sum(fasta32(sb + f, st));
    } else {
      for (int i = 0; i < 32; i++) {
        const uint32_t r = step_fastq(sb[f + i], st);
        if (r < 4) { c.nb++; c.lb = 0; }
        else if (r == 4) { if (c.nb == 0) c.fb = 1; c.lb = 1; }
      }
    }
    s = BaseOp::combine(s, c);
  }
  BaseSum tot;
  BaseSum excl =
      BaseOp::combine(tile_pre, block_exclusive_scan<BaseSum, BaseOp, PACK_THREADS>(s, &tot, shs));
  if (threadIdx.x == 0 && (tile_info[tile] & 1u)) input_base[tile_info[tile] >> 2] = tile_pre.nb;
  // pass B: write codes and start bits into the staging buffers
  const uint64_t tb = tile_pre.nb;        // first base of this tile
  const uint64_t w0 = tb >> 4, f0 = tb >> 5;
  uint64_t p = excl.nb;
  uint32_t pending = (excl.nb == 0) ? 1u : excl.lb;
  st = st0;
#pragma unroll
  for (int h = 0; h < NCH; h++) {
    const int f = first + 32 * h;
    if (fast[h]) {
      // 32 bases at p: spread the 64 code bits over (up to) three staging words
      stage_codes(spk, p, w0, codes[h]);
      if (pending) atomicOr(&sfb[(p >> 5) - f0], 1u << (uint32_t)(p & 31));
      pending = 0;
      p += 32;
      if (!fastq) st = SEQ;
    } else if (!fastq) {
      // runs of consecutive bases, each staged like a fast chunk; a break
      // before a run makes its first base a fragment start
      const Fasta32 fc = fasta32(sb + f, st);
      fasta32_runs(fc, pending, [&](int len, uint64_t run, bool start) {
        stage_codes(spk, p, w0, run);
        if (start) atomicOr(&sfb[(p >> 5) - f0], 1u << (uint32_t)(p & 31));
        p += (uint64_t)len;
      });
    } else {
      for (int i = 0; i < 32; i++) {
        const uint32_t r = step_fastq(sb[f + i], st);
        if (r < 4) {
          atomicOr(&spk[(p >> 4) - w0], r << (30 - 2 * (uint32_t)(p & 15)));
          if (pending) atomicOr(&sfb[(p >> 5) - f0], 1u << (uint32_t)(p & 31));
          pending = 0;
          p++;
        } else if (r == 4) {
          pending = 1;
        }
      }
    }
  }
  __syncthreads();
  const uint64_t nb = tot.nb;
  if (nb == 0) return;
  const uint64_t wl = (tb + nb - 1) >> 4, fl = (tb + nb - 1) >> 5;
  for (uint64_t w = w0 + threadIdx.x; w <= wl; w += PACK_THREADS) {
    uint32_t v = spk[w - w0];
    if (w == w0 || w == wl) atomicOr(&packed[w], v);
    else packed[w] = v;
  }
  for (uint64_t f = f0 + threadIdx.x; f <= fl; f += PACK_THREADS) {
    uint32_t v = sfb[f - f0];
    if (f == f0 || f == fl) { if (v) atomicOr(&fbits[f], v); }
    else fbits[f] = v;
  }
}

// pre[i] = carry (+) pre[i] for i < n: a segment's local exclusive prefix
// made global (the carry is the total of all earlier segments)
template <class T, class Op>
__global__ void k_apply_carry(T* __restrict__ pre, uint64_t n, const T* __restrict__ carry) {
  const T c = *carry;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    pre[i] = Op::combine(c, pre[i]);
}

void launch_pack(const PackArgs& a, cudaStream_t s) { launch_pack_segment(a, 0, a.n_tiles, nullptr, nullptr, s); }

void launch_pack_segment(const PackArgs& a, uint64_t t0, uint64_t t1, LineSum* carry_line, BaseSum* carry_base,
                         cudaStream_t s) {
  if (t1 <= t0) return;
  const uint64_t n = t1 - t0;
  const unsigned grid = (unsigned)n;
  const unsigned cgrid = (unsigned)std::min<uint64_t>((n + 1 + 255) / 256, 1024);
  // a later segment saves the running totals (written at its first tile by the
  // previous segment) before its local scans overwrite them
  const bool chained = t0 > 0;
  k_pack_lines<<<grid, PACK_THREADS, 0, s>>>(a.text, a.tile_info, t0, t1, a.line_sum);
  if (chained) cudaMemcpyAsync(carry_line, a.line_pre + t0, sizeof(LineSum), cudaMemcpyDeviceToDevice, s);
  exclusive_scan<LineSum, LineOp>(a.line_sum + t0, a.line_pre + t0, n, a.line_tmp, s);
  if (chained) k_apply_carry<LineSum, LineOp><<<cgrid, 256, 0, s>>>(a.line_pre + t0, n + 1, carry_line);
  k_pack_count<<<grid, PACK_THREADS, 0, s>>>(a.text, a.tile_info, a.input_tile0, a.line_pre, t0, t1, a.base_sum);
  if (chained) cudaMemcpyAsync(carry_base, a.base_pre + t0, sizeof(BaseSum), cudaMemcpyDeviceToDevice, s);
  exclusive_scan<BaseSum, BaseOp>(a.base_sum + t0, a.base_pre + t0, n, a.base_tmp, s);
  if (chained) k_apply_carry<BaseSum, BaseOp><<<cgrid, 256, 0, s>>>(a.base_pre + t0, n + 1, carry_base);
  k_pack_write<<<grid, PACK_THREADS, 0, s>>>(a.text, a.tile_info, a.input_tile0, a.line_pre, a.base_pre, t0, t1,
                                             a.packed, a.fbits, a.input_base);
}

}  // namespace mczi
