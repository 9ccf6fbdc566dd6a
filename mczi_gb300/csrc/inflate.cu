// inflate.cu -- gzip (DEFLATE, RFC 1951 / RFC 1952) decoding on the device.
//
// Replaces the decompression in front of MC's FASTX parser for gzip inputs
// (src/lib.rs:3127-3143, 3218-3308: a multi-member gzip decoder) when every
// member of the input carries its compressed size, as BGZF members do (the
// "BC" extra subfield): the member boundaries are then known without
// decoding, and the members decode independently, one warp each.  Other
// gzip inputs are decoded on the host.
//
// All 32 lanes of a warp run the same bit reader and Huffman decode in step:
// the decoder state is warp-uniform and every lane loads the same byte (a
// broadcast), so no lane waits for another's decode and no shuffles are
// needed.  Lane 0 writes literals; the lanes split the bytes of each match (a
// match at distance d repeats the d bytes before it, so its byte j is the
// byte j mod d of that period) and of stored blocks.  A Huffman code decodes
// through a 9-bit lookup table in shared memory, a longer code bit by bit
// over the canonical code's length counts.  At the member's end the warp
// checks the decoded length against ISIZE and the CRC-32 (each lane takes a
// slice; the slices' CRC registers combine by multiplication with x^(8n) mod
// the CRC polynomial).  Every read and write is bounds-checked: an invalid
// member sets ST_GZ_CORRUPT and never accesses memory outside its input and
// output ranges.  The length and distance tables below are the format's own
// (RFC 1951 section 3.2.5).
#include "mczi_internal.h"
#include "mczi_common.cuh"

namespace mczi {

namespace {

constexpr int INF_WARPS = 4;  // warps (members in flight) per CTA
constexpr int FAST_BITS = 9;
constexpr int MAX_LEN = 15;
constexpr uint32_t CRC_POLY = 0xEDB88320u;  // CRC-32, bit-reflected

__constant__ uint16_t LEN_BASE[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                                      31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
__constant__ uint8_t LEN_EXTRA[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
__constant__ uint16_t DIST_BASE[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                       193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
__constant__ uint8_t DIST_EXTRA[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
// order in which a dynamic block lists the code-length code's lengths
__constant__ uint8_t CL_ORDER[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

// a canonical Huffman code, for decoding
struct Huff {
  uint16_t fast[1 << FAST_BITS];  // next 9 stream bits -> symbol << 4 | code length; 0: a longer code
  uint16_t count[MAX_LEN + 1];    // codes of each length
  uint16_t first_code[MAX_LEN + 1];
  uint16_t first_index[MAX_LEN + 2];  // index in sym of the first code of each length
  uint16_t sym[288];                  // symbols in canonical order (length, then value)
};
struct WarpSmem {
  Huff lit, dist;
  uint8_t lens[320];  // code lengths being read (literal/length, then distance)
  uint32_t bad;
};

// Builds h from lens[0..n) (all lanes call it; lane 0 does the counting).
// False for an over-subscribed code; an incomplete code is kept (a missing
// code then fails to decode).
__device__ bool huff_build(Huff& h, const uint8_t* lens, int n, uint32_t* bad, int lane) {
  if (lane == 0) {
    for (int l = 0; l <= MAX_LEN; l++) h.count[l] = 0;
    for (int s = 0; s < n; s++) h.count[lens[s]]++;
    h.count[0] = 0;
    int left = 1;
    uint32_t over = 0;
    uint32_t code = 0, idx = 0;
    for (int l = 1; l <= MAX_LEN; l++) {
      left = (left << 1) - h.count[l];
      if (left < 0) over = 1;
      code = (code + (l > 1 ? h.count[l - 1] : 0u)) << (l > 1 ? 1 : 0);
      h.first_code[l] = (uint16_t)code;
      h.first_index[l] = (uint16_t)idx;
      idx += h.count[l];
    }
    h.first_index[MAX_LEN + 1] = (uint16_t)idx;
    // symbols in canonical order
    uint16_t at[MAX_LEN + 1];
    for (int l = 1; l <= MAX_LEN; l++) at[l] = h.first_index[l];
    for (int s = 0; s < n; s++)
      if (lens[s]) h.sym[at[lens[s]]++] = (uint16_t)s;
    *bad = over;
  }
  for (int e = lane; e < (1 << FAST_BITS); e += 32) h.fast[e] = 0;
  __syncwarp();
  if (*bad) return false;
  // codes of <= 9 bits fill every table entry whose low bits are the code
  // (stream order: the code's first bit is the entry's lowest)
  const int n_fast = h.first_index[FAST_BITS + 1];
  for (int i = lane; i < n_fast; i += 32) {
    const int s = h.sym[i];
    const int l = lens[s];
    const uint32_t c = h.first_code[l] + (uint32_t)(i - h.first_index[l]);
    const uint32_t rev = __brev(c) >> (32 - l);
    for (uint32_t e = rev; e < (1u << FAST_BITS); e += 1u << l) h.fast[e] = (uint16_t)((s << 4) | l);
  }
  __syncwarp();
  return true;
}

// next symbol of h from the bit buffer (>= 15 bits buffered), -1 if none
__device__ __forceinline__ int huff_decode(const Huff& h, uint64_t& bb, int& bn) {
  const uint32_t e = h.fast[bb & ((1u << FAST_BITS) - 1)];
  if (e) {
    const int l = (int)(e & 15u);
    bb >>= l;
    bn -= l;
    return (int)(e >> 4);
  }
  // canonical decode, most significant code bit first: the codes of length
  // l are [first, first + count) and every shorter prefix was tried before
  int code = 0, first = 0, index = 0;
  for (int l = 1; l <= MAX_LEN; l++) {
    code |= (int)(bb & 1u);
    bb >>= 1;
    bn--;
    const int c = h.count[l];
    if (code - first < c) return h.sym[index + code - first];
    index += c;
    first = (first + c) << 1;
    code <<= 1;
  }
  return -1;
}

// a * b mod the CRC polynomial, bit-reflected (bit 31 is x^0)
__device__ uint32_t gf2_mul(uint32_t a, uint32_t b) {
  uint32_t r = 0;
  for (int i = 0; i < 32; i++) {
    if (a & (0x80000000u >> i)) r ^= b;
    b = (b & 1u) ? (b >> 1) ^ CRC_POLY : b >> 1;
  }
  return r;
}
// x^(8 n) mod the CRC polynomial: the effect of n zero bytes on a CRC register
__device__ uint32_t x_pow_8n(uint64_t n) {
  uint32_t r = 0x80000000u, base = 0x00800000u;  // x^0, x^8
  while (n) {
    if (n & 1) r = gf2_mul(r, base);
    base = gf2_mul(base, base);
    n >>= 1;
  }
  return r;
}

// Decodes one member; false if it is not valid.  Warp-uniform control flow.
__device__ bool inflate_member(const uint8_t* __restrict__ in, uint32_t in_len, uint8_t* out,
                               uint32_t out_len, uint32_t want_crc, WarpSmem& ws, const uint32_t* crc_tab,
                               int lane) {
  uint64_t bb = 0;  // bit buffer, next stream bit lowest
  int bn = 0;       // bits in bb
  uint32_t q = 0;   // next input byte
  uint32_t pos = 0; // decoded bytes
  bool err = false;
  // tops the buffer up to >= 32 bits, four input bytes at a time (two
  // aligned words and a funnel shift: the bytes after a member's data are
  // its trailer, so the second word stays inside the member); past the input
  // it feeds zero bytes, and a member that needs more than 8 of them is
  // corrupt
  auto refill = [&]() {
    if (bn < 32) {
      uint32_t w = 0;
      if (q + 4u <= in_len) {
        const uintptr_t a = reinterpret_cast<uintptr_t>(in + q);
        const uint32_t* p = reinterpret_cast<const uint32_t*>(a & ~(uintptr_t)3);
        const uint32_t sh = (uint32_t)(a & 3u) * 8u;
        w = sh ? __funnelshift_r(p[0], p[1], sh) : p[0];
      } else {
        for (uint32_t i = 0; i < 4; i++)
          if (q + i < in_len) w |= (uint32_t)in[q + i] << (8 * i);
      }
      bb |= (uint64_t)w << bn;
      bn += 32;
      q += 4;
    }
    if (q > in_len + 8u) err = true;
  };
  auto take = [&](int n) -> uint32_t {  // n <= 32 bits, buffered
    const uint32_t v = (uint32_t)(bb & ((1ull << n) - 1ull));
    bb >>= n;
    bn -= n;
    return v;
  };
  bool last = false;
  while (!last && !err) {
    refill();
    last = take(1) != 0;
    const uint32_t type = take(2);
    if (type == 0) {
      // stored block: from the next byte boundary, LEN, ~LEN, LEN bytes
      const int drop = bn & 7;
      bb >>= drop;
      bn -= drop;
      const uint32_t start = q - (uint32_t)(bn >> 3);
      if (start + 4u > in_len) { err = true; break; }
      const uint32_t len = (uint32_t)in[start] | ((uint32_t)in[start + 1] << 8);
      const uint32_t nlen = (uint32_t)in[start + 2] | ((uint32_t)in[start + 3] << 8);
      if (len != (~nlen & 0xffffu) || start + 4u + len > in_len || pos + len > out_len) { err = true; break; }
      for (uint32_t j = (uint32_t)lane; j < len; j += 32) out[pos + j] = in[start + 4 + j];
      __syncwarp();
      pos += len;
      q = start + 4u + len;
      bb = 0;
      bn = 0;
      continue;
    }
    if (type == 3) { err = true; break; }
    uint32_t nlit = 288, ndist = 32;
    if (type == 1) {
      // fixed codes
      for (int s = lane; s < 320; s += 32)
        ws.lens[s] = s < 144 ? 8 : s < 256 ? 9 : s < 280 ? 7 : s < 288 ? 8 : 5;
      __syncwarp();
    } else {
      // dynamic codes: the code-length code, then both codes' lengths
      nlit = take(5) + 257;
      ndist = take(5) + 1;
      const uint32_t ncl = take(4) + 4;
      if (nlit > 286 || ndist > 30) { err = true; break; }
      for (int s = lane; s < 19; s += 32) ws.lens[s] = 0;
      __syncwarp();
      for (uint32_t i = 0; i < ncl; i++) {
        refill();
        const uint32_t l = take(3);
        if (lane == 0) ws.lens[CL_ORDER[i]] = (uint8_t)l;
      }
      __syncwarp();
      if (!huff_build(ws.lit, ws.lens, 19, &ws.bad, lane)) { err = true; break; }
      uint32_t i = 0;
      while (i < nlit + ndist) {
        refill();
        if (err) break;
        const int sym = huff_decode(ws.lit, bb, bn);
        uint32_t val = 0, rep = 1;
        if (sym < 0) { err = true; break; }
        if (sym < 16) {
          val = (uint32_t)sym;
        } else if (sym == 16) {
          if (i == 0) { err = true; break; }
          val = ws.lens[i - 1];
          rep = 3 + take(2);
        } else if (sym == 17) {
          rep = 3 + take(3);
        } else {
          rep = 11 + take(7);
        }
        if (i + rep > nlit + ndist) { err = true; break; }
        __syncwarp();  // lens[i - 1] was read by every lane
        for (uint32_t r = (uint32_t)lane; r < rep; r += 32) ws.lens[i + r] = (uint8_t)val;
        __syncwarp();
        i += rep;
      }
      if (err) break;
      if (ws.lens[256] == 0) { err = true; break; }  // no end-of-block code
    }
    // the distance lengths follow the literal/length ones in lens
    if (!huff_build(ws.lit, ws.lens, (int)nlit, &ws.bad, lane)) { err = true; break; }
    if (!huff_build(ws.dist, ws.lens + nlit, (int)ndist, &ws.bad, lane)) { err = true; break; }
    // the block's symbols: >= 32 bits before a literal/length code and its
    // extra bits (<= 20), again before a distance code and its extra bits (<= 28)
    for (;;) {
      refill();
      if (err) break;
      int sym = huff_decode(ws.lit, bb, bn);
      if (sym < 0) { err = true; break; }
      if (sym < 256) {
        if (pos >= out_len) { err = true; break; }
        if (lane == 0) out[pos] = (uint8_t)sym;
        pos++;
        continue;
      }
      if (sym == 256) break;
      sym -= 257;
      if (sym >= 29) { err = true; break; }
      const uint32_t len = LEN_BASE[sym] + take(LEN_EXTRA[sym]);
      refill();
      const int ds = huff_decode(ws.dist, bb, bn);
      if (ds < 0 || ds >= 30) { err = true; break; }
      const uint32_t d = DIST_BASE[ds] + take(DIST_EXTRA[ds]);
      if (d > pos || pos + len > out_len) { err = true; break; }
      __syncwarp();  // the bytes the match repeats are visible to every lane
      const uint8_t* src = out + pos - d;
      for (uint32_t j = (uint32_t)lane; j < len; j += 32) out[pos + j] = src[d >= len ? j : j % d];
      __syncwarp();
      pos += len;
    }
  }
  // every bit consumed came from the input, and the output is complete
  if (err || (uint64_t)q * 8u - (uint64_t)bn > (uint64_t)in_len * 8u || pos != out_len) return false;
  __syncwarp();
  // CRC-32: each lane's slice with a zero register, combined over the warp
  const uint32_t S = (out_len + 31u) / 32u;
  const uint32_t a = min(out_len, (uint32_t)lane * S), b = min(out_len, a + S);
  uint32_t r = 0;
  for (uint32_t i = a; i < b; i++) r = crc_tab[(r ^ out[i]) & 0xffu] ^ (r >> 8);
  uint32_t n = b - a;
  for (int step = 1; step < 32; step <<= 1) {
    const uint32_t r2 = __shfl_down_sync(0xffffffffu, r, step);
    const uint32_t n2 = __shfl_down_sync(0xffffffffu, n, step);
    if ((lane & (2 * step - 1)) == 0) {
      r = gf2_mul(r, x_pow_8n(n2)) ^ r2;
      n += n2;
    }
  }
  // the standard CRC starts from all ones and is inverted at the end
  const uint32_t crc = ~(r ^ gf2_mul(0xffffffffu, x_pow_8n(out_len)));
  return __shfl_sync(0xffffffffu, crc, 0) == want_crc;
}

__global__ void __launch_bounds__(32 * INF_WARPS) k_inflate(const uint8_t* __restrict__ comp,
                                                            const GzMember* __restrict__ members, uint32_t n,
                                                            uint8_t* out, unsigned int* work,
                                                            uint32_t* status) {
  __shared__ WarpSmem ws[INF_WARPS];
  __shared__ uint32_t crc_tab[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) {
    uint32_t c = (uint32_t)i;
    for (int j = 0; j < 8; j++) c = (c & 1u) ? (c >> 1) ^ CRC_POLY : c >> 1;
    crc_tab[i] = c;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  WarpSmem& w = ws[threadIdx.x >> 5];
  for (;;) {
    uint32_t mi = 0;
    if (lane == 0) mi = atomicAdd(work, 1u);
    mi = __shfl_sync(0xffffffffu, mi, 0);
    if (mi >= n) break;
    const GzMember m = members[mi];
    if (!inflate_member(comp + m.in_off, m.in_len, out + m.out_off, m.out_len, m.crc, w, crc_tab, lane) &&
        lane == 0)
      set_status(status, ST_GZ_CORRUPT);
  }
}

}  // namespace

void launch_inflate(const uint8_t* comp, const GzMember* members, uint32_t n_members, uint8_t* out,
                    unsigned int* work, uint32_t* status, int ctas, cudaStream_t s) {
  if (n_members == 0) return;
  const uint32_t need = (n_members + INF_WARPS - 1) / INF_WARPS;
  const unsigned grid = (unsigned)(need < (uint32_t)ctas ? need : (uint32_t)ctas);
  k_inflate<<<grid, 32 * INF_WARPS, 0, s>>>(comp, members, n_members, out, work, status);
}

}  // namespace mczi
