// mc_scan.cu -- K2: canonical minimizer scan and superkmer extraction.
//
// Replaces simd-minimizers' canonical scan + `run_hashes` and MC's run
// visitor (src/lib.rs:3694-3789; vendor/simd-minimizers-2.3.1/src/
// minimizers.rs:259-291, sliding_min.rs:556-593, collect.rs:116-286).
//
// Order: an m-mer's value is min(H(fwd), H(rc)) for m <= 32 (H multiplicative,
// see mmer_hash64) and H of a mix of its canonical value for m > 32 -- either
// way the same for both strands; a window's minimizer value is the minimum of
// the w = k - m + 1 values it contains.  Both strands of a k-mer contain the
// same m-mers up to strand, so the minimizer value -- and the partition
// derived from it -- is a function of the canonical k-mer alone,
// which is the invariant MC's counting relies on (each k-mer occurrence lands
// in the partition of its canonical form).  A superkmer is a maximal run of
// consecutive valid windows with the same minimizer value, cut at tile edges.
//
// One CTA scans SCAN_TILE windows of the concatenated base stream, so reads of
// any length (150 bp .. 100 kbp) are load-balanced by construction.  Each
// thread owns 16 consecutive positions: it rolls their m-mers (forward and
// reverse complement, one base per step) into a shared hash array, then takes
// the minima of its 16 windows in registers -- for w >= 16 all 16 windows
// contain the thread's last position, so each minimum is min(suffix minimum
// up to that position, prefix minimum after it) (van Herk / Gil-Werman with
// one split per thread); for w < 16 directly.
#include "mczi_internal.h"
#include "mczi_common.cuh"
#include "scan.cuh"
#include "bulk.cuh"

namespace mczi {

namespace {

constexpr int MAXW = 64;
constexpr int HL = SCAN_TILE + MAXW;                 // hashes per tile
constexpr int HLP = HL + HL / 16 + 1;                // padded: position j at j + j / 16
constexpr int PKW = (SCAN_TILE + 128) / 16 + 4;      // packed words staged
constexpr int FBW = (SCAN_TILE + 128) / 32 + 4;      // fragment-bit words staged
constexpr int WPT = SCAN_TILE / SCANK_THREADS;       // windows per thread
static_assert(SCAN_TILE <= 8192, "event encoding holds 13-bit positions");
static_assert(SCAN_TILE % 512 == 0, "a tile's packed words and fragment bits start on 16-byte boundaries");

struct Cnt2 {
  uint32_t ev, st;
};
struct Cnt2Op {
  static __device__ Cnt2 identity() { return Cnt2{0, 0}; }
  static __device__ Cnt2 combine(const Cnt2& a, const Cnt2& b) { return Cnt2{a.ev + b.ev, a.st + b.st}; }
};

// order of an m-mer (m <= 32) from both strands' values: the smaller of the
// two strands' hashes, a function of the canonical m-mer.  The multiplies run
// on the FMA pipe; the compare and select of the canonical value would load
// the integer pipe, which bounds the scan.
__device__ __forceinline__ uint32_t mmer_order(uint64_t f, uint64_t r) {
  return min(mmer_hash64(f), mmer_hash64(r));
}

__device__ __forceinline__ uint32_t mmer_hash_at(const uint32_t* spk, uint32_t rel, int m) {
  if (m <= 32) {
    const uint64_t f = field64_s(spk, rel, m);
    const uint64_t r = rc64_full(f) >> (64 - 2 * m);
    return mmer_order(f, r);
  }
  // 32 < m <= 64: hi = first m - 32 bases, lo = last 32 bases
  const int mh = m - 32;
  const uint64_t hi = field64_s(spk, rel, mh);
  const uint64_t lo = field64_s(spk, rel + mh, 32);
  const uint64_t rlo_full = rc64_full(hi), rhi_full = rc64_full(lo);
  const int sh = 128 - 2 * m;  // 0 .. 62
  uint64_t rlo, rhi;
  if (sh == 0) { rlo = rlo_full; rhi = rhi_full; }
  else { rlo = (rlo_full >> sh) | (rhi_full << (64 - sh)); rhi = rhi_full >> sh; }
  const bool fwd = (hi < rhi) || (hi == rhi && lo < rlo);
  const uint64_t chi = fwd ? hi : rhi, clo = fwd ? lo : rlo;
  return mmer_hash64(clo ^ (chi * 0xD6E8FEB86659FD93ull + 0x2545F4914F6CDD1Dull));
}

// (lo, hi) |= (lo, hi) >> s as one 128-bit value, 1 <= s < 64
__device__ __forceinline__ void smear128(uint64_t& lo, uint64_t& hi, int s) {
  lo |= (lo >> s) | (hi << (64 - s));
  hi |= hi >> s;
}

// padded shared index: 16 consecutive positions per thread -> stride 17 words
__device__ __forceinline__ int hp(int j) { return j + (j >> 4); }

// hashes of the m-mers at [j0, j0 + n) (m <= 32), rolled one base at a time
__device__ __forceinline__ void hash_run(const uint32_t* spk, uint32_t* sh_h, int j0, int n, int m) {
  const uint64_t mask = m == 32 ? ~0ull : ((1ull << (2 * m)) - 1);
  const int hs = 2 * (m - 1);
  uint64_t f = field64_s(spk, (uint32_t)j0, m);
  uint64_t r = rc64_full(f) >> (64 - 2 * m);
  uint64_t nxt = field64_s(spk, (uint32_t)(j0 + m), 32);  // bases j0 + m .., MSB-first
  sh_h[hp(j0)] = mmer_order(f, r);
  for (int i = 1; i < n; i++) {
    const uint32_t b = (uint32_t)(nxt >> 62);
    nxt <<= 2;
    f = ((f << 2) | b) & mask;
    r = (r >> 2) | ((uint64_t)(b ^ 3u) << hs);
    sh_h[hp(j0 + i)] = mmer_order(f, r);
  }
}

__device__ __forceinline__ bool in_range(uint32_t mval, uint32_t lo, uint32_t hi) {
  const uint32_t p1 = mix32(mval) >> (32 - P1_BITS);
  return p1 >= lo && p1 < hi;
}

}  // namespace

constexpr int MVL = SCAN_TILE + SCAN_TILE / 16 + 2;  // minimizer values, padded like hp()
constexpr int VBW = SCAN_TILE / 32;                   // validity bitmask words
static_assert(WPT == 16, "one thread owns 16 windows");
static_assert(HLP >= SCAN_TILE + 2, "events reuse the hash array");

size_t scan_smem_bytes() { return (size_t)(PKW + FBW + HLP + MVL + VBW) * sizeof(uint32_t); }

// KC, MC > 0 compile the kernel for one (k, m): the minima loops then have
// constant trip counts and unroll; 0 takes both from the arguments
template <int KC, int MC>
__global__ void __launch_bounds__(SCANK_THREADS) k_scan(ScanArgs a) {
  extern __shared__ __align__(16) uint32_t dyn[];
  uint32_t* spk = dyn;
  uint32_t* sfb = spk + PKW;
  uint32_t* sh_h = sfb + FBW;
  uint32_t* sh_mv = sh_h + HLP;
  uint32_t* sh_vb = sh_mv + MVL;
  uint32_t* ev = sh_h;  // reused once the minima are known: pos | start << 13 | rank << 14
  __shared__ Cnt2 shc[SCAN_THREADS + 1];
  __shared__ unsigned long long s_base;
  __shared__ __align__(8) uint64_t s_bar;  // completion of the staging copies

  const uint64_t nb = *a.n_bases;
  uint64_t tile = blockIdx.x;
  if (a.tile_range) {
    tile += a.tile_range[0];
    if (tile >= a.tile_range[1]) return;
  }
  const uint64_t t0 = tile * SCAN_TILE;
  const int k = KC > 0 ? KC : a.k, m = MC > 0 ? MC : a.m, w = k - m + 1;
  if (t0 + (uint64_t)k > nb) return;  // no valid window in this tile (uniform per CTA)
  const int tid = threadIdx.x;

  // stage packed words and fragment bits.  The tile's words start on a 1 KiB
  // (packed) and 512-byte (bits) boundary, so their in-range body goes by
  // two bulk copies (whole 16-byte groups) on one mbarrier; the words past
  // the streams' ends (the last tile) are zeros written by the threads.
  const uint64_t pw0 = t0 >> 4, fw0 = t0 >> 5;  // pw0 < packed_words: the tile holds a window
  const uint64_t fwords = (a.packed_words + 1) >> 1;
  const uint32_t npk = (uint32_t)(a.packed_words - pw0 < (uint64_t)PKW ? a.packed_words - pw0 : (uint64_t)PKW) & ~3u;
  const uint32_t nfb = (uint32_t)(fwords - fw0 < (uint64_t)FBW ? fwords - fw0 : (uint64_t)FBW) & ~3u;
  if (tid == 0) mbar_init(&s_bar, 1);
  __syncthreads();
  if (tid == 0) {
    mbar_arrive_expect_tx(&s_bar, (npk + nfb) * 4u);
    if (npk) bulk_load(spk, a.packed + pw0, npk * 4u, &s_bar);
    if (nfb) bulk_load(sfb, a.fbits + fw0, nfb * 4u, &s_bar);
  }
  for (int i = (int)npk + tid; i < PKW; i += SCANK_THREADS) {
    const uint64_t wi = pw0 + (uint64_t)i;
    spk[i] = wi < a.packed_words ? a.packed[wi] : 0u;
  }
  for (int i = (int)nfb + tid; i < FBW; i += SCANK_THREADS) {
    const uint64_t wi = fw0 + (uint64_t)i;
    sfb[i] = wi < fwords ? a.fbits[wi] : 0u;
  }
  const bool staged = mbar_wait(&s_bar, 0, 1u << 20);
  if (__syncthreads_or(!staged)) {
    // the copies did not complete: record it, wait once more (bounded) so
    // nothing lands after the block exits, and leave the tile
    if (tid == 0) {
      set_status(a.status, ST_SPIN_TIMEOUT);
      mbar_wait(&s_bar, 0, 1u << 20);
    }
    return;
  }

  // m-mer hashes for positions [t0, t0 + SCAN_TILE + w - 1): 16 per thread,
  // then the tail of w - 1 positions in runs of 16
  const int L = SCAN_TILE + w - 1;
  const int r0 = tid * WPT;
  if (m <= 32) {
    hash_run(spk, sh_h, r0, WPT, m);
    for (int j0 = SCAN_TILE + tid * WPT; j0 < L; j0 += SCANK_THREADS * WPT) hash_run(spk, sh_h, j0, min(WPT, L - j0), m);
  } else {
    for (int j = tid; j < L; j += SCANK_THREADS) sh_h[hp(j)] = mmer_hash_at(spk, (uint32_t)j, m);
  }
  __syncthreads();

  // minima of this thread's windows r0 .. r0 + 15 (window r spans h[r .. r + w - 1]):
  // van Herk / Gil-Werman blocks of w aligned at r0.  Window i is block
  // floor(i / w) when w divides i, else the suffix of that block from i plus
  // the prefix of the next block up to i + w - 1.
  uint32_t mvv[WPT];
  {
    const int nb_end = ((WPT - 1) / w + 1) * w;  // end of the block holding position 15
    uint32_t run = 0xffffffffu;
#pragma unroll
    for (int j = nb_end - 1; j >= WPT; j--) run = min(run, sh_h[hp(r0 + j)]);
    int rem = (WPT - 1) % w;  // position within its block, counting down
#pragma unroll
    for (int i = WPT - 1; i >= 0; i--) {
      run = min(run, sh_h[hp(r0 + i)]);
      mvv[i] = run;  // suffix minimum of the block, from i
      if (rem == 0) { run = 0xffffffffu; rem = w - 1; } else rem--;
    }
    int rb = 0;  // i mod w
#pragma unroll
    for (int i = 0; i < WPT; i++) {
      const uint32_t hy = sh_h[hp(r0 + i + w - 1)];
      if (rb == 0) run = 0xffffffffu;   // the window is one whole block
      else if (rb == 1) run = hy;       // first position of the next block
      else run = min(run, hy);
      if (w == 1) run = 0xffffffffu;
      mvv[i] = min(mvv[i], run);
      if (++rb == w) rb = 0;
    }
  }
#pragma unroll
  for (int i = 0; i < WPT; i++) sh_mv[hp(r0 + i)] = mvv[i];

  // validity, 32 windows per thread (threads 0 .. VBW-1): window r is valid iff
  // t0 + r + k <= n_bases and no fragment starts at r + 1 .. r + k - 1.  With
  // Y = fragment bits from position 32g + 1 on, the invalid windows are the
  // OR of Y over k - 1 consecutive bits, built by doubling shifts (fragment
  // starts are rare: most words skip it).
  if (tid < VBW) {
    const int g = tid;
    const uint64_t xlo = (uint64_t)sfb[g] | ((uint64_t)sfb[g + 1] << 32);
    const uint64_t xhi = (uint64_t)sfb[g + 2] | ((uint64_t)sfb[g + 3] << 32);
    uint64_t ylo = (xlo >> 1) | (xhi << 63), yhi = xhi >> 1;
    uint32_t inv = 0;
    const int span = k - 1;
    if (span > 0 && (ylo | yhi)) {
      int c = 1;
      while (2 * c <= span) { smear128(ylo, yhi, c); c *= 2; }
      if (c < span) smear128(ylo, yhi, span - c);
      inv = (uint32_t)ylo;
    }
    const uint64_t first = t0 + 32u * (uint64_t)g;
    uint32_t inb;
    if (first + 31u + (uint64_t)k <= nb) inb = 0xffffffffu;
    else if (first + (uint64_t)k > nb) inb = 0u;
    else inb = (1u << (uint32_t)(nb - (uint64_t)k - first + 1u)) - 1u;  // 1 .. 31 valid
    sh_vb[g] = ~inv & inb;
  }
  __syncthreads();
  uint32_t mv[WPT + 1];
  mv[0] = r0 > 0 ? sh_mv[hp(r0 - 1)] : 0u;  // the window before this thread's range
#pragma unroll
  for (int i = 1; i <= WPT; i++) mv[i] = mvv[i - 1];
  // 16-bit masks over this thread's windows (bit i = window r0 + i)
  const uint32_t vb = (sh_vb[r0 >> 5] >> (r0 & 31)) & 0xffffu;
  const uint32_t vbefore = r0 > 0 ? (sh_vb[(r0 - 1) >> 5] >> ((r0 - 1) & 31)) & 1u : 0u;
  const uint32_t vprev = ((vb << 1) | vbefore) & 0xffffu;  // validity of the window before
  uint32_t diff = 0;
#pragma unroll
  for (int i = 0; i < WPT; i++) diff |= (uint32_t)(mv[i + 1] != mv[i]) << i;
  const uint32_t starts = vb & (~vprev | diff);  // a run begins
  const uint32_t terms = ~vb & vprev;            // a run ends at an invalid window
  // key-range pass: only superkmers whose p1 digit is in [p1_lo, p1_hi) are
  // emitted; every start still ends the run before it
  const uint32_t p1_lo = a.p1_lo, p1_hi = a.p1_hi;
  const bool ranged = p1_lo > 0 || p1_hi < (uint32_t)NP1;  // uniform: one pass needs no check
  uint32_t emitm = starts;
  if (ranged) {
    uint32_t inr = 0;
#pragma unroll
    for (int i = 0; i < WPT; i++) inr |= (uint32_t)in_range(mv[i + 1], p1_lo, p1_hi) << i;
    emitm &= inr;
  }
  const Cnt2 c{(uint32_t)__popc(starts | terms), (uint32_t)__popc(emitm)};
  Cnt2 tot;
  const Cnt2 pre = block_exclusive_scan<Cnt2, Cnt2Op, SCANK_THREADS>(c, &tot, shc);
  // sh_h is free from here on (all reads of it finished before the scan's barriers)
  {
    uint32_t e = pre.ev;
    for (uint32_t evm = starts | terms; evm; evm &= evm - 1) {
      const int i = __ffs(evm) - 1;
      const uint32_t emit = (emitm >> i) & 1u;
      const uint32_t sr = pre.st + (uint32_t)__popc(emitm & ((1u << i) - 1u));
      ev[e++] = (uint32_t)(r0 + i) | (emit << 13) | (sr << 14);
    }
  }
  if (tid == 0) {
    ev[tot.ev] = (uint32_t)SCAN_TILE;  // sentinel: runs end at the tile edge
    unsigned long long base = atomicAdd(a.n_desc, (unsigned long long)tot.st);
    if (base + tot.st > a.desc_cap) set_status(a.status, ST_DESC_OVERFLOW);
    s_base = base;
  }
  __syncthreads();
  const unsigned long long base = s_base;
  if (base + tot.st > a.desc_cap) return;
  for (uint32_t e = tid; e < tot.ev; e += SCANK_THREADS) {
    const uint32_t v = ev[e];
    if (!((v >> 13) & 1u)) continue;
    const uint32_t r = v & 0x1fffu;
    const uint32_t end = ev[e + 1] & 0x1fffu;
    const uint32_t len = end - r;
    const uint32_t mval = sh_mv[hp((int)r)];
    const uint64_t d = base + (v >> 14);
    a.desc[d] = ((t0 + r) << 24) | (uint64_t)(len - 1);
    a.key[d] = mix32(mval);
  }
}

// packed bases a tile reads past its first window: the staged words and bits
constexpr uint64_t SCAN_NEED = (uint64_t)(PKW * 16 > FBW * 32 ? PKW * 16 : FBW * 32);

__global__ void k_scan_window(const uint64_t* __restrict__ avail, uint64_t* __restrict__ range, int final,
                              uint64_t max_tiles, uint32_t* __restrict__ status) {
  const uint64_t nb = *avail, lo = range[1];
  uint64_t hi;
  if (final) hi = (nb + SCAN_TILE - 1) / SCAN_TILE;
  else hi = nb >= SCAN_NEED ? (nb - SCAN_NEED) / SCAN_TILE + 1 : 0;
  if (hi < lo) hi = lo;
  if (hi - lo > max_tiles) {
    // more tiles than this launch covers: the rest waits for the next window,
    // and a final window that cannot finish sends the host to a full rescan
    hi = lo + max_tiles;
    if (final) atomicOr(status, ST_DESC_OVERFLOW);
  }
  range[0] = lo;
  range[1] = hi;
}

// the (k, m) pairs of the benchmark workloads get their own kernels
using ScanKernel = void (*)(ScanArgs);
static ScanKernel scan_kernel(int k, int m) {
  if (k == 63 && m == 21) return k_scan<63, 21>;
  if (k == 31 && m == 21) return k_scan<31, 21>;
  if (k == 31 && m == 19) return k_scan<31, 19>;
  return k_scan<0, 0>;
}

// the attribute is per device: set before every launch (a host-side call of
// microseconds, allowed during stream capture)
static ScanKernel scan_attr(const ScanArgs& a) {
  const ScanKernel f = scan_kernel(a.k, a.m);
  cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)scan_smem_bytes());
  return f;
}

void launch_scan(const ScanArgs& a, cudaStream_t s) {
  const uint64_t ntiles = (a.max_bases + SCAN_TILE - 1) / SCAN_TILE;
  if (ntiles == 0) return;
  const ScanKernel f = scan_attr(a);
  f<<<(unsigned)ntiles, SCANK_THREADS, scan_smem_bytes(), s>>>(a);
}

void launch_scan_window(const uint64_t* avail, uint64_t* range, bool final, uint64_t max_tiles, uint32_t* status,
                        cudaStream_t s) {
  k_scan_window<<<1, 1, 0, s>>>(avail, range, final ? 1 : 0, max_tiles, status);
}

void launch_scan_range(const ScanArgs& a, uint64_t max_tiles, cudaStream_t s) {
  if (max_tiles == 0) return;
  const ScanKernel f = scan_attr(a);
  f<<<(unsigned)max_tiles, SCANK_THREADS, scan_smem_bytes(), s>>>(a);
}

}  // namespace mczi
