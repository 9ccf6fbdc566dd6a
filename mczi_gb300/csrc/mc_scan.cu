// mc_scan.cu -- K2: canonical minimizer scan and superkmer extraction.
//
// Replaces simd-minimizers' canonical scan + `run_hashes` and MC's run
// visitor (src/lib.rs:3694-3789; vendor/simd-minimizers-2.3.1/src/
// minimizers.rs:259-291, sliding_min.rs:556-593, collect.rs:116-286).
//
// Order: every m-mer is hashed as H(min(fwd, rc)); a window's minimizer value
// is the minimum of the w = k - m + 1 hashes it contains.  Both strands of a
// k-mer contain the same canonical m-mers, so the minimizer value -- and the
// partition derived from it -- is a function of the canonical k-mer alone,
// which is the invariant MC's counting relies on (each k-mer occurrence lands
// in the partition of its canonical form).  A superkmer is a maximal run of
// consecutive valid windows with the same minimizer value, cut at tile edges.
//
// One CTA scans SCAN_TILE windows of the concatenated base stream, so reads of
// any length (150 bp .. 100 kbp) are load-balanced by construction.  The
// sliding minimum uses van Herk / Gil-Werman blocks of w in shared memory
// (a constant number of shared-memory accesses per position, whatever w is).
#include "mczi_internal.h"
#include "mczi_common.cuh"
#include "scan.cuh"

namespace mczi {

namespace {

constexpr int MAXW = 64;
constexpr int HL = SCAN_TILE + MAXW;                 // hashes per tile
constexpr int PKW = (SCAN_TILE + 128) / 16 + 4;      // packed words staged
constexpr int FBW = (SCAN_TILE + 128) / 32 + 4;      // fragment-bit words staged
constexpr int WPT = SCAN_TILE / SCANK_THREADS;       // windows per thread
static_assert(SCAN_TILE <= 8192, "event encoding holds 13-bit positions");

struct Cnt2 {
  uint32_t ev, st;
};
struct Cnt2Op {
  static __device__ Cnt2 identity() { return Cnt2{0, 0}; }
  static __device__ Cnt2 combine(const Cnt2& a, const Cnt2& b) { return Cnt2{a.ev + b.ev, a.st + b.st}; }
};

__device__ __forceinline__ uint32_t mmer_hash_at(const uint32_t* spk, uint32_t rel, int m) {
  if (m <= 32) {
    const uint64_t f = field64_s(spk, rel, m);
    const uint64_t r = rc64_full(f) >> (64 - 2 * m);
    return mmer_hash64(f < r ? f : r);
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

__device__ __forceinline__ bool in_range(uint32_t mval, uint32_t lo, uint32_t hi) {
  const uint32_t p1 = mix32(mval) >> (32 - P1_BITS);
  return p1 >= lo && p1 < hi;
}

// 64 fragment-start bits beginning at relative bit q
__device__ __forceinline__ uint64_t bits64(const uint32_t* sfb, uint32_t q) {
  const uint32_t i = q >> 5, o = q & 31;
  const uint64_t a = (uint64_t)sfb[i] | ((uint64_t)sfb[i + 1] << 32);
  const uint64_t b = (uint64_t)sfb[i + 2];
  return o ? ((a >> o) | (b << (64 - o))) : a;
}

}  // namespace

constexpr int MVL = SCAN_TILE + SCAN_TILE / 32 + 2;  // padded minimizer values
constexpr int VBW = SCAN_TILE / 32;                   // validity bitmask words

size_t scan_smem_bytes() { return (size_t)(PKW + FBW + 3 * HL + MVL + VBW) * sizeof(uint32_t); }

__global__ void __launch_bounds__(SCANK_THREADS) k_scan(ScanArgs a) {
  extern __shared__ __align__(16) uint32_t dyn[];
  uint32_t* spk = dyn;
  uint32_t* sfb = spk + PKW;
  uint32_t* sh_h = sfb + FBW;
  uint32_t* sh_pl = sh_h + HL;
  uint32_t* sh_sr = sh_pl + HL;
  uint32_t* sh_mv = sh_sr + HL;
  uint32_t* sh_vb = sh_mv + MVL;
  uint32_t* ev = sh_h;  // reused once the minima are known: pos | start << 13 | rank << 14
  __shared__ Cnt2 shc[SCAN_THREADS + 1];
  __shared__ unsigned long long s_base;

  const uint64_t nb = *a.n_bases;
  const uint64_t t0 = (uint64_t)blockIdx.x * SCAN_TILE;
  const int k = a.k, m = a.m, w = k - m + 1;
  if (t0 + (uint64_t)k > nb) return;  // no valid window in this tile (uniform per CTA)
  const int tid = threadIdx.x;

  // stage packed words and fragment bits (t0 is a multiple of 32)
  const uint64_t pw0 = t0 >> 4, fw0 = t0 >> 5;
  for (int i = tid; i < PKW; i += SCANK_THREADS) {
    const uint64_t wi = pw0 + (uint64_t)i;
    spk[i] = wi < a.packed_words ? a.packed[wi] : 0u;
  }
  const uint64_t fwords = (a.packed_words + 1) >> 1;
  for (int i = tid; i < FBW; i += SCANK_THREADS) {
    const uint64_t wi = fw0 + (uint64_t)i;
    sfb[i] = wi < fwords ? a.fbits[wi] : 0u;
  }
  __syncthreads();

  // m-mer hashes for positions [t0, t0 + SCAN_TILE + w - 1)
  const int L = SCAN_TILE + w - 1;
  for (int j = tid; j < L; j += SCANK_THREADS) sh_h[j] = mmer_hash_at(spk, (uint32_t)j, m);
  __syncthreads();

  // van Herk / Gil-Werman: prefix and suffix minima inside blocks of w
  const int nblk = (L + w - 1) / w;
  for (int b = tid; b < nblk; b += SCANK_THREADS) {
    const int lo = b * w, hi = min(lo + w, L);
    uint32_t run = 0xffffffffu;
    for (int j = lo; j < hi; j++) { run = min(run, sh_h[j]); sh_pl[j] = run; }
    run = 0xffffffffu;
    for (int j = hi - 1; j >= lo; j--) { run = min(run, sh_h[j]); sh_sr[j] = run; }
  }
  __syncthreads();

  // per window: minimizer value and validity, computed with consecutive
  // threads on consecutive windows (conflict-free), kept as a padded array and
  // a bitmask for the per-thread run logic below
  const uint64_t vmask = (k - 1) >= 64 ? ~0ull : ((1ull << (k - 1)) - 1);
  for (int r = tid; r < SCAN_TILE; r += SCANK_THREADS) {
    const uint64_t gi = t0 + (uint64_t)r;
    bool v = (gi + (uint64_t)k <= nb);
    if (v && k > 1) v = (bits64(sfb, (uint32_t)(r + 1)) & vmask) == 0;
    const unsigned bal = __ballot_sync(0xffffffffu, v);
    if ((tid & 31) == 0) sh_vb[r >> 5] = bal;
    sh_mv[r + (r >> 5)] = min(sh_sr[r], sh_pl[r + w - 1]);
  }
  __syncthreads();
  const int r0 = tid * WPT;
  uint32_t mv[WPT + 1];
  bool vd[WPT + 1];
#pragma unroll
  for (int i = 0; i <= WPT; i++) {
    const int r = r0 + i - 1;  // i = 0 is the window before this thread's range
    if (r < 0) { vd[i] = false; mv[i] = 0; continue; }
    vd[i] = (sh_vb[r >> 5] >> (r & 31)) & 1u;
    mv[i] = sh_mv[r + (r >> 5)];
  }
  // key-range pass: only superkmers whose p1 digit is in [p1_lo, p1_hi) are
  // emitted; every start still ends the run before it
  const uint32_t p1_lo = a.p1_lo, p1_hi = a.p1_hi;
  const bool ranged = p1_lo > 0 || p1_hi < (uint32_t)NP1;  // uniform: one pass needs no check
  Cnt2 c{0, 0};
#pragma unroll
  for (int i = 1; i <= WPT; i++) {
    const int r = r0 + i - 1;
    const bool start = vd[i] && (r == 0 || !vd[i - 1] || mv[i] != mv[i - 1]);
    const bool term = !vd[i] && r > 0 && vd[i - 1];
    c.ev += (start || term);
    if (start) c.st += !ranged || in_range(mv[i], p1_lo, p1_hi);
  }
  Cnt2 tot;
  const Cnt2 pre = block_exclusive_scan<Cnt2, Cnt2Op>(c, &tot, shc);
  // sh_h is free from here on (all reads of it finished before the scan's barriers)
  {
    uint32_t e = pre.ev, sr = pre.st;
#pragma unroll
    for (int i = 1; i <= WPT; i++) {
      const int r = r0 + i - 1;
      const bool start = vd[i] && (r == 0 || !vd[i - 1] || mv[i] != mv[i - 1]);
      const bool term = !vd[i] && r > 0 && vd[i - 1];
      const bool emit = start && (!ranged || in_range(mv[i], p1_lo, p1_hi));
      if (start || term) {
        ev[e] = (uint32_t)r | ((uint32_t)emit << 13) | (sr << 14);
        e++;
      }
      sr += emit;
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
    const uint32_t mval = sh_mv[r + (r >> 5)];
    const uint64_t d = base + (v >> 14);
    a.desc[d] = ((t0 + r) << 24) | (uint64_t)(len - 1);
    a.key[d] = mix32(mval);
  }
}

void launch_scan(const ScanArgs& a, cudaStream_t s) {
  const uint64_t ntiles = (a.max_bases + SCAN_TILE - 1) / SCAN_TILE;
  if (ntiles == 0) return;
  const size_t smem = scan_smem_bytes();
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(k_scan, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr_set = true;
  }
  k_scan<<<(unsigned)ntiles, SCANK_THREADS, smem, s>>>(a);
}

}  // namespace mczi
