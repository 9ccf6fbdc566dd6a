// zi.cu -- ZI on the GPU: a device-resident SSHash-style dictionary of the
// index k-mers and a streamed probe of query k-mers.
//
// Replaces ZI's build_dictionary (src/zi.rs:114-141, sshash-lib
// DictionaryBuilder::build_from_sequences) and its query loop
// collect_query_kmers_absent_from_index (src/zi.rs:152-175: per window
// `lookup(window).is_found()`, absent canonical k-mers into a set).
//
// Dictionary (all in HBM):
//   * the index's 2-bit stream, exactly as K1 packs it;
//   * its superkmers (K2), grouped into buckets by minimizer;
//   * an MPHF over the distinct minimizer keys, BBHash-style (Limasset et
//     al., "Fast and scalable minimal perfect hashing for massive key sets",
//     SEA 2017): level l keeps a bit array of gamma * (keys left) bits; a key
//     whose hashed position is hit by no other key owns that bit, the rest
//     retry at level l + 1; the index of a key is the rank of its bit;
//   * bucket offsets (CSR) from MPHF index to superkmer list.
// Membership of a query k-mer: its superkmer's minimizer key -> MPHF ->
// bucket -> compare against the canonical k-mers of the bucket's superkmers.
// The minimizer value is a function of the canonical k-mer (both strands hold
// the same canonical m-mers), so a present k-mer always finds its index
// superkmer in that bucket; a key outside the MPHF's set lands in an
// arbitrary bucket or none, and the comparison rejects it.  sshash-lib's own
// layout is not reproduced; only its answers are.
//
// Streaming: one lookup per query superkmer (consecutive windows share the
// minimizer), like sshash's streaming query.  Absent windows are emitted as
// run descriptors carrying the superkmer's partition key, so the MC partition
// and counting kernels (threshold 0) deduplicate them exactly.
#include "api_internal.h"
#include "mczi_common.cuh"
#include "scan.cuh"

#include <algorithm>
#include <cstring>
#include <vector>

namespace mczi {

namespace {

constexpr int ZI_THREADS = 256;
constexpr uint64_t MPHF_NOT_FOUND = ~0ull;
constexpr int Q_CHUNK = 8;

struct MphfView {
  const unsigned long long* bits;
  const uint32_t* rank;
  int levels;
  uint64_t off[MPHF_MAX_LEVELS];
  uint64_t size[MPHF_MAX_LEVELS];
};

__host__ __device__ __forceinline__ uint64_t level_seed(int l) {
  uint64_t z = 0x9E3779B97F4A7C15ull * (uint64_t)(l + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  return z ^ (z >> 27);
}

__device__ __forceinline__ uint64_t level_pos(uint32_t key, int l, uint64_t size) {
  const uint64_t h = mix64(((uint64_t)key << 7) ^ level_seed(l));
  return ((h & 0xffffffffull) * size) >> 32;
}

__device__ __forceinline__ uint64_t mphf_lookup(const MphfView& v, uint32_t key) {
  for (int l = 0; l < v.levels; l++) {
    const uint64_t p = v.off[l] + level_pos(key, l, v.size[l]);
    const unsigned long long w = v.bits[p >> 6];
    const uint32_t b = (uint32_t)(p & 63);
    if ((w >> b) & 1ull) return (uint64_t)v.rank[p >> 6] + (uint64_t)__popcll(w & ((1ull << b) - 1ull));
  }
  return MPHF_NOT_FOUND;
}

// ---- distinct keys of the index superkmers
__global__ void k_zi_key_set(const uint32_t* __restrict__ key, uint64_t n, unsigned long long* tab, uint64_t mask,
                             uint32_t* status) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t k = key[i];
    const unsigned long long want = ((unsigned long long)k << 32) | 1ull;
    uint64_t s = mix64((uint64_t)k ^ 0x2545F4914F6CDD1Dull) & mask;
    bool done = false;
    for (uint64_t probe = 0; probe <= mask; probe++) {
      unsigned long long cur = tab[s];
      if (cur == 0ull) {
        const unsigned long long prev = atomicCAS(&tab[s], 0ull, want);
        if (prev == 0ull) { done = true; break; }
        cur = prev;
      }
      if ((uint32_t)(cur >> 32) == k) { done = true; break; }
      s = (s + 1) & mask;
    }
    if (!done) set_status(status, ST_MINTAB_FULL);
  }
}

__global__ void k_zi_key_compact(const unsigned long long* __restrict__ tab, uint64_t slots, uint32_t* out,
                                 unsigned long long* n_out) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < slots; i += (uint64_t)gridDim.x * blockDim.x) {
    const unsigned long long v = tab[i];
    if (v) out[atomicAdd(n_out, 1ull)] = (uint32_t)(v >> 32);
  }
}

// ---- BBHash levels
__global__ void k_bb_mark(const uint32_t* __restrict__ keys, uint64_t n, int level, uint64_t size,
                          unsigned long long* A, unsigned long long* Cw) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t p = level_pos(keys[i], level, size);
    const unsigned long long bit = 1ull << (p & 63);
    const unsigned long long old = atomicOr(&A[p >> 6], bit);
    if (old & bit) atomicOr(&Cw[p >> 6], bit);
  }
}

__global__ void k_bb_next(const uint32_t* __restrict__ keys, uint64_t n, int level, uint64_t size,
                          const unsigned long long* __restrict__ Cw, uint32_t* next, unsigned long long* n_next) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t key = keys[i];
    const uint64_t p = level_pos(key, level, size);
    if ((Cw[p >> 6] >> (p & 63)) & 1ull) next[atomicAdd(n_next, 1ull)] = key;
  }
}

__global__ void k_bb_clear(unsigned long long* A, const unsigned long long* __restrict__ Cw, uint64_t words) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < words; i += (uint64_t)gridDim.x * blockDim.x)
    A[i] &= ~Cw[i];
}

__global__ void k_bb_popc(const unsigned long long* __restrict__ bits, uint64_t words, uint32_t* pc) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < words; i += (uint64_t)gridDim.x * blockDim.x)
    pc[i] = (uint32_t)__popcll(bits[i]);
}

// ---- buckets
__global__ void k_zi_bucket_count(const uint32_t* __restrict__ key, uint64_t n, MphfView v, uint64_t n_keys,
                                  uint32_t* cnt, uint32_t* status) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t b = mphf_lookup(v, key[i]);
    if (b >= n_keys) { set_status(status, ST_BAD_INDEX); continue; }
    atomicAdd(&cnt[b], 1u);
  }
}

__global__ void k_zi_bucket_fill(const uint64_t* __restrict__ desc, const uint32_t* __restrict__ key, uint64_t n,
                                 MphfView v, uint64_t n_keys, uint32_t* cursor, uint64_t* sk) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t b = mphf_lookup(v, key[i]);
    if (b >= n_keys) continue;
    sk[atomicAdd(&cursor[b], 1u)] = desc[i];
  }
}

struct ProbeArgs {
  const uint64_t* qdesc;
  const uint32_t* qkey;
  const unsigned long long* n_q;
  const uint32_t* qpacked;
  const uint32_t* ipacked;
  const uint64_t* sk;
  const uint32_t* bucket_off;
  uint64_t n_keys;
  MphfView v;
  int k;
  uint64_t* out_desc;
  uint32_t* out_key;
  unsigned long long* n_runs;
  uint64_t cap;
};

__device__ __forceinline__ void emit_run(const ProbeArgs& a, uint64_t start, uint32_t len, uint32_t key) {
  const unsigned long long idx = atomicAdd(a.n_runs, 1ull);
  if (idx < a.cap) {
    a.out_desc[idx] = (start << 24) | (uint64_t)(len - 1);
    a.out_key[idx] = key;
  }
}

template <class K, class R>
__device__ __forceinline__ void roll_set(R& r, const uint32_t* packed, uint64_t s0, int k) {
  r.init(k);
  if constexpr (sizeof(K) == 8) {
    r.set(field64(packed, s0, k), k);
  } else {
    if (k > 32) r.set(field64(packed, s0, k - 32), field64(packed, s0 + (uint64_t)(k - 32), 32), k);
    else r.set(0ull, field64(packed, s0, k), k);
  }
}

template <class K, class R>
__global__ void __launch_bounds__(ZI_THREADS) k_zi_probe(ProbeArgs a) {
  const uint64_t n = *a.n_q;
  const int k = a.k;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t d = a.qdesc[i];
    const uint64_t s0 = d >> 24;
    const uint32_t nw = (uint32_t)(d & 0xffffffu) + 1u;
    const uint32_t key = a.qkey[i];
    const uint64_t b = mphf_lookup(a.v, key);
    uint32_t blo = 0, bhi = 0;
    if (b < a.n_keys) { blo = a.bucket_off[b]; bhi = a.bucket_off[b + 1]; }
    int64_t run = -1;
    for (uint32_t c0 = 0; c0 < nw; c0 += Q_CHUNK) {
      const uint32_t cn = min((uint32_t)Q_CHUNK, nw - c0);
      K q[Q_CHUNK];
      {
        R r;
        roll_set<K, R>(r, a.qpacked, s0 + c0, k);
        uint64_t p = s0 + c0 + (uint64_t)k;
#pragma unroll
        for (int t = 0; t < Q_CHUNK; t++) {
          if (t < (int)cn) {
            if (t > 0) { r.push(base_at(a.qpacked, p)); p++; }
            q[t] = r.canon();
          }
        }
      }
      const uint32_t full = (cn == 32) ? 0xffffffffu : ((1u << cn) - 1u);
      uint32_t found = 0;
      for (uint32_t j = blo; j < bhi && found != full; j++) {
        const uint64_t e = a.sk[j];
        const uint64_t e0 = e >> 24;
        const uint32_t en = (uint32_t)(e & 0xffffffu) + 1u;
        R r;
        roll_set<K, R>(r, a.ipacked, e0, k);
        uint64_t p = e0 + (uint64_t)k;
        for (uint32_t u = 0; u < en; u++) {
          if (u > 0) { r.push(base_at(a.ipacked, p)); p++; }
          const K ek = r.canon();
#pragma unroll
          for (int t = 0; t < Q_CHUNK; t++)
            if (t < (int)cn && key_eq(q[t], ek)) found |= 1u << t;
          if (found == full) break;
        }
      }
      for (uint32_t t = 0; t < cn; t++) {
        const bool absent = !((found >> t) & 1u);
        if (absent) {
          if (run < 0) run = (int64_t)(c0 + t);
        } else if (run >= 0) {
          emit_run(a, s0 + (uint64_t)run, c0 + t - (uint32_t)run, key);
          run = -1;
        }
      }
    }
    if (run >= 0) emit_run(a, s0 + (uint64_t)run, nw - (uint32_t)run, key);
  }
}


// ---- per-input split of a batch result (records x masks -> per-input lists)
constexpr int SPLIT_CHUNK = 4096;
constexpr int SPLIT_MAX_INPUTS = 4096;

__global__ void __launch_bounds__(ZI_THREADS) k_zi_split_count(const unsigned long long* __restrict__ masks,
                                                               uint64_t n, int W, int n_inputs,
                                                               unsigned long long* __restrict__ cnt) {
  __shared__ uint32_t c[SPLIT_MAX_INPUTS];
  for (int i = threadIdx.x; i < n_inputs; i += blockDim.x) c[i] = 0;
  __syncthreads();
  const uint64_t c0 = (uint64_t)blockIdx.x * SPLIT_CHUNK;
  const uint64_t c1 = c0 + SPLIT_CHUNK < n ? c0 + SPLIT_CHUNK : n;
  for (uint64_t i = c0 + threadIdx.x; i < c1; i += blockDim.x)
    for (int q = 0; q < W; q++)
      for (unsigned long long m = masks[i * W + q]; m; m &= m - 1) atomicAdd(&c[q * 64 + __ffsll((long long)m) - 1], 1u);
  __syncthreads();
  for (int i = threadIdx.x; i < n_inputs; i += blockDim.x)
    if (c[i]) atomicAdd(&cnt[i], (unsigned long long)c[i]);
}

__global__ void __launch_bounds__(ZI_THREADS) k_zi_split_fill(const unsigned long long* __restrict__ masks,
                                                              const uint64_t* __restrict__ lo,
                                                              const uint64_t* __restrict__ hi, uint64_t n, int W,
                                                              int n_inputs, unsigned long long* __restrict__ cursor,
                                                              uint64_t* __restrict__ out_lo,
                                                              uint64_t* __restrict__ out_hi) {
  __shared__ uint32_t c[SPLIT_MAX_INPUTS];
  __shared__ unsigned long long base[SPLIT_MAX_INPUTS];
  for (int i = threadIdx.x; i < n_inputs; i += blockDim.x) c[i] = 0;
  __syncthreads();
  const uint64_t c0 = (uint64_t)blockIdx.x * SPLIT_CHUNK;
  const uint64_t c1 = c0 + SPLIT_CHUNK < n ? c0 + SPLIT_CHUNK : n;
  for (uint64_t i = c0 + threadIdx.x; i < c1; i += blockDim.x)
    for (int q = 0; q < W; q++)
      for (unsigned long long m = masks[i * W + q]; m; m &= m - 1) atomicAdd(&c[q * 64 + __ffsll((long long)m) - 1], 1u);
  __syncthreads();
  for (int i = threadIdx.x; i < n_inputs; i += blockDim.x) {
    base[i] = c[i] ? atomicAdd(&cursor[i], (unsigned long long)c[i]) : 0ull;
    c[i] = 0;
  }
  __syncthreads();
  for (uint64_t i = c0 + threadIdx.x; i < c1; i += blockDim.x)
    for (int q = 0; q < W; q++)
      for (unsigned long long m = masks[i * W + q]; m; m &= m - 1) {
        const int r = q * 64 + __ffsll((long long)m) - 1;
        const uint64_t o = base[r] + atomicAdd(&c[r], 1u);
        out_lo[o] = lo[i];
        if (out_hi) out_hi[o] = hi ? hi[i] : 0ull;
      }
}

int grid_for(mczi_ctx* ctx, uint64_t n) {
  const uint64_t g = (n + ZI_THREADS - 1) / ZI_THREADS;
  const uint64_t cap = (uint64_t)ctx->sm_count * 16;
  return (int)std::max<uint64_t>(1, std::min(g, cap));
}

struct SumU32 {
  static __device__ uint32_t identity() { return 0u; }
  static __device__ uint32_t combine(const uint32_t& a, const uint32_t& b) { return a + b; }
};

MphfView view_of(const ZiIndex& z) {
  MphfView v;
  v.bits = z.bits.as<unsigned long long>();
  v.rank = z.rank.as<uint32_t>();
  v.levels = z.levels;
  for (int l = 0; l < MPHF_MAX_LEVELS; l++) {
    v.off[l] = z.lvl_off[l];
    v.size[l] = z.lvl_size[l];
  }
  return v;
}

// ZI's validate_k (src/zi.rs:103-107) and minimizer bound (src/zi.rs:70-72)
int32_t zi_validate(mczi_ctx* ctx, uint32_t k, uint32_t m) {
  if (k < 3 || k > 63) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "k must be in [3, 63] for sshash-rs");
  if (k % 2 == 0) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "k must be odd for sshash-rs");
  if (m == 0 || m >= k) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "minimizer size must be > 0 and < k");
  return MCZI_OK;
}

int32_t zi_build(mczi_ctx* ctx, const uint8_t* fasta, uint64_t len, uint32_t k, uint32_t m) {
  int32_t rc = zi_validate(ctx, k, m);
  if (rc) return rc;
  ZiIndex& z = ctx->zi;
  z.built = false;
  mczi_input in{fasta, len};
  if ((rc = stage_inputs(ctx, &in, 1))) return rc;
  if (ctx->skipped) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "index FASTA does not start with a FASTA/FASTQ record");
  cudaStream_t s = ctx->stream;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaEventRecord(e0, s));
  Pipe p;
  if ((rc = pipe_pack(ctx, p))) return rc;
  uint64_t nb = 0;
  CK(cudaMemcpyAsync(&nb, p.d_nbases, 8, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (nb == 0)  // src/zi.rs:116-120
    return fail(ctx, MCZI_ERR_INVALID_CONFIG, "index FASTA did not contain any sequence of length >= k");
  if ((rc = pipe_scan(ctx, p, (int)k, (int)m))) return rc;
  const uint64_t n_desc = p.n_desc;
  uint64_t* sc = ctx->scalars.as<uint64_t>();
  // keep the index stream
  CKA(z.packed, p.pwords * 4);
  CK(cudaMemcpyAsync(z.packed.p, ctx->packed.p, p.pwords * 4, cudaMemcpyDeviceToDevice, s));
  z.pwords = p.pwords;
  z.n_bases = nb;
  z.k = (int)k;
  z.m = (int)m;
  z.n_sk = n_desc;
  // distinct minimizer keys
  uint64_t slots = 1024;
  while (slots < 2 * n_desc) slots <<= 1;
  CKA(ctx->zi_tmp0, slots * 8);
  CK(cudaMemsetAsync(ctx->zi_tmp0.p, 0, slots * 8, s));
  CK(cudaMemsetAsync(sc + SC_STATUS, 0, 8, s));
  CK(cudaMemsetAsync(sc + SC_NKEPT, 0, 8, s));
  const uint32_t* d_key = ctx->key.as<uint32_t>();
  if (n_desc) k_zi_key_set<<<grid_for(ctx, n_desc), ZI_THREADS, 0, s>>>(d_key, n_desc, ctx->zi_tmp0.as<unsigned long long>(),
                                                                       slots - 1, reinterpret_cast<uint32_t*>(sc + SC_STATUS));
  CKA(ctx->zi_tmp1, std::max<uint64_t>(n_desc, 1) * 4 * 2);  // two key lists (current, next level)
  uint32_t* keys_a = ctx->zi_tmp1.as<uint32_t>();
  uint32_t* keys_b = keys_a + std::max<uint64_t>(n_desc, 1);
  k_zi_key_compact<<<grid_for(ctx, slots), ZI_THREADS, 0, s>>>(ctx->zi_tmp0.as<unsigned long long>(), slots, keys_a,
                                                               reinterpret_cast<unsigned long long*>(sc + SC_NKEPT));
  CK(cudaGetLastError());
  uint64_t h[2];
  CK(cudaMemcpyAsync(h, sc + SC_NKEPT, 8, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(h + 1, sc + SC_STATUS, 8, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (h[1]) return fail(ctx, MCZI_ERR_DEVICE, "ZI key set overflow");
  const uint64_t n_keys = h[0];
  z.n_keys = n_keys;
  // BBHash levels, gamma = 2
  const uint64_t max_bits = 4 * n_keys + 128ull * MPHF_MAX_LEVELS + 64;
  const uint64_t max_words = max_bits / 64 + 1;
  CKA(z.bits, max_words * 8);
  CK(cudaMemsetAsync(z.bits.p, 0, max_words * 8, s));
  CKA(ctx->zi_tmp2, max_words * 8);  // collision words of the current level
  uint64_t off = 0, rem = n_keys;
  int l = 0;
  while (rem > 0) {
    if (l >= MPHF_MAX_LEVELS) return fail(ctx, MCZI_ERR_DEVICE, "MPHF construction did not converge");
    const uint64_t size = ((std::max<uint64_t>(64, 2 * rem) + 63) / 64) * 64;
    if ((off + size) / 64 > max_words) return fail(ctx, MCZI_ERR_DEVICE, "MPHF bit vector overflow");
    unsigned long long* A = z.bits.as<unsigned long long>() + off / 64;
    unsigned long long* Cw = ctx->zi_tmp2.as<unsigned long long>();
    CK(cudaMemsetAsync(Cw, 0, size / 8, s));
    CK(cudaMemsetAsync(sc + SC_NKEPT, 0, 8, s));
    k_bb_mark<<<grid_for(ctx, rem), ZI_THREADS, 0, s>>>(keys_a, rem, l, size, A, Cw);
    k_bb_next<<<grid_for(ctx, rem), ZI_THREADS, 0, s>>>(keys_a, rem, l, size, Cw, keys_b,
                                                        reinterpret_cast<unsigned long long*>(sc + SC_NKEPT));
    k_bb_clear<<<grid_for(ctx, size / 64), ZI_THREADS, 0, s>>>(A, Cw, size / 64);
    CK(cudaGetLastError());
    uint64_t nn = 0;
    CK(cudaMemcpyAsync(&nn, sc + SC_NKEPT, 8, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    z.lvl_off[l] = off;
    z.lvl_size[l] = size;
    off += size;
    rem = nn;
    std::swap(keys_a, keys_b);
    l++;
  }
  z.levels = l;
  z.lvl_off[l] = off;
  z.n_words = off / 64 + 1;
  // rank: exclusive prefix of per-word popcounts
  CKA(z.rank, (z.n_words + 1) * 4);
  CKA(ctx->zi_tmp0, std::max<uint64_t>(slots * 8, (z.n_words + 1) * 4 + (z.n_words / SCAN_CHUNK + 2) * 4));
  uint32_t* pc = ctx->zi_tmp0.as<uint32_t>();
  uint32_t* tmp = pc + z.n_words + 1;
  k_bb_popc<<<grid_for(ctx, z.n_words), ZI_THREADS, 0, s>>>(z.bits.as<unsigned long long>(), z.n_words, pc);
  exclusive_scan<uint32_t, SumU32>(pc, z.rank.as<uint32_t>(), z.n_words, tmp, s);
  CK(cudaGetLastError());
  // buckets: CSR from MPHF index to superkmers
  const MphfView v = view_of(z);
  CKA(z.bucket_off, (n_keys + 2) * 4);
  CKA(z.sk, std::max<uint64_t>(n_desc, 1) * 8);
  uint32_t* cnt = ctx->zi_tmp1.as<uint32_t>();  // reuse: n_keys + 1 <= 2 * n_desc words
  CKA(ctx->zi_tmp1, std::max<uint64_t>((n_keys + 2) * 4 * 2 + (n_keys / SCAN_CHUNK + 2) * 4, 16));
  cnt = ctx->zi_tmp1.as<uint32_t>();
  uint32_t* cursor = cnt + n_keys + 1;
  CK(cudaMemsetAsync(cnt, 0, (n_keys + 1) * 4, s));
  CK(cudaMemsetAsync(sc + SC_STATUS, 0, 8, s));
  if (n_desc) {
    k_zi_bucket_count<<<grid_for(ctx, n_desc), ZI_THREADS, 0, s>>>(d_key, n_desc, v, n_keys, cnt,
                                                                   reinterpret_cast<uint32_t*>(sc + SC_STATUS));
    exclusive_scan<uint32_t, SumU32>(cnt, z.bucket_off.as<uint32_t>(), n_keys, cursor + n_keys + 1, s);
    CK(cudaMemcpyAsync(cursor, z.bucket_off.p, (n_keys + 1) * 4, cudaMemcpyDeviceToDevice, s));
    k_zi_bucket_fill<<<grid_for(ctx, n_desc), ZI_THREADS, 0, s>>>(ctx->desc.as<uint64_t>(), d_key, n_desc, v, n_keys,
                                                                  cursor, z.sk.as<uint64_t>());
  } else {
    CK(cudaMemsetAsync(z.bucket_off.p, 0, 8, s));
  }
  CK(cudaGetLastError());
  CK(cudaEventRecord(e1, s));
  CK(cudaMemcpyAsync(h + 1, sc + SC_STATUS, 8, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (h[1] & ST_BAD_INDEX) return fail(ctx, MCZI_ERR_DEVICE, "MPHF missed an index key");
  CK(cudaEventElapsedTime(&z.build_ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  z.built = true;
  ctx->have_result = false;
  return MCZI_OK;
}

// absent k-mers of the staged queries; per_input: records carry input masks
int32_t zi_query(mczi_ctx* ctx, const mczi_input* q, size_t n, bool per_input, uint64_t* n_out) {
  ZiIndex& z = ctx->zi;
  if (!z.built) return fail(ctx, MCZI_ERR_STATE, "no ZI index: call mczi_zi_build first");
  int32_t rc;
  if (n == 0) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "at least one query FASTA is required");
  if ((rc = stage_inputs(ctx, q, n))) return rc;
  ctx->have_result = false;
  ctx->mask_words = 0;
  for (int i = 0; i < N_PHASES; i++) ctx->phase_ms[i] = 0.f;
  std::memset(ctx->stats, 0, sizeof ctx->stats);
  cudaStream_t s = ctx->stream;
  Pipe p;
  if ((rc = pipe_pack(ctx, p))) return rc;
  if ((rc = pipe_scan(ctx, p, z.k, z.m))) return rc;
  uint64_t* sc = ctx->scalars.as<uint64_t>();
  // probe: absent-window runs into (desc2, key2)
  uint64_t cap = 2 * p.n_desc + 1024;
  uint64_t n_runs = 0;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaEventRecord(e0, s));
  for (int attempt = 0; attempt < 3 && p.n_desc; attempt++) {
    // (desc, key) hold the query superkmers being probed; the runs go to
    // (desc2, key2), which become the partition's input after the swap
    if (cap > p.desc_cap) p.desc_cap = cap;
    CKA(ctx->desc2, cap * 8);
    CKA(ctx->key2, cap * 4);
    CK(cudaMemsetAsync(sc + SC_NRUNS, 0, 8, s));
    ProbeArgs pa;
    pa.qdesc = ctx->desc.as<uint64_t>();
    pa.qkey = ctx->key.as<uint32_t>();
    pa.n_q = reinterpret_cast<const unsigned long long*>(sc + SC_NDESC);
    pa.qpacked = ctx->packed.as<uint32_t>();
    pa.ipacked = z.packed.as<uint32_t>();
    pa.sk = z.sk.as<uint64_t>();
    pa.bucket_off = z.bucket_off.as<uint32_t>();
    pa.n_keys = z.n_keys;
    pa.v = view_of(z);
    pa.k = z.k;
    pa.out_desc = ctx->desc2.as<uint64_t>();
    pa.out_key = ctx->key2.as<uint32_t>();
    pa.n_runs = reinterpret_cast<unsigned long long*>(sc + SC_NRUNS);
    pa.cap = cap;
    const int grid = grid_for(ctx, p.n_desc);
    if (z.k <= 32) k_zi_probe<K64, Roll64><<<grid, ZI_THREADS, 0, s>>>(pa);
    else k_zi_probe<K128, Roll128><<<grid, ZI_THREADS, 0, s>>>(pa);
    p.launches += 1;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(&n_runs, sc + SC_NRUNS, 8, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (n_runs <= cap) break;
    cap = n_runs + 1024;
    if (attempt == 2) return fail(ctx, MCZI_ERR_DEVICE, "absent-run buffer overflow persisted");
  }
  CK(cudaEventRecord(e1, s));
  std::swap(ctx->desc, ctx->desc2);
  std::swap(ctx->key, ctx->key2);
  p.n_desc = n_runs;
  CK(cudaMemcpyAsync(sc + SC_NDESC, &p.n_desc, 8, cudaMemcpyHostToDevice, s));
  CK(cudaStreamSynchronize(s));
  float probe_ms = 0.f;
  CK(cudaEventElapsedTime(&probe_ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if ((rc = pipe_partition(ctx, p))) return rc;
  const int mode = per_input ? MCZI_MODE_PRESENCE : MCZI_MODE_ABUNDANCE;
  uint64_t out = 0;
  if ((rc = pipe_count(ctx, p, z.k, 0, mode, per_input, &out))) return rc;
  if ((rc = pipe_finish(ctx, p, mode, z.k, z.m, 0, out))) return rc;
  // phases for ZI: [0] pack, [1] scan, [2] partition, [3] dedup count, [4] probe
  ctx->phase_ms[1] -= probe_ms;
  ctx->phase_ms[4] = probe_ms;
  ctx->stats[1] = n_runs;
  if (n_out) *n_out = out;
  (void)p.n_desc_total;
  return MCZI_OK;
}

}  // namespace

}  // namespace mczi

using namespace mczi;

extern "C" {

int32_t mczi_zi_build(mczi_ctx* ctx, const uint8_t* index_fasta, uint64_t len, uint32_t k, uint32_t m) {
  if (!ctx) return MCZI_ERR_STATE;
  cudaSetDevice(ctx->device);
  return zi_build(ctx, index_fasta, len, k, m);
}

int32_t mczi_zi_query(mczi_ctx* ctx, const mczi_input* queries, size_t n, uint64_t* n_absent) {
  if (!ctx) return MCZI_ERR_STATE;
  cudaSetDevice(ctx->device);
  return zi_query(ctx, queries, n, false, n_absent);
}

int32_t mczi_zi_query_per_input(mczi_ctx* ctx, const mczi_input* queries, size_t n, uint64_t* n_records) {
  if (!ctx) return MCZI_ERR_STATE;
  cudaSetDevice(ctx->device);
  return zi_query(ctx, queries, n, true, n_records);
}

int32_t mczi_zi_input_result(mczi_ctx* ctx, int32_t input, uint64_t* key_lo, uint64_t* key_hi, uint64_t cap,
                             uint64_t* n) {
  if (!ctx) return MCZI_ERR_STATE;
  if (!ctx->have_result || ctx->mask_words == 0) return fail(ctx, MCZI_ERR_STATE, "no per-input ZI result");
  if (input < 0 || input >= ctx->n_inputs) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "input index out of range");
  cudaSetDevice(ctx->device);
  const uint64_t nr = ctx->n_out;
  const int W = ctx->mask_words;
  std::vector<uint64_t> lo(nr), hi(ctx->k > 32 ? nr : 0), msk(nr * (uint64_t)W);
  if (nr) {
    CK(cudaMemcpyAsync(lo.data(), ctx->out_lo.p, nr * 8, cudaMemcpyDeviceToHost, ctx->stream));
    if (ctx->k > 32) CK(cudaMemcpyAsync(hi.data(), ctx->out_hi.p, nr * 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(msk.data(), ctx->out_mask.p, nr * 8 * W, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  std::vector<uint64_t> idx;
  for (uint64_t i = 0; i < nr; i++)
    if ((msk[i * W + (input >> 6)] >> (input & 63)) & 1ull) idx.push_back(i);
  if (ctx->k > 32)
    std::sort(idx.begin(), idx.end(), [&](uint64_t a, uint64_t b) { return hi[a] < hi[b] || (hi[a] == hi[b] && lo[a] < lo[b]); });
  else
    std::sort(idx.begin(), idx.end(), [&](uint64_t a, uint64_t b) { return lo[a] < lo[b]; });
  if (n) *n = idx.size();
  if (!key_lo) return MCZI_OK;
  if (cap < idx.size()) return fail(ctx, MCZI_ERR_STATE, "result buffer too small");
  for (size_t i = 0; i < idx.size(); i++) {
    key_lo[i] = lo[idx[i]];
    if (key_hi) key_hi[i] = ctx->k > 32 ? hi[idx[i]] : 0;
  }
  return MCZI_OK;
}

int32_t mczi_zi_result_masks(mczi_ctx* ctx, uint64_t* masks, uint64_t cap_words, int32_t* words_per_record) {
  if (!ctx) return MCZI_ERR_STATE;
  if (!ctx->have_result || ctx->mask_words == 0) return fail(ctx, MCZI_ERR_STATE, "no per-input ZI result");
  if (words_per_record) *words_per_record = ctx->mask_words;
  if (!masks) return MCZI_OK;
  const uint64_t need = ctx->n_out * (uint64_t)ctx->mask_words;
  if (cap_words < need) return fail(ctx, MCZI_ERR_STATE, "mask buffer too small");
  cudaSetDevice(ctx->device);
  if (need) {
    CK(cudaMemcpyAsync(masks, ctx->out_mask.p, need * 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  return MCZI_OK;
}

int32_t mczi_zi_batch_split(mczi_ctx* ctx, uint64_t* key_lo, uint64_t* key_hi, uint64_t* offsets, uint64_t cap,
                            uint64_t* total) {
  if (!ctx) return MCZI_ERR_STATE;
  if (!ctx->have_result || ctx->mask_words == 0) return fail(ctx, MCZI_ERR_STATE, "no per-input ZI result");
  const int ni = ctx->n_inputs;
  if (ni > SPLIT_MAX_INPUTS) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "more than 4096 inputs in one batch");
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  const uint64_t nr = ctx->n_out;
  const int W = ctx->mask_words;
  const bool wide = ctx->k > 32;
  // per-input sizes on the device (block-aggregated), offsets on the host
  CKA(ctx->zi_tmp0, ((size_t)ni + 1) * 8 * 2);
  unsigned long long* cnt = ctx->zi_tmp0.as<unsigned long long>();
  unsigned long long* cursor = cnt + ni + 1;
  CK(cudaMemsetAsync(cnt, 0, ((size_t)ni + 1) * 8, s));
  const unsigned blocks = (unsigned)((nr + SPLIT_CHUNK - 1) / SPLIT_CHUNK);
  if (nr) k_zi_split_count<<<blocks, ZI_THREADS, 0, s>>>(ctx->out_mask.as<unsigned long long>(), nr, W, ni, cnt);
  CK(cudaGetLastError());
  std::vector<uint64_t> off((size_t)ni + 1, 0);
  CK(cudaMemcpyAsync(off.data() + 1, cnt, (size_t)ni * 8, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  for (int i = 0; i < ni; i++) off[i + 1] += off[i];
  if (total) *total = off[ni];
  if (offsets) std::copy(off.begin(), off.end(), offsets);
  if (!key_lo) return MCZI_OK;
  if (cap < off[ni]) return fail(ctx, MCZI_ERR_STATE, "result buffer too small");
  if (off[ni] == 0) return MCZI_OK;
  CKA(ctx->zi_tmp1, off[ni] * 8 * (wide ? 2 : 1));
  uint64_t* dlo = ctx->zi_tmp1.as<uint64_t>();
  uint64_t* dhi = wide ? dlo + off[ni] : nullptr;
  CK(cudaMemcpyAsync(cursor, off.data(), (size_t)ni * 8, cudaMemcpyHostToDevice, s));
  k_zi_split_fill<<<blocks, ZI_THREADS, 0, s>>>(ctx->out_mask.as<unsigned long long>(), ctx->out_lo.as<uint64_t>(),
                                                wide ? ctx->out_hi.as<uint64_t>() : nullptr, nr, W, ni, cursor, dlo,
                                                dhi);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(key_lo, dlo, off[ni] * 8, cudaMemcpyDeviceToHost, s));
  if (key_hi) {
    if (wide) CK(cudaMemcpyAsync(key_hi, dhi, off[ni] * 8, cudaMemcpyDeviceToHost, s));
    else std::fill(key_hi, key_hi + off[ni], 0ull);
  }
  CK(cudaStreamSynchronize(s));
  return MCZI_OK;
}

int32_t mczi_zi_info(mczi_ctx* ctx, uint64_t* out, int32_t cap) {
  if (!ctx) return MCZI_ERR_STATE;
  const ZiIndex& z = ctx->zi;
  const uint64_t v[8] = {z.built ? 1ull : 0ull, (uint64_t)z.k, (uint64_t)z.m, z.n_bases, z.n_sk, z.n_keys,
                         (uint64_t)z.levels, (uint64_t)(z.build_ms * 1000.f)};
  const int32_t n = std::min<int32_t>(cap, 8);
  for (int32_t i = 0; i < n; i++) out[i] = v[i];
  return n;
}

}  // extern "C"
