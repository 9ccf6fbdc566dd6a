// api_internal.h -- the context object and the pipeline stages shared by the
// MC and ZI host code of libmczi_gpu (not part of the public C ABI).
#pragma once
#include "../../include/mczi_gpu.h"
#include "mczi_internal.h"

#include <string>
#include <vector>

namespace mczi {

// owns one device allocation: freed when the owner (the context) is deleted;
// movable (the pipeline swaps buffers), not copyable
struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), cap(o.cap) {
    o.p = nullptr;
    o.cap = 0;
  }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p;
      cap = o.cap;
      o.p = nullptr;
      o.cap = 0;
    }
    return *this;
  }
  ~DevBuf() { release(); }
  // grows by at least half the current size, so a stream of slightly larger
  // requests does not reallocate (cudaFree synchronises the whole device)
  cudaError_t ensure(size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (bytes <= cap) return cudaSuccess;
    const size_t want = cap && bytes < cap + cap / 2 ? cap + cap / 2 : bytes;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess && want > bytes) {
      cudaGetLastError();
      e = cudaMalloc(&p, bytes);
      if (e == cudaSuccess) cap = bytes;
      return e;
    }
    if (e == cudaSuccess) cap = want;
    return e;
  }
  // grows like ensure() but keeps the first `keep` bytes
  cudaError_t grow_keep(size_t bytes, size_t keep, cudaStream_t s) {
    if (bytes <= cap) return cudaSuccess;
    if (!p || keep == 0) return ensure(bytes);
    const size_t want = bytes < cap + cap / 2 ? cap + cap / 2 : bytes;
    void* np = nullptr;
    cudaError_t e = cudaMalloc(&np, want);
    if (e != cudaSuccess) return e;
    e = cudaMemcpyAsync(np, p, keep, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { cudaFree(np); return e; }
    cudaFree(p);
    p = np;
    cap = want;
    return cudaSuccess;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  template <class T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

// owns one pinned host allocation (device-to-host copies at the link's speed)
struct HostPinned {
  void* p = nullptr;
  size_t cap = 0;
  HostPinned() = default;
  HostPinned(const HostPinned&) = delete;
  HostPinned& operator=(const HostPinned&) = delete;
  ~HostPinned() { release(); }
  cudaError_t ensure(size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (bytes <= cap) return cudaSuccess;
    const size_t want = cap && bytes < cap + cap / 2 ? cap + cap / 2 : bytes;
    release();
    cudaError_t e = cudaHostAlloc(&p, want, cudaHostAllocDefault);
    if (e != cudaSuccess) {
      p = nullptr;
      return e;
    }
    cap = want;
    return cudaSuccess;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
  }
};

// device scalars, in u64 slots
enum { SC_NDESC = 0, SC_NOUT = 1, SC_STATS = 2, SC_STATUS = 10, SC_WORK = 11, SC_NKEPT = 12, SC_NRUNS = 13,
       SC_SCANST = 14, SC_NABSW = 15, SC_COUNT = 16 };

constexpr int N_PHASES = 5;
constexpr int MPHF_MAX_LEVELS = 40;

// device-resident SSHash-style dictionary of the ZI index
struct ZiIndex {
  bool built = false;
  int k = 0, m = 0;
  DevBuf packed;         // the index's 2-bit stream (its own copy)
  uint64_t pwords = 0;
  uint64_t n_bases = 0;
  DevBuf sk;             // superkmer descriptors grouped by bucket
  DevBuf bucket_off;     // n_keys + 1 offsets into sk (u32)
  DevBuf bucket_key;     // the superkmer key (minimizer) of each bucket (u32)
  DevBuf bits, rank;     // MPHF bit vector (u64 words) and per-word rank (u32)
  DevBuf mfilter;        // blocked Bloom filter of the minimizer keys (u64 words)
  uint64_t mf_mask = 0;  // its words - 1 (a power of two)
  uint64_t n_keys = 0, n_sk = 0, n_words = 0;
  int levels = 0;
  uint64_t lvl_off[MPHF_MAX_LEVELS + 1] = {};
  uint64_t lvl_size[MPHF_MAX_LEVELS] = {};
  float build_ms = 0.f;
};

// what a captured pipeline depends on; replay only when it matches
struct GraphSig {
  uint64_t text_len = 0, n_tiles = 0, x = 0, desc_cap = 0, out_cap = 0;
  int n_inputs = 0, k = 0, m = 0, mode = 0;
  uint32_t passes = 0, slots = 0, fwords = 0;
  int threads = 0, cps = 0, chunk = 0, filter = 0;
  float fill = 0.f;
  const void* ptrs[13] = {};
  bool operator==(const GraphSig& o) const {
    if (text_len != o.text_len || n_tiles != o.n_tiles || x != o.x || desc_cap != o.desc_cap || out_cap != o.out_cap ||
        n_inputs != o.n_inputs || k != o.k || m != o.m || mode != o.mode || passes != o.passes || slots != o.slots ||
        fwords != o.fwords || threads != o.threads || cps != o.cps || chunk != o.chunk || filter != o.filter ||
        fill != o.fill)
      return false;
    for (int i = 0; i < 13; i++)
      if (ptrs[i] != o.ptrs[i]) return false;
    return true;
  }
};

}  // namespace mczi

struct mczi_ctx {
  int device = 0;
  int sm_count = 0;
  size_t smem_optin = 0;
  size_t smem_per_sm = 0;
  size_t smem_reserved = 0;            // reserved shared memory per block
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  std::string err;

  mczi::DevBuf text, tile_info, input_tile0, line_sum, line_pre, line_tmp, base_sum, base_pre, base_tmp;
  mczi::DevBuf packed, fbits, input_base;
  mczi::DevBuf desc, key, desc2, key2, part_hist, bucket_off;
  mczi::DevBuf out_lo, out_hi, out_cnt, out_mask;
  mczi::DevBuf cnt64;  // counts widened to u64 for direct copies to the caller
  mczi::DevBuf digest_acc;  // mczi_result_digest accumulators (3 u64)
  mczi::DevBuf count_scratch;  // per-CTA window words of fast filtered counting rounds
  std::vector<std::vector<uint8_t>> route;  // mczi_route_superkmers: FASTA records per destination GPU
  mczi::DevBuf kff_dev;          // KFF records formatted on the device
  mczi::HostPinned kff_host;     // their host copy, written to the file as is
  mczi::DevBuf sx_keys, sx_tab, sx_rank, sx_ext;  // simplitig writer: sorted keys, key->rank table, extensions
  mczi::DevBuf stream_scratch;     // streamed staging: pack carries, scan tile range
  // gzip inputs decoded on the device: compressed bytes, member table, work
  // counter / status / per-input formats, and the output of mczi_inflate_gzip
  mczi::DevBuf gz_comp, gz_members, gz_scratch, gz_out;
  cudaStream_t copy_stream = nullptr;  // host-to-device copies of the streamed staging
  cudaEvent_t ev_copy = nullptr;       // last copied segment
  int streamed = 1;                    // one-shot counts overlap staging with pack + scan
  uint64_t stream_seg_tiles = 0;       // segment size in pack tiles (0 = automatic)
  uint32_t zi_bucket_records = 0;      // records per final ZI dedup bucket (0 = half a table)
  mczi::DevBuf scalars;
  mczi::DevBuf mintab, pairtab;
  mczi::DevBuf zi_tmp0, zi_tmp1, zi_tmp2, zi_tmp3, zi_tmp4;

  // staged inputs
  bool staged = false;
  uint64_t text_len = 0, n_tiles = 0;
  int n_inputs = 0;
  uint64_t skipped = 0;
  uint64_t h2d_bytes = 0;

  // last result
  bool have_result = false;
  int mode = 0, k = 0, m = 0;
  uint64_t x = 0;
  uint64_t n_out = 0;
  int mask_words = 0;  // > 0 when the last result carries per-input masks
  float phase_ms[mczi::N_PHASES] = {0, 0, 0, 0, 0};
  float inflate_ms = 0.f;  // device gzip decoding of the last call that decoded members
  uint64_t stats[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  cudaEvent_t ev[mczi::N_PHASES + 1] = {};
  cudaEvent_t ev_pre[2] = {};
  int precount = 0;  // pass-1 minimizer table + filter (results identical either way)

  // tuning (0 = per-key-width defaults)
  int count_threads = 0;
  int count_slots = 0;
  int count_ctas_per_sm = 0;
  float count_fill = 0.f;
  int count_chunk = 0;
  int count_filter = -1;
  uint64_t max_bucket_windows = 0;  // 0 = 2^32 - 1 (the 32-bit counters' range); lowered only by a test hook
  int key_passes = 0;  // 0 = chosen from the input size and free HBM  // two-pass bitmap-filtered rounds: -1 auto (when x >= 1), 0 off, 1 on

  mczi::ZiIndex zi;

  // CUDA-graph replay of the counting pipeline (mczi_set_graph_replay)
  bool graph_mode = false;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  mczi::GraphSig graph_sig;
  uint64_t cap_desc = 0, cap_out = 0;  // sizes of the last uncaptured run
  uint32_t cap_slots = 0, cap_fwords = 0, cap_passes = 0;
  uint64_t graph_replays = 0, graph_captures = 0, graph_launches_per_replay = 0;
  cudaEvent_t ev_graph[2] = {};
};

namespace mczi {

int32_t fail(mczi_ctx* c, int32_t code, const std::string& msg);
int32_t cuda_fail(mczi_ctx* c, cudaError_t e, const char* what);

#define CK(call)                                             \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
  } while (0)

#define CKA(buf, bytes)                                                                 \
  do {                                                                                  \
    cudaError_t e_ = (buf).ensure(bytes);                                               \
    if (e_ != cudaSuccess) {                                                            \
      cudaGetLastError();                                                               \
      return fail(ctx, e_ == cudaErrorMemoryAllocation ? MCZI_ERR_OOM : MCZI_ERR_DEVICE, \
                  std::string("device allocation of ") + std::to_string(bytes) +      \
                      " bytes failed: " + cudaGetErrorString(e_));                     \
    }                                                                                   \
  } while (0)

// state of one pass through the pipeline
struct Pipe {
  uint64_t launches = 0;
  uint64_t desc_cap = 0;
  uint64_t n_desc = 0;
  uint64_t n_desc_total = 0;
  uint64_t pwords = 0;
  const uint64_t* d_nbases = nullptr;
  uint64_t n_bases_host = 0;  // after the pack, when the host read it
  float pre_ms = 0.f;
  float ms[mczi::N_PHASES] = {0, 0, 0, 0, 0};  // accumulated over key-range passes
  // graph capture: enqueue only (no host synchronisation, no event records),
  // with the buffer sizes of the preceding uncaptured run
  bool capture = false;
  uint32_t pass = 0;
};



struct InputPlan {
  std::vector<uint64_t> off, len;  // per input: text offset (tile-aligned), bytes (decoded)
  std::vector<uint32_t> tinfo;     // per tile
  std::vector<uint64_t> tile0;     // per input: first tile
  uint64_t text_len = 0, n_tiles = 0, skipped = 0, h2d_bytes = 0;
  // per input: its text on the host (the caller's bytes, or decoded here when
  // compressed and not decoded on the device); null for an input decoded on
  // the device
  std::vector<const uint8_t*> data;
  std::vector<std::vector<uint8_t>> decoded;
  // gzip inputs whose members carry their sizes: decoded on the device into
  // the text (members' out_off relative to their input's text offset)
  std::vector<mczi::GzMember> gz;
  std::vector<uint32_t> gz_inputs;
};
int32_t plan_inputs(mczi_ctx* ctx, const mczi_input* inputs, size_t n, InputPlan& pl);
int32_t stage_layout(mczi_ctx* ctx, const InputPlan& pl, size_t n);
int32_t copy_text_range(mczi_ctx* ctx, const mczi_input* inputs, size_t n, InputPlan& pl, uint64_t b0,
                        uint64_t b1, cudaStream_t s);
int32_t stage_inputs(mczi_ctx* ctx, const mczi_input* inputs, size_t n);
// Streamed staging: the text (laid out by stage_layout) is copied in segments
// on the copy stream while earlier segments are packed and scanned (one
// key-range pass) on the context stream.  Returns with the inputs staged and
// packed and the superkmers in (desc, key), or with *overflow set when they
// did not fit (then pipe_scan redoes the scan).
bool streamed_worthwhile(const mczi_ctx* ctx, const InputPlan& pl);
int32_t stream_pack_scan(mczi_ctx* ctx, const mczi_input* inputs, size_t n, InputPlan& pl, int k, int m,
                         Pipe& p, bool* overflow);
// simplitig.cu: extension table of n sorted distinct keys (lo, hi host arrays)
// into ext_host (n x SIMPLITIG_STRIDE words; see host_io.h)
int32_t simplitig_extensions(mczi_ctx* ctx, const uint64_t* lo, const uint64_t* hi, uint64_t n, int k,
                             uint32_t* ext_host);
int32_t pack_prepare(mczi_ctx* ctx, Pipe& p, mczi::PackArgs& pa);
int32_t pipe_pack(mczi_ctx* ctx, Pipe& p);
int32_t pipe_scan(mczi_ctx* ctx, Pipe& p, int k, int m, uint32_t p1_lo = 0, uint32_t p1_hi = 1u << 12,
                  uint32_t passes = 1);
int32_t pipe_precount(mczi_ctx* ctx, Pipe& p, int mode, uint64_t x);
int32_t pipe_partition(mczi_ctx* ctx, Pipe& p);
// emit_masks: presence mode only; result records then carry one mask word per
// 64 inputs (which inputs contain the k-mer)
// append: keep the records of earlier key-range passes (out_base of them)
int32_t pipe_count(mczi_ctx* ctx, Pipe& p, int k, uint64_t x, int mode, bool emit_masks, uint64_t* n_out,
                   bool append = false);
// number of key-range passes a staged batch needs (descriptor memory, 32-bit counters)
uint32_t key_range_passes(mczi_ctx* ctx, int k, int m, uint64_t bases);
int32_t pipe_finish(mczi_ctx* ctx, Pipe& p, int mode, int k, int m, uint64_t x, uint64_t n_out);

}  // namespace mczi
