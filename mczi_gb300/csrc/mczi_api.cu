// mczi_api.cu -- device-memory management, the MC pipeline stages and the
// MC half of the C ABI declared in include/mczi_gpu.h.
//
// The MC pipeline on one GPU (all intermediate data stays in HBM; the
// reference round-trips it through temporary partition files):
//   stage   : inputs -> HBM, each at a PACK_TILE-aligned offset
//   K0 gz   : (BGZF inputs, copied compressed) members decoded in HBM into
//             their staged places (inflate.cu)
//   K1 pack : bytes -> 2-bit packed stream + fragment-start bits
//   K2 scan : minimizer scan -> superkmer descriptors + partition keys
//   K4 pre  : (optional) pass-1 minimizer table and superkmer filter
//   K3 part : two-digit radix partition of the descriptors
//   K5 count: per-bucket shared-memory counting, threshold, records out
// Entry points mirror MC's library functions (src/lib.rs:278-524).
#include "api_internal.h"
#include "host_io.h"
#include "mczi_common.cuh"
#include "scan.cuh"

#include <algorithm>
#include <thread>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

using namespace mczi;

namespace mczi {

int32_t fail(mczi_ctx* c, int32_t code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int32_t cuda_fail(mczi_ctx* c, cudaError_t e, const char* what) {
  return fail(c, MCZI_ERR_DEVICE, std::string(what) + ": " + cudaGetErrorString(e));
}

namespace {

// reference messages: src/lib.rs:110-152
int32_t validate(mczi_ctx* ctx, const mczi_counter_config* c, int mode) {
  if (!c) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "missing config");
  if (c->k == 0) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "k must be greater than 0");
  if (c->k > 64) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "k must be <= 64 because MC stores k-mers in u128");
  if (c->minimizer == 0) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "minimizer size must be greater than 0");
  if (c->minimizer > c->k) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "minimizer size must be <= k");
  if (c->minimizer > 64)
    return fail(ctx, MCZI_ERR_INVALID_CONFIG, "minimizer size must be <= 64 because MC stores minimizers in u128");
  if (c->partition_count == 0) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "partition count must be greater than 0");
  if (mode == MCZI_MODE_ABUNDANCE) {
    if (c->threshold >= 255)
      return fail(ctx, MCZI_ERR_INVALID_CONFIG,
                  "threshold must be < 255 because compact minimizer counts saturate in u8");
  } else if (mode == MCZI_MODE_PRESENCE) {
    if (c->k > 32) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "FOFN dataset-presence mode currently requires k <= 32");
    if (c->threshold >= 0x7fffffffull)
      return fail(ctx, MCZI_ERR_INVALID_CONFIG, "FOFN dataset-presence threshold must be < 2^31");
  } else {
    return fail(ctx, MCZI_ERR_INVALID_CONFIG, "unknown counting mode");
  }
  return MCZI_OK;
}

// first non-newline byte: '>' FASTA, '@' FASTQ, otherwise not a FASTX record start
int detect_format(const uint8_t* d, uint64_t n) {
  uint64_t i = 0;
  while (i < n && (d[i] == '\n' || d[i] == '\r')) i++;
  if (i >= n) return 2;  // empty: contributes nothing
  if (d[i] == '>') return 0;
  if (d[i] == '@') return 1;
  return -1;
}

}  // namespace

// Host-side layout of a batch of inputs in HBM: each input starts on a
// PACK_TILE boundary, the gaps are '\n'; per tile: input << 2 | fastq << 1 |
// input starts here.  Compressed inputs: a gzip input whose members carry
// their sizes is decoded on the device when the text is copied (its format is
// checked there); other gzip, xz and zstd inputs are decoded here.
int32_t plan_inputs(mczi_ctx* ctx, const mczi_input* inputs, size_t n, InputPlan& pl) {
  if (n == 0) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "at least one input file is required");
  pl.off.assign(n, 0);
  pl.len.assign(n, 0);
  pl.data.assign(n, nullptr);
  pl.decoded.clear();
  pl.decoded.reserve(n);
  pl.gz.clear();
  pl.gz_inputs.clear();
  std::vector<int> fmt(n);
  uint64_t pos = 0;
  pl.skipped = 0;
  pl.h2d_bytes = 0;
  std::vector<GzSpan> spans;
  for (size_t i = 0; i < n; i++) {
    const uint8_t* d = inputs[i].data;
    uint64_t l = d ? inputs[i].len : 0;
    int f = 0;
    const InputFormat cf = input_format(d, l);
    uint64_t total = 0;
    if (cf == InputFormat::Gzip && gzip_sized_members(d, l, &spans, &total)) {
      uint64_t o = 0;
      for (const GzSpan& sp : spans) {
        pl.gz.push_back(GzMember{sp.in_off, o, sp.in_len, sp.out_len, sp.crc, (uint32_t)i});
        o += sp.out_len;
      }
      pl.gz_inputs.push_back((uint32_t)i);
      pl.h2d_bytes += l;  // the compressed bytes cross the host link
      l = total;
    } else {
      if (cf != InputFormat::Plain) {
        std::vector<uint8_t> raw(d, d + l), dec;
        std::string e;
        if (!decompress_buffer(raw, &dec, "input " + std::to_string(i), &e)) return fail(ctx, MCZI_ERR_IO, e);
        pl.decoded.push_back(std::move(dec));
        d = pl.decoded.back().data();
        l = pl.decoded.back().size();
      }
      pl.data[i] = d;
      f = detect_format(d, l);
      if (f < 0) {
        std::fprintf(stderr, "MC_WARN\tskipped_invalid_fastx_input\tinput\t%zu\terror\tInvalid record start\n", i);
        pl.skipped++;
        l = 0;
        f = 0;
      }
      if (f == 2) { l = 0; f = 0; }
      pl.h2d_bytes += l;
    }
    pl.off[i] = pos;
    pl.len[i] = l;
    fmt[i] = f;
    const uint64_t tiles = l == 0 ? 1 : (l + PACK_TILE - 1) / PACK_TILE;  // every input owns >= 1 tile
    pos += tiles * PACK_TILE;
  }
  pl.text_len = pos;
  pl.n_tiles = pos / PACK_TILE;
  pl.tinfo.assign(pl.n_tiles, 0);
  pl.tile0.assign(n, 0);
  for (size_t i = 0; i < n; i++) {
    const uint64_t t0 = pl.off[i] / PACK_TILE;
    const uint64_t t1 = (i + 1 < n ? pl.off[i + 1] : pl.text_len) / PACK_TILE;
    pl.tile0[i] = t0;
    for (uint64_t t = t0; t < t1; t++) pl.tinfo[t] = ((uint32_t)i << 2) | ((uint32_t)fmt[i] << 1) | (t == t0 ? 1u : 0u);
  }
  return MCZI_OK;
}

// Device buffers for a plan, the tile tables copied (their host vectors are
// pageable: the copies are staged before return); the text is not copied.
int32_t stage_layout(mczi_ctx* ctx, const InputPlan& pl, size_t n) {
  ctx->staged = false;
  ctx->have_result = false;
  CKA(ctx->text, pl.text_len);
  CKA(ctx->tile_info, pl.n_tiles * sizeof(uint32_t));
  CKA(ctx->input_tile0, n * sizeof(uint64_t));
  cudaStream_t s = ctx->stream;
  CK(cudaMemcpyAsync(ctx->tile_info.p, pl.tinfo.data(), pl.n_tiles * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(ctx->input_tile0.p, pl.tile0.data(), n * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
  ctx->text_len = pl.text_len;
  ctx->n_tiles = pl.n_tiles;
  ctx->n_inputs = (int)n;
  ctx->skipped = pl.skipped;
  ctx->h2d_bytes = pl.h2d_bytes;
  return MCZI_OK;
}

namespace {

// first non-newline byte of each device-decoded input: 0 '>', 1 '@', 2 none
// (empty), 3 another byte (not a FASTX record start); one CTA per input
__global__ void k_gz_formats(const uint8_t* __restrict__ text, const uint64_t* __restrict__ span, uint32_t n,
                             int32_t* __restrict__ fmt) {
  __shared__ unsigned long long first;
  if (blockIdx.x >= n) return;
  const uint64_t o = span[2 * blockIdx.x], len = span[2 * blockIdx.x + 1];
  if (threadIdx.x == 0) first = ~0ull;
  __syncthreads();
  for (uint64_t i0 = 0; i0 < len; i0 += blockDim.x) {
    const uint64_t i = i0 + threadIdx.x;
    if (i < len && text[o + i] != '\n' && text[o + i] != '\r') atomicMin(&first, (unsigned long long)i);
    __syncthreads();
    if (first != ~0ull) break;  // uniform: read after the barrier
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    int32_t f = 2;
    if (first != ~0ull) {
      const uint8_t c = text[o + first];
      f = c == '>' ? 0 : c == '@' ? 1 : 3;
    }
    fmt[blockIdx.x] = f;
  }
}

// Decodes the plan's device gzip inputs into the text (their bytes cross the
// host link compressed), then checks each one's first record start and fixes
// its tiles' format bits (a FASTQ input) or blanks it (not FASTX: skipped with
// MC's warning, as a plain input would be).
int32_t inflate_inputs(mczi_ctx* ctx, const mczi_input* inputs, InputPlan& pl, cudaStream_t s) {
  const size_t ng = pl.gz_inputs.size();
  std::vector<uint64_t> coff(ng + 1, 0);
  for (size_t j = 0; j < ng; j++) coff[j + 1] = coff[j] + inputs[pl.gz_inputs[j]].len;
  CKA(ctx->gz_comp, coff[ng] + 16);
  uint8_t* comp = ctx->gz_comp.as<uint8_t>();
  std::vector<uint64_t> slot(pl.off.size(), 0);
  for (size_t j = 0; j < ng; j++) {
    const uint32_t i = pl.gz_inputs[j];
    slot[i] = j;
    CK(cudaMemcpyAsync(comp + coff[j], inputs[i].data, inputs[i].len, cudaMemcpyHostToDevice, s));
  }
  std::vector<GzMember> m(pl.gz);
  for (GzMember& g : m) {
    g.in_off += coff[slot[g.input]];
    g.out_off += pl.off[g.input];
  }
  std::vector<uint64_t> span(2 * ng);
  for (size_t j = 0; j < ng; j++) {
    span[2 * j] = pl.off[pl.gz_inputs[j]];
    span[2 * j + 1] = pl.len[pl.gz_inputs[j]];
  }
  CKA(ctx->gz_members, m.size() * sizeof(GzMember) + span.size() * 8 + 16);
  GzMember* dm = ctx->gz_members.as<GzMember>();
  uint64_t* dspan = reinterpret_cast<uint64_t*>(dm + m.size());
  CK(cudaMemcpyAsync(dm, m.data(), m.size() * sizeof(GzMember), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(dspan, span.data(), span.size() * 8, cudaMemcpyHostToDevice, s));
  CKA(ctx->gz_scratch, 64 + 4 * ng);
  uint32_t* scr = ctx->gz_scratch.as<uint32_t>();
  CK(cudaMemsetAsync(scr, 0, 64 + 4 * ng, s));
  CK(cudaEventRecord(ctx->ev[0], s));
  launch_inflate(comp, dm, (uint32_t)m.size(), ctx->text.as<uint8_t>(), scr, scr + 1, ctx->sm_count * 16, s);
  CK(cudaEventRecord(ctx->ev[1], s));
  k_gz_formats<<<(unsigned)ng, 256, 0, s>>>(ctx->text.as<uint8_t>(), dspan, (uint32_t)ng,
                                           reinterpret_cast<int32_t*>(scr + 16));
  CK(cudaGetLastError());
  std::vector<uint32_t> h(16 + ng);
  CK(cudaMemcpyAsync(h.data(), scr, (16 + ng) * 4, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  CK(cudaEventElapsedTime(&ctx->inflate_ms, ctx->ev[0], ctx->ev[1]));
  if (h[1] & ST_GZ_CORRUPT)
    return fail(ctx, MCZI_ERR_IO, "gzip input: a member is not valid DEFLATE data or does not match its size or CRC-32");
  for (size_t j = 0; j < ng; j++) {
    const uint32_t i = pl.gz_inputs[j];
    const int32_t f = (int32_t)h[16 + j];
    const uint64_t t0 = pl.tile0[i], t1 = i + 1 < pl.off.size() ? pl.tile0[i + 1] : pl.n_tiles;
    if (f == 1) {
      for (uint64_t t = t0; t < t1; t++) pl.tinfo[t] |= 2u;
      CK(cudaMemcpyAsync(ctx->tile_info.as<uint32_t>() + t0, pl.tinfo.data() + t0, (t1 - t0) * 4,
                         cudaMemcpyHostToDevice, s));
    } else if (f == 3) {
      std::fprintf(stderr, "MC_WARN\tskipped_invalid_fastx_input\tinput\t%u\terror\tInvalid record start\n", i);
      pl.skipped++;
      ctx->skipped = pl.skipped;
      CK(cudaMemsetAsync(ctx->text.as<uint8_t>() + pl.off[i], '\n', pl.len[i], s));
    }
  }
  CK(cudaStreamSynchronize(s));  // the tile formats were staged from a host vector
  return MCZI_OK;
}

}  // namespace

// Copies the text bytes [b0, b1) of the batch (inputs and their '\n' gaps)
// on stream s; inputs decoded on the device are decoded when the range
// covers the whole text (callers that stage in segments never have them).
int32_t copy_text_range(mczi_ctx* ctx, const mczi_input* inputs, size_t n, InputPlan& pl, uint64_t b0,
                        uint64_t b1, cudaStream_t s) {
  uint8_t* text = ctx->text.as<uint8_t>();
  for (size_t i = 0; i < n; i++) {
    const uint64_t o = pl.off[i], e = pl.off[i] + pl.len[i];
    const uint64_t end = i + 1 < n ? pl.off[i + 1] : pl.text_len;
    if (end <= b0) continue;
    if (o >= b1) break;
    const uint64_t c0 = std::max(o, b0), c1 = std::min(e, b1);
    if (c1 > c0 && pl.data[i]) CK(cudaMemcpyAsync(text + c0, pl.data[i] + (c0 - o), c1 - c0, cudaMemcpyHostToDevice, s));
    const uint64_t g0 = std::max(e, b0), g1 = std::min(end, b1);
    if (g1 > g0) CK(cudaMemsetAsync(text + g0, '\n', g1 - g0, s));
  }
  if (!pl.gz_inputs.empty()) {
    if (b0 != 0 || b1 != pl.text_len) return fail(ctx, MCZI_ERR_STATE, "device-decoded inputs staged in segments");
    return inflate_inputs(ctx, inputs, pl, s);
  }
  return MCZI_OK;
}

int32_t stage_inputs(mczi_ctx* ctx, const mczi_input* inputs, size_t n) {
  ctx->staged = false;
  ctx->have_result = false;
  InputPlan pl;
  int32_t rc = plan_inputs(ctx, inputs, n, pl);
  if (rc) return rc;
  if ((rc = stage_layout(ctx, pl, n))) return rc;
  if ((rc = copy_text_range(ctx, inputs, n, pl, 0, pl.text_len, ctx->stream))) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->staged = true;
  return MCZI_OK;
}


// pack buffers (zeroed streams) and arguments for the staged layout
int32_t pack_prepare(mczi_ctx* ctx, Pipe& p, PackArgs& pa) {
  cudaStream_t s = ctx->stream;
  const uint64_t n_tiles = ctx->n_tiles, text_len = ctx->text_len;
  const int n_in = ctx->n_inputs;
  CKA(ctx->scalars, SC_COUNT * sizeof(uint64_t));
  CK(cudaMemsetAsync(ctx->scalars.p, 0, SC_COUNT * sizeof(uint64_t), s));
  const uint64_t pwords = text_len / 16 + 8, fwords = text_len / 32 + 8;
  const uint64_t ntmp = n_tiles / SCAN_CHUNK + 2;
  CKA(ctx->packed, pwords * 4);
  CKA(ctx->fbits, fwords * 4);
  CKA(ctx->line_sum, (n_tiles + 1) * sizeof(LineSum));
  CKA(ctx->line_pre, (n_tiles + 1) * sizeof(LineSum));
  CKA(ctx->line_tmp, ntmp * sizeof(LineSum));
  CKA(ctx->base_sum, (n_tiles + 1) * sizeof(BaseSum));
  CKA(ctx->base_pre, (n_tiles + 1) * sizeof(BaseSum));
  CKA(ctx->base_tmp, ntmp * sizeof(BaseSum));
  CKA(ctx->input_base, ((size_t)n_in + 1) * sizeof(uint64_t));
  CK(cudaMemsetAsync(ctx->packed.p, 0, pwords * 4, s));
  CK(cudaMemsetAsync(ctx->fbits.p, 0, fwords * 4, s));
  pa = PackArgs{};
  pa.text = ctx->text.as<uint8_t>();
  pa.tile_info = ctx->tile_info.as<uint32_t>();
  pa.input_tile0 = ctx->input_tile0.as<uint64_t>();
  pa.n_tiles = n_tiles;
  pa.line_sum = ctx->line_sum.as<LineSum>();
  pa.line_pre = ctx->line_pre.as<LineSum>();
  pa.line_tmp = ctx->line_tmp.as<LineSum>();
  pa.base_sum = ctx->base_sum.as<BaseSum>();
  pa.base_pre = ctx->base_pre.as<BaseSum>();
  pa.base_tmp = ctx->base_tmp.as<BaseSum>();
  pa.packed = ctx->packed.as<uint32_t>();
  pa.fbits = ctx->fbits.as<uint32_t>();
  pa.input_base = ctx->input_base.as<uint64_t>();
  p.pwords = pwords;
  p.d_nbases = reinterpret_cast<const uint64_t*>(ctx->base_pre.as<BaseSum>() + n_tiles);
  return MCZI_OK;
}

int32_t pipe_pack(mczi_ctx* ctx, Pipe& p) {
  cudaStream_t s = ctx->stream;
  PackArgs pa;
  int32_t rc = pack_prepare(ctx, p, pa);
  if (rc) return rc;
  if (!p.capture) CK(cudaEventRecord(ctx->ev[0], s));
  launch_pack(pa, s);
  p.launches += 9;
  CK(cudaMemcpyAsync(ctx->input_base.as<uint64_t>() + ctx->n_inputs, p.d_nbases, sizeof(uint64_t),
                     cudaMemcpyDeviceToDevice, s));
  CK(cudaGetLastError());
  if (!p.capture) CK(cudaEventRecord(ctx->ev[1], s));
  return MCZI_OK;
}

// Superkmers one pass may hold: the partition addresses them with 32-bit
// positions.
constexpr uint64_t PASS_MAX_DESC = 4000000000ull;  // < 2^32: the partition's 32-bit bucket counters hold a pass
constexpr uint64_t COUNT_SCRATCH_WORDS = 1ull << 19;  // per counting CTA (2 MiB; a multiple of 4)

uint32_t key_range_passes(mczi_ctx* ctx, int k, int m, uint64_t bases) {
  if (ctx->key_passes > 0) return (uint32_t)ctx->key_passes;
  const int w = k - m + 1;
  // expected superkmers: 2 / (w + 1) per base of a random sequence; before the
  // pack only the text length is known (headers and line breaks included)
  const double est = (double)(bases ? bases : ctx->text_len) * 2.0 / (double)(w + 1);
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) { cudaGetLastError(); free_b = 8ull << 30; }
  // descriptors (12 B) + their pass-1 copy (8 B) + precount/partition slack
  const double per_pass = std::min((double)PASS_MAX_DESC, (double)free_b * 0.45 / 24.0);
  uint32_t r = (uint32_t)std::ceil(est * (bases ? 1.1 : 1.3) / per_pass);
  return std::max(1u, std::min(r, 64u));
}

int32_t pipe_scan(mczi_ctx* ctx, Pipe& p, int k, int m, uint32_t p1_lo, uint32_t p1_hi, uint32_t passes) {
  cudaStream_t s = ctx->stream;
  uint64_t* sc = ctx->scalars.as<uint64_t>();
  const uint64_t text_len = ctx->text_len;
  const uint64_t bases = p.n_bases_host ? p.n_bases_host : text_len;
  const int w = k - m + 1;
  uint64_t desc_cap = bases * 3 / (uint64_t)(w + 1) / passes + (1u << 20);
  if (desc_cap > bases + 1024) desc_cap = bases + 1024;
  if (desc_cap > PASS_MAX_DESC) desc_cap = PASS_MAX_DESC;
  if (p.capture) desc_cap = ctx->cap_desc;
  for (int attempt = 0; attempt < 3; attempt++) {
    if (desc_cap > PASS_MAX_DESC) return fail(ctx, MCZI_ERR_TOO_LARGE, "more superkmers than one key-range pass holds");
    CKA(ctx->desc, desc_cap * 8);
    CKA(ctx->key, desc_cap * 4);
    CK(cudaMemsetAsync(sc + SC_NDESC, 0, 8, s));
    if (!p.capture) CK(cudaMemsetAsync(sc + SC_STATUS, 0, 8, s));
    ScanArgs sa{};
    sa.packed = ctx->packed.as<uint32_t>();
    sa.fbits = ctx->fbits.as<uint32_t>();
    sa.n_bases = p.d_nbases;
    sa.max_bases = text_len;
    sa.packed_words = p.pwords;
    sa.k = k;
    sa.m = m;
    sa.desc = ctx->desc.as<uint64_t>();
    sa.key = ctx->key.as<uint32_t>();
    sa.n_desc = reinterpret_cast<unsigned long long*>(sc + SC_NDESC);
    sa.desc_cap = desc_cap;
    sa.status = reinterpret_cast<uint32_t*>(sc + (p.capture ? SC_SCANST : SC_STATUS));
    sa.p1_lo = p1_lo;
    sa.p1_hi = p1_hi;
    launch_scan(sa, s);
    p.launches += 1;
    CK(cudaGetLastError());
    if (p.capture) {  // sizes come from the uncaptured run; overflow is checked after replay
      p.n_desc = desc_cap;
      p.desc_cap = desc_cap;
      return MCZI_OK;
    }
    uint64_t h[2];
    CK(cudaMemcpyAsync(h, sc + SC_NDESC, 8, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(h + 1, sc + SC_STATUS, 8, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (h[1] & ST_SPIN_TIMEOUT) return fail(ctx, MCZI_ERR_DEVICE, "a scan tile's staging copy did not complete");
    if (!(h[1] & ST_DESC_OVERFLOW)) {
      p.n_desc = h[0];
      p.desc_cap = desc_cap;
      ctx->cap_desc = std::max(ctx->cap_desc, desc_cap);
      return MCZI_OK;
    }
    desc_cap = h[0] + 1024;
  }
  return fail(ctx, MCZI_ERR_DEVICE, "descriptor buffer overflow persisted");
}

int32_t pipe_precount(mczi_ctx* ctx, Pipe& p, int mode, uint64_t x) {
  if (p.n_desc == 0) return MCZI_OK;
  cudaStream_t s = ctx->stream;
  uint64_t* sc = ctx->scalars.as<uint64_t>();
  uint64_t slots = 1024;
  while (slots < 2 * p.n_desc) slots <<= 1;
  CKA(ctx->mintab, slots * 8);
  CKA(ctx->desc2, p.desc_cap * 8);
  CKA(ctx->key2, p.desc_cap * 4);
  CK(cudaMemsetAsync(ctx->mintab.p, 0, slots * 8, s));
  if (mode == MCZI_MODE_PRESENCE) {
    CKA(ctx->pairtab, slots * 8);
    CK(cudaMemsetAsync(ctx->pairtab.p, 0, slots * 8, s));
  }
  CK(cudaMemsetAsync(sc + SC_NKEPT, 0, 8, s));
  CK(cudaEventRecord(ctx->ev_pre[0], s));
  PrecountArgs pc;
  pc.desc = ctx->desc.as<uint64_t>();
  pc.key = ctx->key.as<uint32_t>();
  pc.n_desc = reinterpret_cast<const unsigned long long*>(sc + SC_NDESC);
  pc.table = ctx->mintab.as<unsigned long long>();
  pc.mask = slots - 1;
  pc.pairs = mode == MCZI_MODE_PRESENCE ? ctx->pairtab.as<unsigned long long>() : nullptr;
  pc.pair_mask = slots - 1;
  pc.mode = mode;
  pc.dataset_base = ctx->input_base.as<uint64_t>();
  pc.n_datasets = ctx->n_inputs;
  pc.threshold = x;
  pc.desc_out = ctx->desc2.as<uint64_t>();
  pc.key_out = ctx->key2.as<uint32_t>();
  pc.n_kept = reinterpret_cast<unsigned long long*>(sc + SC_NKEPT);
  pc.status = reinterpret_cast<uint32_t*>(sc + SC_STATUS);
  launch_precount(pc, ctx->sm_count, s);
  p.launches += 2;
  CK(cudaGetLastError());
  CK(cudaEventRecord(ctx->ev_pre[1], s));
  uint64_t h[2];
  CK(cudaMemcpyAsync(h, sc + SC_NKEPT, 8, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(h + 1, sc + SC_STATUS, 8, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (h[1] & ST_MINTAB_FULL) return fail(ctx, MCZI_ERR_DEVICE, "minimizer table full");
  std::swap(ctx->desc, ctx->desc2);
  std::swap(ctx->key, ctx->key2);
  p.n_desc = h[0];
  CK(cudaMemcpyAsync(sc + SC_NDESC, &p.n_desc, 8, cudaMemcpyHostToDevice, s));
  CK(cudaStreamSynchronize(s));
  CK(cudaEventElapsedTime(&p.pre_ms, ctx->ev_pre[0], ctx->ev_pre[1]));
  return MCZI_OK;
}

int32_t pipe_partition(mczi_ctx* ctx, Pipe& p) {
  cudaStream_t s = ctx->stream;
  uint64_t* sc = ctx->scalars.as<uint64_t>();
  if (!p.capture) CK(cudaEventRecord(ctx->ev[2], s));
  CKA(ctx->desc2, p.desc_cap * 8);
  CKA(ctx->key2, p.desc_cap * 4);
  CKA(ctx->part_hist, (2 * NP1 + 128) * sizeof(uint32_t));  // histogram + the two levels' cursors
  CKA(ctx->bucket_off, (NP1 + 1) * sizeof(uint64_t));
  PartArgs qa;
  qa.desc_in = ctx->desc.as<uint64_t>();
  qa.key_in = ctx->key.as<uint32_t>();
  qa.desc_out = ctx->desc2.as<uint64_t>();
  qa.key_out = ctx->key2.as<uint32_t>();
  qa.n_desc = reinterpret_cast<const unsigned long long*>(sc + SC_NDESC);
  qa.desc_cap = p.desc_cap;
  qa.hist = ctx->part_hist.as<uint32_t>();
  qa.bucket_off = ctx->bucket_off.as<uint64_t>();
  qa.status = reinterpret_cast<uint32_t*>(sc + SC_STATUS);
  if (p.n_desc > 0) {
    // two tile-sorted levels: desc -> (desc2, key2 as u16 p1) -> desc, which
    // the counting kernel then reads as buckets unsorted by p2
    launch_partition_tiled(qa, qa.hist, reinterpret_cast<uint16_t*>(ctx->key2.p), ctx->desc.as<uint64_t>(), s);
    p.launches += 5;
  }
  CK(cudaGetLastError());
  if (!p.capture) CK(cudaEventRecord(ctx->ev[3], s));
  return MCZI_OK;
}

int32_t pipe_count(mczi_ctx* ctx, Pipe& p, int k, uint64_t x, int mode, bool emit_masks, uint64_t* n_out_ret,
                   bool append) {
  cudaStream_t s = ctx->stream;
  uint64_t* sc = ctx->scalars.as<uint64_t>();
  const bool wide = k > 32;
  const int n_in = ctx->n_inputs;
  const int W = (n_in + 63) / 64;
  const uint64_t est_out = ctx->text_len / (x + 1) + 1024;
  const uint64_t prior = append ? *n_out_ret : 0;  // records of earlier key-range passes
  uint64_t out_cap = std::max<uint64_t>(std::min<uint64_t>(est_out, 1ull << 25), prior + (1u << 20));
  if (append && ctx->out_lo.cap / 8 > out_cap) out_cap = ctx->out_lo.cap / 8;
  if (p.capture) out_cap = ctx->cap_out;
  uint64_t n_out = prior;
#define CKG(buf, bytes, keep)                                                            \
  do {                                                                                   \
    cudaError_t e_ = (buf).grow_keep((bytes), (keep), s);                                \
    if (e_ != cudaSuccess) {                                                             \
      cudaGetLastError();                                                                \
      return fail(ctx, e_ == cudaErrorMemoryAllocation ? MCZI_ERR_OOM : MCZI_ERR_DEVICE, \
                  std::string("device allocation failed: ") + cudaGetErrorString(e_));  \
    }                                                                                    \
  } while (0)
  if (p.n_desc > 0) {
    // defaults: two CTAs of 512 threads per SM (measured on GB300 on the 4 Gbp
    // k = 63 workload: 46.9 ms against 48.6 ms for one CTA of 1024 threads)
    int threads = ctx->count_threads > 0 ? ctx->count_threads : 512;
    int cps = ctx->count_ctas_per_sm > 0 ? ctx->count_ctas_per_sm : 2;
    const size_t budget = ctx->smem_optin;  // per block, opt-in
    const size_t fixed = count_fixed_smem_bytes(mode, n_in);
    const size_t slotb = count_slot_bytes(k, mode, n_in);
    // shared memory per SM is 228 KiB with 1 KiB per CTA reserved; the
    // kernel's static shared memory counts against the same budget
    const size_t stat = count_static_smem(k, mode);
    size_t per_cta = std::min(budget, (size_t)(228 * 1024) / (size_t)cps - 1024) - stat - 64;
    // two-pass (bitmap-filtered) rounds store only repeated k-mers; they need
    // x >= 1 and leave part of shared memory to the bitmap
    // auto: long k-mers (k > 32) are mostly singletons in sequencing data, so
    // storing only repeats pays; short ones mostly repeat (measured on GB300)
    const bool filt = x >= 1 && (ctx->count_filter > 0 || (ctx->count_filter < 0 && wide));
    const size_t avail = per_cta - fixed - 128;
    uint32_t slots, fwords = 0;
    if (filt) {
      const double share = wide ? 0.6 : 0.5;
      slots = ctx->count_slots > 0 ? (uint32_t)ctx->count_slots : (uint32_t)(avail * share / slotb);
      const size_t used = ((size_t)slots * slotb + 64);
      fwords = used < avail ? (uint32_t)((avail - used) / 4) & ~31u : 0u;
      if (fwords < 1024) fwords = 0;  // too small to help: single pass
    } else {
      slots = ctx->count_slots > 0 ? (uint32_t)ctx->count_slots : (uint32_t)(avail / slotb);
    }
    if (slots < (uint32_t)threads) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "counting table smaller than the CTA");
    if (count_smem_bytes(k, mode, n_in, slots, fwords) > budget)
      return fail(ctx, MCZI_ERR_INVALID_CONFIG, "counting table does not fit in shared memory");
    for (int attempt = 0; attempt < 3; attempt++) {
      // grow the result buffers keeping earlier passes' records
      CKG(ctx->out_lo, out_cap * 8, prior * 8);
      if (wide) CKG(ctx->out_hi, out_cap * 8, prior * 8);
      CKG(ctx->out_cnt, out_cap * 4, prior * 4);
      if (emit_masks) CKG(ctx->out_mask, out_cap * 8 * (uint64_t)W, prior * 8 * (uint64_t)W);
      if (p.capture) {
        // the record counter runs on across passes; statuses accumulate
        if (p.pass == 0) CK(cudaMemsetAsync(sc + SC_NOUT, 0, 8, s));
      } else {
        CK(cudaMemcpyAsync(sc + SC_NOUT, &prior, 8, cudaMemcpyHostToDevice, s));
        CK(cudaMemsetAsync(sc + SC_STATUS, 0, 8, s));
      }
      CK(cudaMemsetAsync(sc + SC_STATS, 0, 8 * 8, s));
      CK(cudaMemsetAsync(sc + SC_WORK, 0, 8, s));
      CountArgs ca;
      ca.packed = ctx->packed.as<uint32_t>();
      // the partition leaves the buckets (unsorted by p2) in desc; the
      // counting kernel sorts each into desc2 and counts from there
      ca.desc = ctx->desc2.as<uint64_t>();
      ca.desc_unsorted = ctx->desc.as<uint64_t>();
      ca.key = ctx->key.as<uint32_t>();
      ca.bucket_off = ctx->bucket_off.as<uint64_t>();
      ca.k = k;
      ca.threshold = x;
      ca.mode = mode;
      ca.dataset_base = ctx->input_base.as<uint64_t>();
      ca.n_datasets = n_in;
      ca.out_lo = ctx->out_lo.as<uint64_t>();
      ca.out_hi = wide ? ctx->out_hi.as<uint64_t>() : nullptr;
      ca.out_count = ctx->out_cnt.as<uint32_t>();
      ca.out_mask = emit_masks ? ctx->out_mask.as<unsigned long long>() : nullptr;
      ca.n_out = reinterpret_cast<unsigned long long*>(sc + SC_NOUT);
      ca.out_cap = out_cap;
      ca.stats = reinterpret_cast<unsigned long long*>(sc + SC_STATS);
      ca.status = reinterpret_cast<uint32_t*>(sc + SC_STATUS);
      ca.table_slots = slots;
      ca.threads = threads;
      ca.ctas = ctx->sm_count * cps;
      ca.work_counter = reinterpret_cast<unsigned int*>(sc + SC_WORK);
      // default target fill: filtered rounds (k > 32, x >= 1) measured faster
      // at 0.8 (fewer, larger rounds), single-pass rounds keep 0.6
      ca.fill = ctx->count_fill > 0.f ? ctx->count_fill : (fwords > 0 ? 0.8f : 0.6f);
      // default: the fast rounds' chunk for filtered k > 32 counts, else 4
      // (k > 32) or 2 windows per work item
      ca.chunk = ctx->count_chunk > 0 ? (uint32_t)ctx->count_chunk
                                      : (wide ? (fwords > 0 ? COUNT_FAST_CHUNK : 4u) : 2u);
      ca.filter_words = fwords;
      ca.max_bucket_windows = ctx->max_bucket_windows ? ctx->max_bucket_windows : 0xffffffffull;
      // filtered rounds whose windows fit COUNT_SCRATCH_WORDS per CTA take the
      // fast path (pass 2 reads one word per window instead of re-rolling)
      ca.win_scratch = nullptr;
      ca.scratch_words = 0;
      if (fwords > 0) {
        CKA(ctx->count_scratch, (size_t)ca.ctas * COUNT_SCRATCH_WORDS * 4);
        ca.win_scratch = ctx->count_scratch.as<uint32_t>();
        ca.scratch_words = COUNT_SCRATCH_WORDS;
      }
      launch_count(ca, s);
      p.launches += 1;
      CK(cudaGetLastError());
      if (p.capture) break;
      ctx->cap_slots = slots;
      ctx->cap_fwords = fwords;
      uint64_t h[SC_COUNT];
      CK(cudaMemcpyAsync(h, sc, sizeof h, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      const uint32_t st = (uint32_t)h[SC_STATUS];
      if (st & ST_TABLE_STUCK) return fail(ctx, MCZI_ERR_DEVICE, "counting round could not be split further");
      if (st & ST_COUNT_WIDTH)
        return fail(ctx, MCZI_ERR_TOO_LARGE,
                    "a minimizer bucket holds more than " +
                        std::to_string(ca.max_bucket_windows) +
                        " k-mer windows, beyond the counting kernel's 32-bit counters");
      if (st & ST_OUT_OVERFLOW) {
        out_cap = h[SC_NOUT] + (1u << 20);
        continue;
      }
      n_out = h[SC_NOUT];
      ctx->cap_out = std::max(ctx->cap_out, out_cap);
      ctx->stats[2] += h[SC_STATS + 2];
      ctx->stats[3] += h[SC_STATS + 3];
      ctx->stats[4] += h[SC_STATS + 1];
      ctx->stats[6] += h[SC_STATS + 0];
      break;
    }
  }
  if (!p.capture) CK(cudaEventRecord(ctx->ev[4], s));
  ctx->mask_words = emit_masks ? W : 0;
  *n_out_ret = n_out;
  return MCZI_OK;
}

int32_t pipe_finish(mczi_ctx* ctx, Pipe& p, int mode, int k, int m, uint64_t x, uint64_t n_out) {
  cudaStream_t s = ctx->stream;
  CK(cudaEventRecord(ctx->ev[5], s));
  CK(cudaStreamSynchronize(s));
  for (int i = 0; i < 4; i++) {
    float t = 0.f;
    CK(cudaEventElapsedTime(&t, ctx->ev[i], ctx->ev[i + 1]));
    p.ms[i] += t;
  }
  p.ms[1] -= p.pre_ms;  // the scan phase window also spans the pre-count
  p.ms[4] += p.pre_ms;
  for (int i = 0; i < N_PHASES; i++) ctx->phase_ms[i] = p.ms[i];
  uint64_t nb = 0;
  CK(cudaMemcpy(&nb, p.d_nbases, 8, cudaMemcpyDeviceToHost));
  ctx->stats[0] = nb;
  ctx->stats[1] = p.n_desc_total;  // superkmers counted (after the pre-count filter, when on)
  ctx->stats[5] = n_out;
  ctx->stats[7] = ctx->skipped;
  ctx->stats[8] = p.launches;
  ctx->stats[9] = ctx->h2d_bytes;
  ctx->mode = mode;
  ctx->k = k;
  ctx->m = m;
  ctx->x = x;
  ctx->n_out = n_out;
  ctx->have_result = true;
  return MCZI_OK;
}

namespace {

int32_t run_count(mczi_ctx* ctx, const mczi_counter_config* cfg, int mode, uint64_t* n_records) {
  int32_t rc = validate(ctx, cfg, mode);
  if (rc) return rc;
  if (!ctx->staged) return fail(ctx, MCZI_ERR_STATE, "no staged inputs");
  ctx->have_result = false;
  ctx->mask_words = 0;
  const int k = (int)cfg->k, m = (int)cfg->minimizer;
  for (int i = 0; i < N_PHASES; i++) ctx->phase_ms[i] = 0.f;
  // fof: the reference returns an empty result when x >= #datasets (src/lib.rs:644-648)
  if (mode == MCZI_MODE_PRESENCE && cfg->threshold >= (uint64_t)ctx->n_inputs) {
    ctx->mode = mode; ctx->k = k; ctx->m = m; ctx->x = cfg->threshold;
    ctx->n_out = 0;
    std::memset(ctx->stats, 0, sizeof ctx->stats);
    ctx->stats[9] = ctx->h2d_bytes;
    ctx->have_result = true;
    if (n_records) *n_records = 0;
    return MCZI_OK;
  }
  Pipe p;
  std::memset(ctx->stats, 0, sizeof ctx->stats);
  if ((rc = pipe_pack(ctx, p))) return rc;
  // inputs with more superkmers than one pass can hold are counted in passes
  // over disjoint ranges of the partition key (disjoint sets of k-mers),
  // decided from the packed base count; a pass that still overflows doubles
  // the number of passes
  CK(cudaMemcpyAsync(&p.n_bases_host, p.d_nbases, 8, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  uint32_t passes = key_range_passes(ctx, k, m, p.n_bases_host);
  uint64_t n_out = 0;
  for (uint32_t r = 0; r < passes; r++) {
    const uint32_t lo = (uint32_t)((uint64_t)NP1 * r / passes), hi = (uint32_t)((uint64_t)NP1 * (r + 1) / passes);
    if (r > 0) {
      // time each pass's phases; the pack ran once
      for (int i = 0; i < 4; i++) {
        float t = 0.f;
        CK(cudaEventSynchronize(ctx->ev[i + 1]));
        CK(cudaEventElapsedTime(&t, ctx->ev[i], ctx->ev[i + 1]));
        p.ms[i] += t;
      }
      p.ms[1] -= p.pre_ms;
      p.ms[4] += p.pre_ms;
      p.pre_ms = 0.f;
      // later passes have no pack: their pack window is empty
      CK(cudaEventRecord(ctx->ev[0], ctx->stream));
      CK(cudaEventRecord(ctx->ev[1], ctx->stream));
    }
    if ((rc = pipe_scan(ctx, p, k, m, lo, hi, passes))) {
      if (rc != MCZI_ERR_TOO_LARGE || passes >= 64 || ctx->key_passes > 0) return rc;
      passes = std::min(64u, passes * 2);  // start over with narrower key ranges
      r = (uint32_t)-1;
      n_out = 0;
      p.n_desc_total = 0;
      p.pre_ms = 0.f;
      for (int i = 0; i < N_PHASES; i++) p.ms[i] = 0.f;
      CK(cudaEventRecord(ctx->ev[0], ctx->stream));
      CK(cudaEventRecord(ctx->ev[1], ctx->stream));
      continue;
    }
    if (ctx->precount && (rc = pipe_precount(ctx, p, mode, cfg->threshold))) return rc;
    if ((rc = pipe_partition(ctx, p))) return rc;
    if ((rc = pipe_count(ctx, p, k, cfg->threshold, mode, false, &n_out, r > 0))) return rc;
    p.n_desc_total += p.n_desc;
  }
  if ((rc = pipe_finish(ctx, p, mode, k, m, cfg->threshold, n_out))) return rc;
  if (n_records) *n_records = n_out;
  return MCZI_OK;
}


// One-shot count with the staging overlapped: the text is copied in segments
// on the copy stream; each segment is packed as soon as it has arrived (the
// pack's prefix scans continue from the previous segment's totals) and the
// base tiles whose packed words are complete are scanned right after.  The
// rest of the pipeline is run_count's.  Inputs that need several key-range
// passes, the minimizer pre-count or no device work at all take the plain
// path (stage, then count).
}  // namespace

// segments of >= 32 MiB of text (4096 pack tiles) unless set
static uint64_t stream_seg_min(const mczi_ctx* ctx) { return ctx->stream_seg_tiles > 0 ? ctx->stream_seg_tiles : 4096; }

bool streamed_worthwhile(const mczi_ctx* ctx, const InputPlan& pl) {
  // inputs decoded on the device are staged whole (their decoded bytes
  // appear in no host buffer to copy in segments)
  return ctx->streamed && pl.gz_inputs.empty() && pl.n_tiles >= 2 * stream_seg_min(ctx);
}

int32_t stream_pack_scan(mczi_ctx* ctx, const mczi_input* inputs, size_t n, InputPlan& pl, int k, int m,
                         Pipe& p, bool* overflow) {
  int32_t rc;
  *overflow = false;
  cudaStream_t s = ctx->stream, cs = ctx->copy_stream;
  PackArgs pa;
  if ((rc = pack_prepare(ctx, p, pa))) return rc;
  // scan buffers, as pipe_scan sizes them
  uint64_t* sc = ctx->scalars.as<uint64_t>();
  const int w = k - m + 1;
  uint64_t desc_cap = pl.text_len * 3 / (uint64_t)(w + 1) + (1u << 20);
  if (desc_cap > pl.text_len + 1024) desc_cap = pl.text_len + 1024;
  if (desc_cap > PASS_MAX_DESC) desc_cap = PASS_MAX_DESC;
  CKA(ctx->desc, desc_cap * 8);
  CKA(ctx->key, desc_cap * 4);
  CK(cudaMemsetAsync(sc + SC_NDESC, 0, 8, s));
  CK(cudaMemsetAsync(sc + SC_STATUS, 0, 8, s));
  CKA(ctx->stream_scratch, 256);
  uint8_t* scr = ctx->stream_scratch.as<uint8_t>();
  LineSum* carry_line = reinterpret_cast<LineSum*>(scr);
  BaseSum* carry_base = reinterpret_cast<BaseSum*>(scr + 64);
  uint64_t* range = reinterpret_cast<uint64_t*>(scr + 128);
  CK(cudaMemsetAsync(range, 0, 16, s));
  ScanArgs sa{};
  sa.packed = ctx->packed.as<uint32_t>();
  sa.fbits = ctx->fbits.as<uint32_t>();
  sa.max_bases = pl.text_len;
  sa.packed_words = p.pwords;
  sa.k = k;
  sa.m = m;
  sa.desc = ctx->desc.as<uint64_t>();
  sa.key = ctx->key.as<uint32_t>();
  sa.n_desc = reinterpret_cast<unsigned long long*>(sc + SC_NDESC);
  sa.desc_cap = desc_cap;
  sa.status = reinterpret_cast<uint32_t*>(sc + SC_STATUS);
  sa.p1_lo = 0;
  sa.p1_hi = NP1;
  sa.tile_range = range;
  // the copy stream starts after this stream's buffer set-up (the memsets of
  // the packed streams and the tile tables)
  CK(cudaEventRecord(ctx->ev_copy, s));
  CK(cudaStreamWaitEvent(cs, ctx->ev_copy, 0));
  CK(cudaEventRecord(ctx->ev[0], s));
  const uint64_t nseg_target = 16;
  const uint64_t seg = ctx->stream_seg_tiles > 0
                           ? ctx->stream_seg_tiles
                           : std::max<uint64_t>(stream_seg_min(ctx), (pl.n_tiles + nseg_target - 1) / nseg_target);
  for (uint64_t t0 = 0; t0 < pl.n_tiles; t0 += seg) {
    const uint64_t t1 = std::min(pl.n_tiles, t0 + seg);
    const bool last = t1 == pl.n_tiles;
    if ((rc = copy_text_range(ctx, inputs, n, pl, t0 * PACK_TILE, t1 * PACK_TILE, cs))) return rc;
    CK(cudaEventRecord(ctx->ev_copy, cs));
    CK(cudaStreamWaitEvent(s, ctx->ev_copy, 0));
    launch_pack_segment(pa, t0, t1, carry_line, carry_base, s);
    p.launches += t0 > 0 ? 11 : 9;
    // bases packed so far (the running total at the next segment's first tile)
    const uint64_t* avail = reinterpret_cast<const uint64_t*>(pa.base_pre + t1);
    sa.n_bases = avail;
    const uint64_t max_tiles = (t1 - t0) * (PACK_TILE / SCAN_TILE) + 4;  // new bases <= new text bytes
    launch_scan_window(avail, range, last, max_tiles, sa.status, s);
    launch_scan_range(sa, max_tiles, s);
    p.launches += 2;
    CK(cudaGetLastError());
  }
  CK(cudaMemcpyAsync(ctx->input_base.as<uint64_t>() + n, p.d_nbases, sizeof(uint64_t), cudaMemcpyDeviceToDevice, s));
  CK(cudaEventRecord(ctx->ev[1], s));
  ctx->staged = true;
  uint64_t h[2];
  CK(cudaMemcpyAsync(h, sc + SC_NDESC, 8, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(h + 1, sc + SC_STATUS, 8, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (h[1] & ST_SPIN_TIMEOUT) return fail(ctx, MCZI_ERR_DEVICE, "a scan tile's staging copy did not complete");
  if (h[1] & ST_DESC_OVERFLOW) {
    *overflow = true;
    return MCZI_OK;
  }
  p.n_desc = h[0];
  p.desc_cap = desc_cap;
  ctx->cap_desc = std::max(ctx->cap_desc, desc_cap);
  return MCZI_OK;
}

namespace {

int32_t run_count_streamed(mczi_ctx* ctx, const mczi_counter_config* cfg, int mode, const mczi_input* inputs,
                           size_t n, uint64_t* n_records) {
  int32_t rc;
  InputPlan pl;
  if ((rc = plan_inputs(ctx, inputs, n, pl))) return rc;
  if ((rc = stage_layout(ctx, pl, n))) return rc;
  ctx->mask_words = 0;
  const int k = (int)cfg->k, m = (int)cfg->minimizer;
  const uint32_t passes = key_range_passes(ctx, k, m, 0);
  // the text-length estimate over-counts bases (headers, line breaks): up to
  // two estimated passes are tried as one, with the plain path as fallback
  const bool plain = passes > 2 || ctx->precount || !streamed_worthwhile(ctx, pl) ||
                     (mode == MCZI_MODE_PRESENCE && cfg->threshold >= (uint64_t)n);
  if (plain) {
    if ((rc = copy_text_range(ctx, inputs, n, pl, 0, pl.text_len, ctx->stream))) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->staged = true;
    return run_count(ctx, cfg, mode, n_records);
  }
  for (int i = 0; i < N_PHASES; i++) ctx->phase_ms[i] = 0.f;
  Pipe p;
  std::memset(ctx->stats, 0, sizeof ctx->stats);
  bool overflow = false;
  if ((rc = stream_pack_scan(ctx, inputs, n, pl, k, m, p, &overflow))) return rc;
  // more superkmers than the streamed pass holds: the inputs are staged, so
  // the plain path (which sizes its passes from the packed bases) redoes it
  if (overflow) return run_count(ctx, cfg, mode, n_records);
  uint64_t n_out = 0;
  if ((rc = pipe_partition(ctx, p))) return rc;
  if ((rc = pipe_count(ctx, p, k, cfg->threshold, mode, false, &n_out, false))) return rc;
  p.n_desc_total += p.n_desc;
  if ((rc = pipe_finish(ctx, p, mode, k, m, cfg->threshold, n_out))) return rc;
  if (n_records) *n_records = n_out;
  return MCZI_OK;
}

GraphSig make_sig(mczi_ctx* ctx, const mczi_counter_config* cfg, int mode, uint32_t passes) {
  GraphSig g;
  g.text_len = ctx->text_len;
  g.n_tiles = ctx->n_tiles;
  g.x = cfg->threshold;
  g.desc_cap = ctx->cap_desc;
  g.out_cap = ctx->cap_out;
  g.n_inputs = ctx->n_inputs;
  g.k = (int)cfg->k;
  g.m = (int)cfg->minimizer;
  g.mode = mode;
  g.passes = passes;
  g.slots = ctx->cap_slots;
  g.fwords = ctx->cap_fwords;
  g.threads = ctx->count_threads;
  g.cps = ctx->count_ctas_per_sm;
  g.chunk = ctx->count_chunk;
  g.filter = ctx->count_filter;
  g.fill = ctx->count_fill;
  const void* ptrs[13] = {ctx->text.p, ctx->packed.p, ctx->fbits.p, ctx->desc.p, ctx->key.p, ctx->desc2.p,
                          ctx->key2.p, ctx->out_lo.p, ctx->out_hi.p, ctx->out_cnt.p, ctx->scalars.p,
                          ctx->part_hist.p, ctx->count_scratch.p};
  for (int i = 0; i < 13; i++) g.ptrs[i] = ptrs[i];
  return g;
}

void drop_graph(mczi_ctx* ctx) {
  if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
  if (ctx->graph) cudaGraphDestroy(ctx->graph);
  ctx->graph_exec = nullptr;
  ctx->graph = nullptr;
}

// Enqueues the whole counting pipeline on the capturing stream: no host
// synchronisation, the buffer sizes of the uncaptured run just before.
int32_t capture_pipeline(mczi_ctx* ctx, const mczi_counter_config* cfg, int mode, uint32_t passes) {
  cudaStream_t s = ctx->stream;
  drop_graph(ctx);
  if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return MCZI_OK;  // no graph: the plain path keeps working
  }
  const int k = (int)cfg->k, m = (int)cfg->minimizer;
  Pipe p;
  p.capture = true;
  int32_t rc = MCZI_OK;
  uint64_t n_out = 0;
  uint64_t* sc = ctx->scalars.as<uint64_t>();
  cudaMemsetAsync(sc + SC_STATUS, 0, 8, s);
  cudaMemsetAsync(sc + SC_SCANST, 0, 8, s);
  rc = pipe_pack(ctx, p);
  for (uint32_t r = 0; r < passes && rc == MCZI_OK; r++) {
    p.pass = r;
    const uint32_t lo = (uint32_t)((uint64_t)NP1 * r / passes), hi = (uint32_t)((uint64_t)NP1 * (r + 1) / passes);
    if ((rc = pipe_scan(ctx, p, k, m, lo, hi, passes))) break;
    if ((rc = pipe_partition(ctx, p))) break;
    rc = pipe_count(ctx, p, k, cfg->threshold, mode, false, &n_out, r > 0);
  }
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(s, &g);
  if (rc != MCZI_OK || e != cudaSuccess || !g) {
    cudaGetLastError();
    if (g) cudaGraphDestroy(g);
    return MCZI_OK;
  }
  cudaGraphExec_t ex = nullptr;
  if (cudaGraphInstantiate(&ex, g, 0) != cudaSuccess) {
    cudaGetLastError();
    cudaGraphDestroy(g);
    return MCZI_OK;
  }
  ctx->graph = g;
  ctx->graph_exec = ex;
  ctx->graph_sig = make_sig(ctx, cfg, mode, passes);
  ctx->graph_captures++;
  ctx->graph_launches_per_replay = p.launches;
  return MCZI_OK;
}

// Replays the captured pipeline when it matches the staged inputs and the
// configuration; otherwise runs the plain path and captures it for next time.
int32_t run_count_graph(mczi_ctx* ctx, const mczi_counter_config* cfg, int mode, uint64_t* n_records) {
  int32_t rc = validate(ctx, cfg, mode);
  if (rc) return rc;
  if (!ctx->staged) return fail(ctx, MCZI_ERR_STATE, "no staged inputs");
  if (ctx->precount || (mode == MCZI_MODE_PRESENCE && cfg->threshold >= (uint64_t)ctx->n_inputs))
    return run_count(ctx, cfg, mode, n_records);
  const uint32_t passes = key_range_passes(ctx, (int)cfg->k, (int)cfg->minimizer, 0);
  if (ctx->graph_exec && make_sig(ctx, cfg, mode, passes) == ctx->graph_sig) {
    cudaStream_t s = ctx->stream;
    CK(cudaEventRecord(ctx->ev_graph[0], s));
    CK(cudaGraphLaunch(ctx->graph_exec, s));
    CK(cudaEventRecord(ctx->ev_graph[1], s));
    uint64_t h[SC_COUNT];
    CK(cudaMemcpyAsync(h, ctx->scalars.p, sizeof h, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    const uint32_t st = (uint32_t)(h[SC_STATUS] | h[SC_SCANST]);
    if (st & ST_SPIN_TIMEOUT) return fail(ctx, MCZI_ERR_DEVICE, "a scan tile's staging copy did not complete");
    if (st & (ST_DESC_OVERFLOW | ST_OUT_OVERFLOW | ST_TABLE_STUCK | ST_COUNT_WIDTH)) {
      drop_graph(ctx);  // these inputs outgrew the captured sizes (or fail on the plain path)
      rc = run_count(ctx, cfg, mode, n_records);
      if (rc == MCZI_OK) capture_pipeline(ctx, cfg, mode, passes);
      return rc;
    }
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, ctx->ev_graph[0], ctx->ev_graph[1]));
    for (int i = 0; i < N_PHASES; i++) ctx->phase_ms[i] = 0.f;
    ctx->phase_ms[3] = ms;  // one graph: the whole pipeline's device time
    std::memset(ctx->stats, 0, sizeof ctx->stats);
    const uint64_t* nb = reinterpret_cast<const uint64_t*>(ctx->base_pre.as<BaseSum>() + ctx->n_tiles);
    CK(cudaMemcpy(&ctx->stats[0], nb, 8, cudaMemcpyDeviceToHost));
    ctx->stats[5] = h[SC_NOUT];
    ctx->stats[7] = ctx->skipped;
    ctx->stats[8] = ctx->graph_launches_per_replay;
    ctx->stats[9] = ctx->h2d_bytes;
    ctx->mode = mode;
    ctx->k = (int)cfg->k;
    ctx->m = (int)cfg->minimizer;
    ctx->x = cfg->threshold;
    ctx->n_out = h[SC_NOUT];
    ctx->mask_words = 0;
    ctx->have_result = true;
    ctx->graph_replays++;
    if (n_records) *n_records = h[SC_NOUT];
    return MCZI_OK;
  }
  rc = run_count(ctx, cfg, mode, n_records);
  if (rc == MCZI_OK) capture_pipeline(ctx, cfg, mode, passes);
  return rc;
}

__global__ void k_widen_counts(const uint32_t* __restrict__ in, uint64_t n, unsigned long long* __restrict__ out) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = in[i];
}

// KFF records (src/lib.rs:3089-3117): the k-mer as ceil(k/4) big-endian bytes
// of its 2k-bit value, then the count (count_size 1: saturated at sat; 4 or
// 8: big-endian)
__global__ void k_kff_records(const uint64_t* __restrict__ lo, const uint64_t* __restrict__ hi,
                              const uint32_t* __restrict__ cnt, uint64_t n, int nb, int count_size, uint32_t sat,
                              uint8_t* __restrict__ out) {
  const int rl = nb + count_size;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    uint8_t* o = out + i * (uint64_t)rl;
    const uint64_t l = lo[i], h = hi ? hi[i] : 0ull;
    for (int j = 0; j < nb; j++) {
      const int bit = 8 * (nb - 1 - j);
      o[j] = (uint8_t)(bit >= 64 ? (h >> (bit - 64)) : (l >> bit));
    }
    const uint32_t c = cnt[i];
    if (count_size == 1) {
      o[nb] = (uint8_t)(c < sat ? c : sat);
    } else {
      for (int j = 0; j < count_size; j++) {
        const int bit = 8 * (count_size - 1 - j);
        o[nb + j] = (uint8_t)(bit >= 32 ? 0u : (c >> bit));
      }
    }
  }
}

void launch_kff_records(const uint64_t* lo, const uint64_t* hi, const uint32_t* cnt, uint64_t n, int nb,
                        int count_size, uint32_t sat, uint8_t* out, int sm_count, cudaStream_t s) {
  const uint64_t g = (n + 255) / 256;
  const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(g, (uint64_t)sm_count * 16));
  k_kff_records<<<grid, 256, 0, s>>>(lo, hi, cnt, n, nb, count_size, sat, out);
}

int32_t fetch_records(mczi_ctx* ctx, HostRecords* r) {
  const uint64_t n = ctx->n_out;
  r->lo.resize(n);
  r->count.resize(n);
  if (ctx->k > 32) r->hi.resize(n);
  else r->hi.clear();
  if (n == 0) return MCZI_OK;
  std::vector<uint32_t> c32(n);
  CK(cudaMemcpyAsync(r->lo.data(), ctx->out_lo.p, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
  if (ctx->k > 32) CK(cudaMemcpyAsync(r->hi.data(), ctx->out_hi.p, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(c32.data(), ctx->out_cnt.p, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  for (uint64_t i = 0; i < n; i++) r->count[i] = c32[i];
  return MCZI_OK;
}

int32_t count_paths(mczi_ctx* ctx, const char* const* paths, size_t n, const mczi_counter_config* cfg, int mode,
                    const char* out, bool kff) {
  if (!ctx) return MCZI_ERR_STATE;
  int32_t rc = validate(ctx, cfg, mode);
  if (rc) return rc;
  if (n == 0) return fail(ctx, MCZI_ERR_INVALID_CONFIG, mode ? "at least one dataset file is required"
                                                              : "at least one input file is required");
  // plain, gzip, xz or zstd files, decoded on parallel host threads
  std::vector<std::vector<uint8_t>> data;
  std::string e;
  // (gzip files whose members carry their sizes stay compressed: decoded on the device)
  if (!read_input_files(paths, n, &data, &e, true)) return fail(ctx, MCZI_ERR_IO, e);
  std::vector<mczi_input> in(n);
  for (size_t i = 0; i < n; i++) {
    in[i].data = data[i].data();
    in[i].len = data[i].size();
  }
  rc = mczi_count(ctx, cfg, mode, in.data(), n, nullptr);
  if (rc) return rc;
  return kff ? mczi_result_write_kff(ctx, out) : mczi_result_write_fasta(ctx, out);
}

}  // namespace

}  // namespace

extern "C" {

int32_t mczi_open(int32_t device, mczi_ctx** out) {
  if (!out) return MCZI_ERR_STATE;
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    return MCZI_ERR_DEVICE;
  }
  if (device < 0 || device >= n) return MCZI_ERR_DEVICE;
  if (cudaSetDevice(device) != cudaSuccess) return MCZI_ERR_DEVICE;
  mczi_ctx* ctx = new mczi_ctx();
  ctx->device = device;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) {
    delete ctx;
    return MCZI_ERR_DEVICE;
  }
  ctx->sm_count = prop.multiProcessorCount;
  ctx->smem_optin = prop.sharedMemPerBlockOptin;
  ctx->smem_per_sm = prop.sharedMemPerMultiprocessor;
  ctx->smem_reserved = prop.reservedSharedMemPerBlock;
  if (cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete ctx;
    return MCZI_ERR_DEVICE;
  }
  ctx->stream = ctx->own_stream;
  for (auto& ev : ctx->ev) cudaEventCreate(&ev);
  for (auto& ev : ctx->ev_pre) cudaEventCreate(&ev);
  for (auto& ev : ctx->ev_graph) cudaEventCreate(&ev);
  cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking);
  cudaEventCreateWithFlags(&ctx->ev_copy, cudaEventDisableTiming);
  *out = ctx;
  return MCZI_OK;
}

int32_t mczi_close(mczi_ctx* ctx) {
  if (!ctx) return MCZI_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
  // every device buffer is a DevBuf member: deleting the context frees them
  for (auto& ev : ctx->ev) if (ev) cudaEventDestroy(ev);
  for (auto& ev : ctx->ev_pre) if (ev) cudaEventDestroy(ev);
  for (auto& ev : ctx->ev_graph) if (ev) cudaEventDestroy(ev);
  if (ctx->ev_copy) cudaEventDestroy(ctx->ev_copy);
  if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
  drop_graph(ctx);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
  return MCZI_OK;
}

const char* mczi_last_error(const mczi_ctx* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

int32_t mczi_set_stream(mczi_ctx* ctx, void* stream) {
  if (!ctx) return MCZI_ERR_STATE;
  ctx->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
  return MCZI_OK;
}

int32_t mczi_validate_config(mczi_ctx* ctx, const mczi_counter_config* cfg, int32_t mode) {
  return validate(ctx, cfg, mode);
}

int32_t mczi_stage(mczi_ctx* ctx, const mczi_input* inputs, size_t n_inputs) {
  if (!ctx) return MCZI_ERR_STATE;
  cudaSetDevice(ctx->device);
  return stage_inputs(ctx, inputs, n_inputs);
}

int32_t mczi_count_staged(mczi_ctx* ctx, const mczi_counter_config* cfg, int32_t mode, uint64_t* n_records) {
  if (!ctx) return MCZI_ERR_STATE;
  cudaSetDevice(ctx->device);
  return ctx->graph_mode ? run_count_graph(ctx, cfg, mode, n_records) : run_count(ctx, cfg, mode, n_records);
}

int32_t mczi_count(mczi_ctx* ctx, const mczi_counter_config* cfg, int32_t mode, const mczi_input* inputs,
                   size_t n_inputs, uint64_t* n_records) {
  if (!ctx) return MCZI_ERR_STATE;
  cudaSetDevice(ctx->device);
  int32_t rc = validate(ctx, cfg, mode);
  if (rc) return rc;
  if (!ctx->graph_mode) return run_count_streamed(ctx, cfg, mode, inputs, n_inputs, n_records);
  rc = stage_inputs(ctx, inputs, n_inputs);
  if (rc) return rc;
  return run_count_graph(ctx, cfg, mode, n_records);
}

int32_t mczi_result_copy(mczi_ctx* ctx, uint64_t* key_lo, uint64_t* key_hi, uint64_t* counts, uint64_t cap,
                         int32_t sorted) {
  if (!ctx) return MCZI_ERR_STATE;
  if (!ctx->have_result) return fail(ctx, MCZI_ERR_STATE, "no result");
  if (cap < ctx->n_out) return fail(ctx, MCZI_ERR_STATE, "result buffer too small");
  cudaSetDevice(ctx->device);
  if (!sorted) {
    // emission order: straight into the caller's buffers (counts widened on
    // the device), no host-side pass over the records
    const uint64_t n = ctx->n_out;
    cudaStream_t s = ctx->stream;
    if (n == 0) return MCZI_OK;
    if (key_lo) CK(cudaMemcpyAsync(key_lo, ctx->out_lo.p, n * 8, cudaMemcpyDeviceToHost, s));
    if (key_hi) {
      if (ctx->k > 32) CK(cudaMemcpyAsync(key_hi, ctx->out_hi.p, n * 8, cudaMemcpyDeviceToHost, s));
      else std::fill(key_hi, key_hi + n, 0ull);
    }
    if (counts) {
      CKA(ctx->cnt64, n * 8);
      const unsigned grid = (unsigned)std::min<uint64_t>((n + 255) / 256, (uint64_t)ctx->sm_count * 8);
      k_widen_counts<<<grid, 256, 0, s>>>(ctx->out_cnt.as<uint32_t>(), n, ctx->cnt64.as<unsigned long long>());
      CK(cudaGetLastError());
      CK(cudaMemcpyAsync(counts, ctx->cnt64.p, n * 8, cudaMemcpyDeviceToHost, s));
    }
    CK(cudaStreamSynchronize(s));
    return MCZI_OK;
  }
  HostRecords r;
  int32_t rc = fetch_records(ctx, &r);
  if (rc) return rc;
  const uint64_t n = ctx->n_out;
  std::vector<uint64_t> idx(n);
  std::iota(idx.begin(), idx.end(), 0ull);
  if (sorted) {
    if (r.hi.empty()) std::sort(idx.begin(), idx.end(), [&](uint64_t a, uint64_t b) { return r.lo[a] < r.lo[b]; });
    else
      std::sort(idx.begin(), idx.end(), [&](uint64_t a, uint64_t b) {
        return r.hi[a] < r.hi[b] || (r.hi[a] == r.hi[b] && r.lo[a] < r.lo[b]);
      });
  }
  for (uint64_t i = 0; i < n; i++) {
    const uint64_t j = idx[i];
    if (key_lo) key_lo[i] = r.lo[j];
    if (key_hi) key_hi[i] = r.hi.empty() ? 0 : r.hi[j];
    if (counts) counts[i] = r.count[j];
  }
  return MCZI_OK;
}

// order-independent digest of the result records: the murmur3 64-bit
// finaliser chained over (lo, hi, count); summed (wrapping) and xor-ed over
// the records, so the value does not depend on emission order
__device__ __forceinline__ uint64_t dg_mix64(uint64_t x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ull;
  return x ^ (x >> 33);
}

__global__ void k_result_digest(const uint64_t* __restrict__ lo, const uint64_t* __restrict__ hi,
                                const uint32_t* __restrict__ cnt, uint64_t n, int unit_counts,
                                unsigned long long* __restrict__ acc) {
  uint64_t cs = 0, sum = 0, x = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t c = unit_counts ? 1ull : (uint64_t)cnt[i];
    const uint64_t h = dg_mix64(lo[i]) ^ (hi ? hi[i] : 0ull);
    const uint64_t w = dg_mix64(dg_mix64(h) + c);
    cs += c;
    sum += w;
    x ^= w;
  }
  for (int o = 16; o; o >>= 1) {
    cs += __shfl_xor_sync(0xffffffffu, cs, o);
    sum += __shfl_xor_sync(0xffffffffu, sum, o);
    x ^= __shfl_xor_sync(0xffffffffu, x, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&acc[0], (unsigned long long)cs);
    atomicAdd(&acc[1], (unsigned long long)sum);
    atomicXor(&acc[2], (unsigned long long)x);
  }
}

int32_t mczi_inflate_gzip(mczi_ctx* ctx, const uint8_t* gz, uint64_t len, uint8_t* out, uint64_t cap,
                          uint64_t* n_out) {
  if (!ctx) return MCZI_ERR_STATE;
  if (!n_out) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "n_out must not be NULL");
  *n_out = 0;
  std::vector<GzSpan> spans;
  uint64_t total = 0;
  if (!gz || !gzip_sized_members(gz, len, &spans, &total))
    return fail(ctx, MCZI_ERR_INVALID_CONFIG, "not a gzip buffer whose members carry their sizes (BGZF)");
  *n_out = total;
  if (total > cap || (total && !out)) return fail(ctx, MCZI_ERR_TOO_LARGE, "output buffer smaller than the decoded bytes");
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  std::vector<GzMember> m;
  m.reserve(spans.size());
  uint64_t o = 0;
  for (const GzSpan& sp : spans) {
    m.push_back(GzMember{sp.in_off, o, sp.in_len, sp.out_len, sp.crc, 0});
    o += sp.out_len;
  }
  CKA(ctx->gz_comp, len + 16);
  CKA(ctx->gz_members, m.size() * sizeof(GzMember));
  CKA(ctx->gz_out, total + 16);
  CKA(ctx->gz_scratch, 64);
  uint32_t* scr = ctx->gz_scratch.as<uint32_t>();
  CK(cudaMemcpyAsync(ctx->gz_comp.p, gz, len, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(ctx->gz_members.p, m.data(), m.size() * sizeof(GzMember), cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(scr, 0, 64, s));
  CK(cudaEventRecord(ctx->ev[0], s));
  launch_inflate(ctx->gz_comp.as<uint8_t>(), ctx->gz_members.as<GzMember>(), (uint32_t)m.size(),
                 ctx->gz_out.as<uint8_t>(), scr, scr + 1, ctx->sm_count * 16, s);
  CK(cudaGetLastError());
  CK(cudaEventRecord(ctx->ev[1], s));
  uint32_t st = 0;
  CK(cudaMemcpyAsync(&st, scr + 1, 4, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  CK(cudaEventElapsedTime(&ctx->inflate_ms, ctx->ev[0], ctx->ev[1]));
  if (st & ST_GZ_CORRUPT)
    return fail(ctx, MCZI_ERR_IO, "gzip input: a member is not valid DEFLATE data or does not match its size or CRC-32");
  if (total) {
    CK(cudaMemcpyAsync(out, ctx->gz_out.p, total, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
  }
  return MCZI_OK;
}

int32_t mczi_result_digest(mczi_ctx* ctx, int32_t unit_counts, uint64_t* out) {
  if (!ctx) return MCZI_ERR_STATE;
  if (!out) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "out must not be NULL");
  if (!ctx->have_result) return fail(ctx, MCZI_ERR_STATE, "no result");
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  const uint64_t n = ctx->n_out;
  CKA(ctx->digest_acc, 4 * sizeof(uint64_t));
  CK(cudaMemsetAsync(ctx->digest_acc.p, 0, 4 * sizeof(uint64_t), s));
  if (n) {
    const unsigned grid = (unsigned)std::min<uint64_t>((n + 255) / 256, (uint64_t)ctx->sm_count * 8);
    k_result_digest<<<grid, 256, 0, s>>>(ctx->out_lo.as<uint64_t>(), ctx->k > 32 ? ctx->out_hi.as<uint64_t>() : nullptr,
                                         ctx->out_cnt.as<uint32_t>(), n, unit_counts ? 1 : 0,
                                         ctx->digest_acc.as<unsigned long long>());
    CK(cudaGetLastError());
  }
  uint64_t acc[4] = {0, 0, 0, 0};
  CK(cudaMemcpyAsync(acc, ctx->digest_acc.p, 3 * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  out[0] = n;
  out[1] = acc[0];
  out[2] = acc[1];
  out[3] = acc[2];
  return MCZI_OK;
}

int32_t mczi_result_write_kff(mczi_ctx* ctx, const char* path) {
  if (!ctx) return MCZI_ERR_STATE;
  if (!ctx->have_result) return fail(ctx, MCZI_ERR_STATE, "no result");
  cudaSetDevice(ctx->device);
  // records formatted on the device as the file stores them, copied once
  const int count_size = ctx->mode == MCZI_MODE_PRESENCE ? 4 : (ctx->k <= 32 ? 1 : 8);
  const int nb = (ctx->k + 3) / 4;
  const uint64_t n = ctx->n_out, bytes = n * (uint64_t)(nb + count_size);
  if (n) {
    CKA(ctx->kff_dev, bytes);
    const cudaError_t he = ctx->kff_host.ensure(bytes);
    if (he != cudaSuccess) {
      cudaGetLastError();
      return fail(ctx, MCZI_ERR_OOM, "pinned host allocation for the KFF records failed");
    }
    const uint64_t sat = ctx->x + 1 < 255 ? ctx->x + 1 : 255;
    launch_kff_records(ctx->out_lo.as<uint64_t>(), ctx->k > 32 ? ctx->out_hi.as<uint64_t>() : nullptr,
                       ctx->out_cnt.as<uint32_t>(), n, nb, count_size, (uint32_t)sat, ctx->kff_dev.as<uint8_t>(),
                       ctx->sm_count, ctx->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(ctx->kff_host.p, ctx->kff_dev.p, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  std::string e;
  if (!write_kff_records(path, ctx->k, ctx->m, ctx->x, count_size, n, static_cast<const uint8_t*>(ctx->kff_host.p),
                         bytes, &e))
    return fail(ctx, MCZI_ERR_IO, e);
  return MCZI_OK;
}

int32_t mczi_result_write_fasta(mczi_ctx* ctx, const char* path) {
  if (!ctx) return MCZI_ERR_STATE;
  if (!ctx->have_result) return fail(ctx, MCZI_ERR_STATE, "no result");
  cudaSetDevice(ctx->device);
  HostRecords r;
  int32_t rc = fetch_records(ctx, &r);
  if (rc) return rc;
  std::string e;
  if (r.lo.size() >= (1ull << 31)) {  // ranks must fit 31 bits: the plain writer
    if (!write_simplitig_file(path, r, ctx->k, &e)) return fail(ctx, MCZI_ERR_IO, e);
    return MCZI_OK;
  }
  // seeds in ascending order (host, parallel), their extensions on the device,
  // then the greedy walk over the table (host)
  std::vector<uint64_t> lo, hi;
  const unsigned hw = std::thread::hardware_concurrency();
  sorted_keys(r, &lo, &hi, (int)std::max(1u, std::min(hw, 64u)));
  r = HostRecords();
  std::vector<uint32_t> ext(lo.size() * SIMPLITIG_STRIDE);
  if ((rc = simplitig_extensions(ctx, lo.data(), hi.data(), lo.size(), ctx->k, ext.data()))) return rc;
  if (!write_simplitig_walk(path, lo.data(), hi.data(), lo.size(), ctx->k, ext.data(), &e)) return fail(ctx, MCZI_ERR_IO, e);
  return MCZI_OK;
}

int32_t mczi_count_inputs_to_kff_path(mczi_ctx* ctx, const char* const* inputs, size_t n,
                                      const mczi_counter_config* cfg, const char* out) {
  return count_paths(ctx, inputs, n, cfg, MCZI_MODE_ABUNDANCE, out, true);
}
int32_t mczi_count_inputs_to_fasta_path(mczi_ctx* ctx, const char* const* inputs, size_t n,
                                        const mczi_counter_config* cfg, const char* out) {
  return count_paths(ctx, inputs, n, cfg, MCZI_MODE_ABUNDANCE, out, false);
}
int32_t mczi_count_datasets_to_kff_path(mczi_ctx* ctx, const char* const* inputs, size_t n,
                                        const mczi_counter_config* cfg, const char* out) {
  return count_paths(ctx, inputs, n, cfg, MCZI_MODE_PRESENCE, out, true);
}
int32_t mczi_count_datasets_to_fasta_path(mczi_ctx* ctx, const char* const* inputs, size_t n,
                                          const mczi_counter_config* cfg, const char* out) {
  return count_paths(ctx, inputs, n, cfg, MCZI_MODE_PRESENCE, out, false);
}

int32_t mczi_phase_times(mczi_ctx* ctx, float* ms, int32_t cap) {
  if (!ctx) return MCZI_ERR_STATE;
  int32_t n = std::min<int32_t>(cap, N_PHASES + 1);
  for (int32_t i = 0; i < n; i++) ms[i] = i < N_PHASES ? ctx->phase_ms[i] : ctx->inflate_ms;
  return n;
}

int32_t mczi_run_stats(mczi_ctx* ctx, uint64_t* out, int32_t cap) {
  if (!ctx) return MCZI_ERR_STATE;
  int32_t n = std::min<int32_t>(cap, 10);
  for (int32_t i = 0; i < n; i++) out[i] = ctx->stats[i];
  return n;
}

int32_t mczi_set_count_tuning(mczi_ctx* ctx, int32_t threads, int32_t slots, int32_t ctas_per_sm) {
  if (!ctx) return MCZI_ERR_STATE;
  if (threads < 0 || threads > 1024 || (threads & 31)) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "bad thread count");
  if (ctas_per_sm < 0 || ctas_per_sm > 4) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "bad CTAs per SM");
  if (slots < 0) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "bad slot count");
  ctx->count_threads = threads;
  ctx->count_slots = slots;
  ctx->count_ctas_per_sm = ctas_per_sm;
  return MCZI_OK;
}

int32_t mczi_set_count_options(mczi_ctx* ctx, int32_t chunk, float fill) {
  if (!ctx) return MCZI_ERR_STATE;
  if (chunk < 0 || chunk > 4096) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "bad chunk");
  if (fill < 0.f || fill > 0.85f) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "fill must be in (0, 0.85]");
  ctx->count_chunk = chunk;
  ctx->count_fill = fill;
  return MCZI_OK;
}

int32_t mczi_set_graph_replay(mczi_ctx* ctx, int32_t enable) {
  if (!ctx) return MCZI_ERR_STATE;
  ctx->graph_mode = enable != 0;
  if (!ctx->graph_mode) drop_graph(ctx);
  return MCZI_OK;
}

int32_t mczi_set_key_range_passes(mczi_ctx* ctx, int32_t passes) {
  if (!ctx) return MCZI_ERR_STATE;
  if (passes < 0 || passes > 64) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "passes must be in [0, 64]");
  ctx->key_passes = passes;
  return MCZI_OK;
}

int32_t mczi_set_count_filter(mczi_ctx* ctx, int32_t mode) {
  if (!ctx) return MCZI_ERR_STATE;
  if (mode < -1 || mode > 1) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "filter mode must be -1, 0 or 1");
  ctx->count_filter = mode;
  return MCZI_OK;
}

int32_t mczi_set_streamed_staging(mczi_ctx* ctx, int32_t enable, uint64_t segment_bytes) {
  if (!ctx) return MCZI_ERR_STATE;
  if (segment_bytes % PACK_TILE) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "segment size must be a multiple of 8192");
  ctx->streamed = enable ? 1 : 0;
  ctx->stream_seg_tiles = segment_bytes / PACK_TILE;
  return MCZI_OK;
}

int32_t mczi_set_zi_bucket_records(mczi_ctx* ctx, uint32_t records) {
  if (!ctx) return MCZI_ERR_STATE;
  ctx->zi_bucket_records = records;
  return MCZI_OK;
}

int32_t mczi_set_minimizer_precount(mczi_ctx* ctx, int32_t enable) {
  if (!ctx) return MCZI_ERR_STATE;
  ctx->precount = enable ? 1 : 0;
  return MCZI_OK;
}

int32_t mczi_debug_set_bucket_window_limit(mczi_ctx* ctx, uint64_t windows) {
  if (!ctx) return MCZI_ERR_STATE;
  if (windows > 0xffffffffull) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "limit above the 32-bit counters' range");
  ctx->max_bucket_windows = windows;
  drop_graph(ctx);
  return MCZI_OK;
}

int32_t mczi_debug_packed(mczi_ctx* ctx, uint8_t* codes, uint8_t* starts, uint64_t cap, uint64_t* n_bases) {
  if (!ctx || !ctx->have_result) return fail(ctx, MCZI_ERR_STATE, "no result");
  cudaSetDevice(ctx->device);
  const uint64_t nb = ctx->stats[0];
  if (n_bases) *n_bases = nb;
  if (!codes && !starts) return MCZI_OK;
  if (cap < nb) return fail(ctx, MCZI_ERR_STATE, "buffer too small");
  std::vector<uint32_t> pk(nb / 16 + 1), fb(nb / 32 + 1);
  CK(cudaMemcpy(pk.data(), ctx->packed.p, pk.size() * 4, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(fb.data(), ctx->fbits.p, fb.size() * 4, cudaMemcpyDeviceToHost));
  for (uint64_t i = 0; i < nb; i++) {
    if (codes) codes[i] = (uint8_t)((pk[i >> 4] >> (30 - 2 * (i & 15))) & 3u);
    if (starts) starts[i] = (uint8_t)((fb[i >> 5] >> (i & 31)) & 1u);
  }
  return MCZI_OK;
}

}  // extern "C"
