// exchange.cu -- the local step of MC counting on several GPUs: route each
// superkmer of this GPU's share of the reads to the GPU that counts its
// minimizer bucket.
//
// MC's k-mer set partitions by minimizer: every occurrence of a canonical
// k-mer lies in a superkmer with the same minimizer key (the hash is
// strand-symmetric), so the partition buckets (p1 = key >> 20, the 4096
// buckets of one GPU's own pipeline) can be counted on different GPUs with
// no further exchange.  Bucket p goes to GPU p mod G.  The reference's
// counterpart is its partition files (src/lib.rs:4821-4925 writes every
// superkmer to partition_NNNN.skm, src/lib.rs:2803-2845 the temp folders),
// which each partition's counter then reads back.
//
// Here a GPU packs and scans its reads as for a count, then writes every
// superkmer as a one-line FASTA record (its windows + k - 1 bases) into the
// group of its destination; the groups go to their GPUs (one all-to-all), and
// each GPU counts what it received with mczi_count.  The k-mers of a record
// are exactly the superkmer's windows, so the union of the GPUs' results is
// the single-GPU result, record for record.
#include "api_internal.h"
#include "mczi_common.cuh"

#include <algorithm>
#include <cstring>
#include <vector>

namespace mczi {

namespace {

constexpr uint32_t ROUTE_MAX_DEST = 1024;
constexpr int ROUTE_THREADS = 256;

__device__ __forceinline__ uint32_t route_dest(uint32_t key, uint32_t n_dest) { return (key >> 20) % n_dest; }

// record bytes: '>' '\n' bases '\n'
__device__ __forceinline__ uint64_t route_rec_bytes(uint64_t d, int k) {
  return (uint64_t)((uint32_t)(d & 0xffffffu) + 1u) + (uint64_t)(k - 1) + 3u;
}

__global__ void __launch_bounds__(ROUTE_THREADS) k_route_count(const uint64_t* __restrict__ desc,
                                                               const uint32_t* __restrict__ key, uint64_t n, int k,
                                                               uint32_t n_dest, unsigned long long* bytes) {
  __shared__ unsigned long long sb[ROUTE_MAX_DEST];
  for (uint32_t i = threadIdx.x; i < n_dest; i += blockDim.x) sb[i] = 0;
  __syncthreads();
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    atomicAdd(&sb[route_dest(key[i], n_dest)], (unsigned long long)route_rec_bytes(desc[i], k));
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < n_dest; i += blockDim.x)
    if (sb[i]) atomicAdd(&bytes[i], sb[i]);
}

// each superkmer takes its place in its destination's group from a cursor
// (the order inside a group does not matter to the count) and writes itself
// as ASCII bases
__global__ void __launch_bounds__(ROUTE_THREADS) k_route_write(const uint64_t* __restrict__ desc,
                                                               const uint32_t* __restrict__ key, uint64_t n,
                                                               const uint32_t* __restrict__ packed, int k,
                                                               uint32_t n_dest, unsigned long long* cursor,
                                                               uint8_t* __restrict__ out) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t d = desc[i];
    const uint64_t nb = route_rec_bytes(d, k);
    const uint64_t at = atomicAdd(&cursor[route_dest(key[i], n_dest)], (unsigned long long)nb);
    uint8_t* o = out + at;
    o[0] = '>';
    o[1] = '\n';
    const uint64_t s0 = d >> 24, len = nb - 3;
    for (uint64_t j = 0; j < len; j++) o[2 + j] = (uint8_t)"ACGT"[base_at(packed, s0 + j)];
    o[2 + len] = '\n';
  }
}

}  // namespace

}  // namespace mczi

using namespace mczi;

extern "C" {

int32_t mczi_route_superkmers(mczi_ctx* ctx, const mczi_counter_config* cfg, const mczi_input* inputs,
                              size_t n_inputs, uint32_t n_dest, uint64_t* dest_bytes) {
  if (!ctx) return MCZI_ERR_STATE;
  int32_t rc = mczi_validate_config(ctx, cfg, MCZI_MODE_ABUNDANCE);
  if (rc) return rc;
  if (n_dest < 1 || n_dest > ROUTE_MAX_DEST) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "n_dest must be in [1, 1024]");
  if (!dest_bytes) return fail(ctx, MCZI_ERR_INVALID_CONFIG, "dest_bytes must not be NULL");
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  const int k = (int)cfg->k, m = (int)cfg->minimizer;
  ctx->route.assign(n_dest, {});
  ctx->have_result = false;
  if ((rc = stage_inputs(ctx, inputs, n_inputs))) return rc;
  Pipe p;
  if ((rc = pipe_pack(ctx, p))) return rc;
  CK(cudaMemcpyAsync(&p.n_bases_host, p.d_nbases, 8, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  const uint32_t passes = key_range_passes(ctx, k, m, p.n_bases_host);
  std::vector<uint64_t> bytes(n_dest), cur(n_dest);
  for (uint32_t r = 0; r < passes; r++) {
    const uint32_t lo = (uint32_t)((uint64_t)NP1 * r / passes), hi = (uint32_t)((uint64_t)NP1 * (r + 1) / passes);
    if ((rc = pipe_scan(ctx, p, k, m, lo, hi, passes))) return rc;
    if (p.n_desc == 0) continue;
    const uint64_t* desc = ctx->desc.as<uint64_t>();
    const uint32_t* key = ctx->key.as<uint32_t>();
    const unsigned grid = (unsigned)std::min<uint64_t>((p.n_desc + ROUTE_THREADS - 1) / ROUTE_THREADS,
                                                       (uint64_t)ctx->sm_count * 8);
    CKA(ctx->zi_tmp0, (size_t)n_dest * 8 * 2);
    unsigned long long* d_bytes = ctx->zi_tmp0.as<unsigned long long>();
    unsigned long long* d_cur = d_bytes + n_dest;
    CK(cudaMemsetAsync(d_bytes, 0, (size_t)n_dest * 8, s));
    k_route_count<<<grid, ROUTE_THREADS, 0, s>>>(desc, key, p.n_desc, k, n_dest, d_bytes);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(bytes.data(), d_bytes, (size_t)n_dest * 8, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    uint64_t total = 0;
    for (uint32_t d = 0; d < n_dest; d++) {
      cur[d] = total;
      total += bytes[d];
    }
    CKA(ctx->zi_tmp1, total);
    CK(cudaMemcpyAsync(d_cur, cur.data(), (size_t)n_dest * 8, cudaMemcpyHostToDevice, s));
    k_route_write<<<grid, ROUTE_THREADS, 0, s>>>(desc, key, p.n_desc, ctx->packed.as<uint32_t>(), k, n_dest, d_cur,
                                                 ctx->zi_tmp1.as<uint8_t>());
    CK(cudaGetLastError());
    for (uint32_t d = 0; d < n_dest; d++) {
      std::vector<uint8_t>& g = ctx->route[d];
      const size_t old = g.size();
      g.resize(old + bytes[d]);
      if (bytes[d])
        CK(cudaMemcpyAsync(g.data() + old, ctx->zi_tmp1.as<uint8_t>() + cur[d], bytes[d], cudaMemcpyDeviceToHost, s));
    }
    CK(cudaStreamSynchronize(s));
  }
  for (uint32_t d = 0; d < n_dest; d++) dest_bytes[d] = ctx->route[d].size();
  return MCZI_OK;
}

int32_t mczi_route_copy(mczi_ctx* ctx, uint32_t dest, uint8_t* out, uint64_t cap) {
  if (!ctx) return MCZI_ERR_STATE;
  if (dest >= ctx->route.size()) return fail(ctx, MCZI_ERR_STATE, "no routed group for this destination");
  const std::vector<uint8_t>& g = ctx->route[dest];
  if (cap < g.size()) return fail(ctx, MCZI_ERR_STATE, "buffer smaller than the routed group");
  if (!g.empty()) std::memcpy(out, g.data(), g.size());
  return MCZI_OK;
}

}  // extern "C"
