// mc_pack_noalloc.cu -- the FASTA/FASTQ packer for callers that cannot
// allocate device memory.
//
// Some callers cannot call cudaMalloc at the point where they need the
// packer: services that hand out device memory only from their own pre-sized
// arena (a cudaMalloc behind the arena's back breaks its accounting and can
// fail once the arena holds the free HBM), or real-time request paths where
// an allocation -- and the device-wide synchronisation it can cause -- is not
// acceptable.  For them this entry point runs the same three packing kernels
// as mczi_count's first phase, but keeps their per-tile scratch (line and
// base summaries and the scan temporaries) in one file-scope device array of
// fixed size instead of context buffers.  The call ends by copying the base
// count to the host and synchronising the caller's stream.
//
// The array belongs to this library's CUDA module: it is reserved on a device
// when the module is loaded there -- when the library is loaded under eager
// module loading, at the first kernel launch or symbol lookup on that device
// under lazy loading (CUDA_MODULE_LOADING=LAZY, the default since CUDA 12) --
// and held until the process exits.  Its host-side name is only a stand-in:
// the device address is looked up with cudaGetSymbolAddress, once per device,
// with that device current, on the first call on that device (the lookup
// may itself load the module there).
// The cached address is valid for the life of the device's primary context:
// a caller that ends it (cudaDeviceReset) must not call this entry point on
// that device again in the same process.  All calls share the array and it
// keeps the contents of the last call; everything that must start at zero is
// cleared on each call, and calls that overlap on the GPU (several streams,
// several host threads) race on it -- serialise them.
#include "../../include/mczi_gpu.h"
#include "mczi_internal.h"
#include "scan.cuh"

#include <mutex>

namespace mczi {

namespace {

constexpr uint64_t NOALLOC_SCRATCH_BYTES = 8ull << 20;  // 8 MiB
constexpr uint64_t NOALLOC_MAX_TILES = 65536;            // 512 MiB of text in PACK_TILE tiles

// per-tile scratch: tile_info (4 B), line sum + prefix (2 x 24 B), base sum +
// prefix (2 x 24 B), plus the scan temporaries, two per-input words and the
// 256-byte alignment of each of the nine pieces
constexpr uint64_t bytes_for_tiles(uint64_t n) {
  return n * 4 + 2 * (n + 1) * sizeof(LineSum) + 2 * (n + 1) * sizeof(BaseSum) +
         (n / SCAN_CHUNK + 2) * (sizeof(LineSum) + sizeof(BaseSum)) + 2 * 16 + 9 * 256;
}
static_assert(bytes_for_tiles(NOALLOC_MAX_TILES) <= NOALLOC_SCRATCH_BYTES, "scratch too small for the tile limit");

static __device__ __align__(256) uint8_t g_pack_scratch[NOALLOC_SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
uint8_t* g_addr[MAX_DEVICES] = {};

__global__ void k_noalloc_tile_info(uint32_t* tile_info, uint64_t n_tiles, uint32_t fastq) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n_tiles; t += (uint64_t)gridDim.x * blockDim.x)
    tile_info[t] = (fastq << 1) | (t == 0 ? 1u : 0u);  // one input, starting at tile 0
}

inline uint64_t align256(uint64_t x) { return (x + 255) & ~255ull; }

}  // namespace

}  // namespace mczi

using namespace mczi;

extern "C" int32_t mczi_pack_fastx_noalloc(const uint8_t* d_text, uint64_t text_len, int32_t fastq,
                                           uint32_t* d_packed, uint64_t packed_words, uint32_t* d_fbits,
                                           uint64_t fbits_words, uint64_t* n_bases, void* stream) {
  if (!d_text || !d_packed || !d_fbits || !n_bases) return MCZI_ERR_INVALID_CONFIG;
  if (text_len == 0 || text_len % PACK_TILE != 0) return MCZI_ERR_INVALID_CONFIG;
  if (text_len / PACK_TILE > NOALLOC_MAX_TILES) return MCZI_ERR_TOO_LARGE;
  if (packed_words < text_len / 16 + 8 || fbits_words < text_len / 32 + 8) return MCZI_ERR_INVALID_CONFIG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return MCZI_ERR_DEVICE;
  uint8_t* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_pack_scratch) != cudaSuccess || !p) {
        cudaGetLastError();
        return MCZI_ERR_DEVICE;
      }
      g_addr[dev] = static_cast<uint8_t*>(p);
    }
    base = g_addr[dev];
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const uint64_t n_tiles = text_len / PACK_TILE;
  const uint64_t ntmp = n_tiles / SCAN_CHUNK + 2;
  // carve the scratch
  uint64_t off = 0;
  auto take = [&](uint64_t bytes) {
    uint8_t* p = base + off;
    off = align256(off + bytes);
    return p;
  };
  PackArgs pa;
  pa.text = d_text;
  uint32_t* tile_info = reinterpret_cast<uint32_t*>(take(n_tiles * 4));
  uint64_t* input_tile0 = reinterpret_cast<uint64_t*>(take(16));
  uint64_t* input_base = reinterpret_cast<uint64_t*>(take(16));
  pa.line_sum = reinterpret_cast<LineSum*>(take((n_tiles + 1) * sizeof(LineSum)));
  pa.line_pre = reinterpret_cast<LineSum*>(take((n_tiles + 1) * sizeof(LineSum)));
  pa.line_tmp = reinterpret_cast<LineSum*>(take(ntmp * sizeof(LineSum)));
  pa.base_sum = reinterpret_cast<BaseSum*>(take((n_tiles + 1) * sizeof(BaseSum)));
  pa.base_pre = reinterpret_cast<BaseSum*>(take((n_tiles + 1) * sizeof(BaseSum)));
  pa.base_tmp = reinterpret_cast<BaseSum*>(take(ntmp * sizeof(BaseSum)));
  if (off > NOALLOC_SCRATCH_BYTES) return MCZI_ERR_TOO_LARGE;
  pa.tile_info = tile_info;
  pa.input_tile0 = input_tile0;
  pa.input_base = input_base;
  pa.n_tiles = n_tiles;
  pa.packed = d_packed;
  pa.fbits = d_fbits;
  // zero what must start at zero: the outputs (edge words are OR-ed) and the
  // per-input words; the summaries are fully overwritten by the kernels
  if (cudaMemsetAsync(input_tile0, 0, 16, s) != cudaSuccess) return MCZI_ERR_DEVICE;
  if (cudaMemsetAsync(input_base, 0, 16, s) != cudaSuccess) return MCZI_ERR_DEVICE;
  if (cudaMemsetAsync(d_packed, 0, packed_words * 4, s) != cudaSuccess) return MCZI_ERR_DEVICE;
  if (cudaMemsetAsync(d_fbits, 0, fbits_words * 4, s) != cudaSuccess) return MCZI_ERR_DEVICE;
  k_noalloc_tile_info<<<(unsigned)((n_tiles + 255) / 256 < 1024 ? (n_tiles + 255) / 256 : 1024), 256, 0, s>>>(
      tile_info, n_tiles, fastq ? 1u : 0u);
  launch_pack(pa, s);
  if (cudaGetLastError() != cudaSuccess) return MCZI_ERR_DEVICE;
  // total bases = base_pre[n_tiles].nb (first field of BaseSum)
  if (cudaMemcpyAsync(n_bases, pa.base_pre + n_tiles, sizeof(uint64_t), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return MCZI_ERR_DEVICE;
  if (cudaStreamSynchronize(s) != cudaSuccess) return MCZI_ERR_DEVICE;
  return MCZI_OK;
}
