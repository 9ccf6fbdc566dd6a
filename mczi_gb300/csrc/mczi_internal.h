// mczi_internal.h -- kernel launch interfaces shared between the .cu files
// of libmczi_gpu (not part of the public C ABI).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace mczi {

// ---------------------------------------------------------------- K1 packer
// The tile sizes are compile-time constants (shared-memory arrays and unrolled
// per-thread loops are sized by them); a build may override the packer's
// threads per 8 KiB tile with -DMCZI_PACK_THREADS=n (64, 128 or 256: 128, 64
// or 32 text bytes per thread) and the scan tile with -DMCZI_SCAN_TILE=n
// (<= 8192 windows, 16 per thread) to measure other sizes.  The defaults are
// the fastest of those measured on GB300.
#ifndef MCZI_PACK_THREADS
#define MCZI_PACK_THREADS 128
#endif
#ifndef MCZI_SCAN_TILE
#define MCZI_SCAN_TILE 4096
#endif
constexpr int PACK_THREADS = MCZI_PACK_THREADS;
constexpr int PACK_TILE = 8192;  // text bytes per CTA (inputs are laid out in whole tiles)
constexpr int PACK_PER_THREAD = PACK_TILE / PACK_THREADS;
static_assert(PACK_PER_THREAD % 32 == 0 && PACK_THREADS % 32 == 0, "whole 32-byte chunks, whole warps per tile");

struct LineSum {
  int64_t last;   // absolute position of the last '\n' (or -1)
  uint32_t nl;    // newline count
  uint32_t reset; // an input starts at this tile
  uint32_t pad;
};

struct BaseSum {
  uint64_t nb;    // bases
  uint32_t fb;    // a break precedes the first base (nb > 0)
  uint32_t lb;    // a break follows the last base (nb > 0) / any break (nb == 0)
  uint32_t pad;
};

struct PackArgs {
  const uint8_t* text;       // tile-aligned input bytes
  const uint32_t* tile_info; // input << 2 | fastq << 1 | input starts here
  const uint64_t* input_tile0;  // first tile of each input
  uint64_t n_tiles;
  LineSum* line_sum;  LineSum* line_pre;  LineSum* line_tmp;
  BaseSum* base_sum;  BaseSum* base_pre;  BaseSum* base_tmp;  // base_pre[n_tiles].nb = total bases
  uint32_t* packed;   // zeroed, >= n_bases/16 + 8 words
  uint32_t* fbits;    // zeroed, >= n_bases/32 + 8 words
  uint64_t* input_base;  // first base of each input
};
void launch_pack(const PackArgs& a, cudaStream_t s);
// tiles [t0, t1) only, after tiles [0, t0): the prefix scans continue from the
// running totals (carry_* are one-element device scratch each)
void launch_pack_segment(const PackArgs& a, uint64_t t0, uint64_t t1, LineSum* carry_line, BaseSum* carry_base,
                         cudaStream_t s);

// ------------------------------------------------------ gzip on the device
// One gzip member (RFC 1952) of an input whose members carry their size
// (BGZF's "BC" extra field): its raw DEFLATE data in the compressed buffer,
// where its bytes go in the output, and its trailer.
struct GzMember {
  uint64_t in_off;   // DEFLATE data offset in the compressed buffer
  uint64_t out_off;  // offset of the decoded bytes in the output
  uint32_t in_len;   // DEFLATE data bytes (header and trailer excluded)
  uint32_t out_len;  // ISIZE: decoded bytes
  uint32_t crc;      // CRC-32 of the decoded bytes
  uint32_t input;    // index of the input the member belongs to
};
// Decodes every member into out (one warp per member, members taken from
// *work, which must start at 0); a member that is not valid DEFLATE, decodes
// to another length or fails its CRC sets ST_GZ_CORRUPT in *status.
void launch_inflate(const uint8_t* comp, const GzMember* members, uint32_t n_members, uint8_t* out,
                    unsigned int* work, uint32_t* status, int ctas, cudaStream_t s);

// partition digits of the superkmer key (mix32 of the minimizer value)
constexpr int P1_BITS = 12;
constexpr int P2_BITS = 11;
constexpr int NP1 = 1 << P1_BITS;
constexpr int NP2 = 1 << P2_BITS;

// ---------------------------------------------------------------- K2 scan
constexpr int SCAN_TILE = MCZI_SCAN_TILE;  // windows per CTA
constexpr int SCANK_THREADS = SCAN_TILE / 16;  // one thread owns 16 windows

struct ScanArgs {
  const uint32_t* packed;
  const uint32_t* fbits;
  const uint64_t* n_bases;   // device scalar
  uint64_t max_bases;        // grid bound (host upper bound on n_bases)
  uint64_t packed_words;     // allocated words (reads beyond are zero)
  int k, m;
  uint64_t* desc;            // start << 24 | (windows - 1)
  uint32_t* key;             // partition key = mix32(minimizer hash)
  unsigned long long* n_desc;  // device counter
  uint64_t desc_cap;
  uint32_t* status;
  uint32_t p1_lo, p1_hi;     // emit superkmers with key >> (32 - P1_BITS) in [p1_lo, p1_hi)
  const uint64_t* tile_range;  // null: every tile; else device [first, end) of the tiles to scan
};
void launch_scan(const ScanArgs& a, cudaStream_t s);
// Streamed scan: `range` (device, two words, start zeroed) advances to the
// tiles whose packed words are complete given `avail` packed bases (all tiles
// when `final`), at most `max_tiles` of them; a final window with more sets
// ST_DESC_OVERFLOW.  launch_scan_range then scans the range.
void launch_scan_window(const uint64_t* avail, uint64_t* range, bool final, uint64_t max_tiles, uint32_t* status,
                        cudaStream_t s);
void launch_scan_range(const ScanArgs& a, uint64_t max_tiles, cudaStream_t s);

// ---------------------------------------------------------------- K3 partition
constexpr int PART_CTAS = 152;   // 1 per SM on a 152-SM GB300
constexpr int PART_THREADS = 1024;

struct PartArgs {
  const uint64_t* desc_in;
  const uint32_t* key_in;
  uint64_t* desc_out;
  uint32_t* key_out;
  const unsigned long long* n_desc;  // device scalar
  uint64_t desc_cap;
  uint32_t* hist;       // scratch: NP1 histogram + the two levels' cursors
  uint64_t* bucket_off; // NP1 + 1 bucket offsets (p1 buckets)
  uint32_t* status;
};
// p1 in two tile-sorted levels: (desc_in, key_in) -> (desc_out, tmp_p1)
// grouped by the top p1 bits -> final_out grouped by p1 (bucket_off set);
// scratch holds NP1 + 64 + NP1 u32 (histogram and cursors).  final_out may
// be desc_in (level A has read it by then).
void launch_partition_tiled(const PartArgs& a, uint32_t* scratch, uint16_t* tmp_p1, uint64_t* final_out,
                            cudaStream_t s);

// ---------------------------------------------------------------- K4 pre-count
struct PrecountArgs {
  const uint64_t* desc;
  const uint32_t* key;
  const unsigned long long* n_desc;   // device scalar
  unsigned long long* table;          // key << 32 | count, 0 = empty
  uint64_t mask;                      // slots - 1 (power of two)
  unsigned long long* pairs;          // fof: key << 32 | (dataset + 1)
  uint64_t pair_mask;
  int mode;
  const uint64_t* dataset_base;
  int n_datasets;
  uint64_t threshold;
  uint64_t* desc_out;
  uint32_t* key_out;
  unsigned long long* n_kept;
  uint32_t* status;
};
void launch_precount(const PrecountArgs& a, int sm_count, cudaStream_t s);

// ---------------------------------------------------------------- K5 count
struct CountArgs {
  const uint32_t* packed;
  const uint64_t* desc;       // sorted by (p1, p2)
  // when set: the pass-1 output (grouped by p1 only); each CTA sorts its
  // bucket by p2 into `desc` itself (partition pass 2 fused into counting)
  const uint64_t* desc_unsorted;
  const uint32_t* key;
  const uint64_t* bucket_off; // NP1 + 1
  int k;
  uint64_t threshold;         // emit iff count > threshold
  int mode;                   // 0 abundance, 1 presence (fof)
  const uint64_t* dataset_base;  // n_datasets + 1 base offsets (presence mode)
  int n_datasets;
  // outputs
  uint64_t* out_lo;
  uint64_t* out_hi;           // only for k > 32
  uint32_t* out_count;
  unsigned long long* out_mask;  // presence mode: W words per record when non-null
  unsigned long long* n_out;
  uint64_t out_cap;
  unsigned long long* stats;  // [0] occurrences inserted, [1] distinct keys, [2] rounds, [3] splits
  uint32_t* status;
  uint32_t table_slots;       // hash-table slots per CTA
  int threads;
  int ctas;
  unsigned int* work_counter;
  float fill;                 // target fill of a round's table
  uint32_t chunk;             // windows per work item in the insert phase (COUNT_FAST_CHUNK for fast filtered rounds)
  uint32_t filter_words;      // > 0: two-pass rounds with a bitmap of this many u32 words (needs x >= 1)
  // k-mer windows one bucket may hold: the bin occupancies, their prefix and
  // the per-slot counts are 32-bit and each is bounded by the bucket's
  // windows; a bucket above this sets ST_COUNT_WIDTH and is not counted
  uint64_t max_bucket_windows;
  // fast filtered rounds: one word per window of a round, scratch_words per
  // CTA (a multiple of 4); nullptr keeps every filtered round on the slow path
  uint32_t* win_scratch;
  uint64_t scratch_words;
};
// Windows per chunk of the counting kernel's fast filtered rounds (4 or 8;
// a filtered count takes the fast rounds only with chunk equal to it).  A
// build may override it with -DMCZI_COUNT_FAST_CHUNK=n to measure the other.
#ifndef MCZI_COUNT_FAST_CHUNK
#define MCZI_COUNT_FAST_CHUNK 4
#endif
constexpr uint32_t COUNT_FAST_CHUNK = MCZI_COUNT_FAST_CHUNK;
static_assert(COUNT_FAST_CHUNK == 4 || COUNT_FAST_CHUNK == 8, "fast chunks hold 4 or 8 windows");
void launch_count(const CountArgs& a, cudaStream_t s);
size_t count_smem_bytes(int k, int mode, int n_datasets, uint32_t table_slots, uint32_t filter_words);
size_t count_fixed_smem_bytes(int mode, int n_datasets);
size_t count_slot_bytes(int k, int mode, int n_datasets);
size_t scan_smem_bytes();
size_t count_static_smem(int k, int mode);

}  // namespace mczi
