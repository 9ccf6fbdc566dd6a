// host_io.h -- host-side writers of libmczi_gpu (KFF records, simplitig FASTA)
// and plain-file reading for the path-based entry points.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace mczi {

struct HostRecords {
  std::vector<uint64_t> lo, hi, count;  // hi empty for k <= 32
};

// KFF file (src/lib.rs:1633-1670, 3071-3121) around n records already laid
// out as the format stores them (rec_bytes = n x (ceil(k/4) + count_size)).
// count_size: 1, 4 or 8.
bool write_kff_records(const std::string& path, int k, int m, uint64_t x, int count_size, uint64_t n,
                       const uint8_t* rec, uint64_t rec_bytes, std::string* err);

// Selected k-mer FASTA (src/lib.rs:1535-1544): record i (from 1) is
// ">MC_kmer_<i> count=<count>" and the k-mer's bases on one line (k <= 64;
// the reference wraps at 80 columns).  hi may be null for k <= 32.
bool write_kmer_fasta(const std::string& path, const uint64_t* lo, const uint64_t* hi, const uint64_t* count,
                      uint64_t n, int k, std::string* err);

// Greedy simplitig FASTA (src/lib.rs:1469-1533).  Returns false on I/O error.
bool write_simplitig_file(const std::string& path, const HostRecords& r, int k, std::string* err);

// The same FASTA from the keys in ascending order (lo, hi; hi all 0 for k <= 32)
// and their extension table, SIMPLITIG_STRIDE words per key: ext[i *
// SIMPLITIG_STRIDE + o * 4 + b] = j << 1 | o' when k-mer i in orientation o
// (0: canonical string, 1: its reverse complement) followed by base b (A0 C1
// G2 T3) is k-mer j in orientation o', else SIMPLITIG_NO_EXT.  Byte-identical
// to write_simplitig_file.
constexpr uint32_t SIMPLITIG_NO_EXT = 0xffffffffu;
constexpr int SIMPLITIG_STRIDE = 8;
bool write_simplitig_walk(const std::string& path, const uint64_t* lo, const uint64_t* hi, uint64_t n, int k,
                          const uint32_t* ext, std::string* err);

// The distinct keys of r in ascending (hi, lo) order, sorted on up to
// `threads` host threads.
void sorted_keys(const HostRecords& r, std::vector<uint64_t>* lo, std::vector<uint64_t>* hi, int threads);

bool read_file(const std::string& path, std::vector<uint8_t>* out, std::string* err);

// Compressed inputs (decompress.cpp): the format is recognised by magic
// bytes; gzip, xz and zstd decode through the system's zlib, liblzma and
// libzstd, loaded at run time.
enum class InputFormat { Plain, Gzip, Xz, Zstd };
InputFormat input_format(const uint8_t* p, size_t n);
bool decompress_buffer(const std::vector<uint8_t>& in, std::vector<uint8_t>* out, const std::string& name,
                       std::string* err);
// One gzip member's DEFLATE data (offset and length in the buffer, header and
// trailer excluded) and its trailer (ISIZE, CRC-32).
struct GzSpan {
  uint64_t in_off;
  uint32_t in_len, out_len, crc;
};
// The members of a gzip buffer when every member carries its size in a BGZF
// "BC" extra subfield (so the boundaries are known without decoding), with
// their decoded total; false for any other buffer (then it is decoded on the
// host).  Zero bytes after the last member are allowed.
bool gzip_sized_members(const uint8_t* p, uint64_t n, std::vector<GzSpan>* members, uint64_t* out_total);
// a FASTA/FASTQ file, decompressed when it is gzip, xz or zstd; with
// keep_sized_gzip a gzip file whose members carry their sizes is returned as
// it is, for decoding on the device
bool read_input_file(const std::string& path, std::vector<uint8_t>* out, std::string* err,
                     bool keep_sized_gzip = false);
// several files, decoded on parallel host threads; the first failure's message
bool read_input_files(const char* const* paths, size_t n, std::vector<std::vector<uint8_t>>* out,
                      std::string* err, bool keep_sized_gzip = false);

}  // namespace mczi
