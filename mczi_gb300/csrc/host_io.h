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

// KFF file (src/lib.rs:1633-1670, 3071-3121).  count_size: 1, 4 or 8.
bool write_kff_file(const std::string& path, const HostRecords& r, int k, int m, uint64_t x, int count_size,
                    std::string* err);

// Greedy simplitig FASTA (src/lib.rs:1469-1533).  Returns false on I/O error.
bool write_simplitig_file(const std::string& path, const HostRecords& r, int k, std::string* err);

bool read_file(const std::string& path, std::vector<uint8_t>* out, std::string* err);

}  // namespace mczi
