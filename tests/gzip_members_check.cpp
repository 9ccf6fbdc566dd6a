// Host check of gzip_sized_members (csrc/decompress.cpp): reads one file and
// prints "members <n> total <bytes>" and one "m <in_off> <in_len> <out_len>
// <crc>" line per member, or "none" when the buffer is not a gzip buffer
// whose members carry their sizes.  Built with decompress.cpp by
// tests/test_gzip_members.py (read_file is provided here).
#include <cstdio>
#include <string>
#include <vector>

#include "host_io.h"

namespace mczi {
bool read_file(const std::string& path, std::vector<uint8_t>* out, std::string* err) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) {
    *err = "cannot open " + path;
    return false;
  }
  out->clear();
  uint8_t buf[65536];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) out->insert(out->end(), buf, buf + n);
  std::fclose(f);
  return true;
}
}  // namespace mczi

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  std::vector<uint8_t> data;
  std::string err;
  if (!mczi::read_file(argv[1], &data, &err)) return 2;
  std::vector<mczi::GzSpan> m;
  uint64_t total = 0;
  if (!mczi::gzip_sized_members(data.data(), data.size(), &m, &total)) {
    std::printf("none\n");
    return 0;
  }
  std::printf("members %zu total %llu\n", m.size(), (unsigned long long)total);
  for (const auto& s : m)
    std::printf("m %llu %u %u %u\n", (unsigned long long)s.in_off, s.in_len, s.out_len, s.crc);
  return 0;
}
