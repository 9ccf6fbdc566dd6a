// host_io.cpp -- host-side output writers for libmczi_gpu.
//
// The reference formats its outputs on the host (src/lib.rs:1190-1676).
// Here the device produces the (canonical k-mer, count) records and, for KFF,
// also formats them as the file stores them (k_kff_records in mczi_api.cu);
// the host writes the KFF header, the values section and the raw section's
// header before those bytes and the trailer after them (write_kff_records),
// walks the simplitigs over the device's extension table
// (write_simplitig_walk), and keeps a self-contained simplitig writer for
// records already on the host (write_simplitig_file).
#include "host_io.h"

#include "../../include/mczi_gpu.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <thread>

namespace mczi {

namespace {

typedef unsigned __int128 u128;

struct File {
  FILE* f = nullptr;
  std::vector<uint8_t> buf;
  bool ok = true;
  explicit File(const std::string& p) : f(std::fopen(p.c_str(), "wb")) { buf.reserve(1 << 20); }
  ~File() { close(); }
  void put(const void* p, size_t n) {
    const uint8_t* b = static_cast<const uint8_t*>(p);
    buf.insert(buf.end(), b, b + n);
    if (buf.size() >= (1u << 20)) flush();
  }
  void put_u8(uint8_t v) { put(&v, 1); }
  void put_be(uint64_t v, int bytes) {
    uint8_t b[8];
    for (int i = 0; i < bytes; i++) b[i] = (uint8_t)(v >> (8 * (bytes - 1 - i)));
    put(b, (size_t)bytes);
  }
  void flush() {
    if (f && !buf.empty()) {
      if (std::fwrite(buf.data(), 1, buf.size(), f) != buf.size()) ok = false;
    }
    buf.clear();
  }
  bool close() {
    if (f) {
      flush();
      if (std::fclose(f) != 0) ok = false;
      f = nullptr;
    }
    return ok;
  }
};

inline u128 key_at(const HostRecords& r, size_t i) {
  return ((u128)(r.hi.empty() ? 0 : r.hi[i]) << 64) | r.lo[i];
}

inline uint64_t mix64(uint64_t x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ull;
  return x ^ (x >> 33);
}
inline uint64_t hash128(u128 k) { return mix64((uint64_t)k ^ mix64((uint64_t)(k >> 64) + 0x9e3779b97f4a7c15ull)); }

// open-addressing set with tombstone removal (keys are never re-inserted)
struct RemainingSet {
  std::vector<u128> keys;
  std::vector<uint8_t> state;  // 0 empty, 1 live, 2 removed
  uint64_t mask = 0;
  explicit RemainingSet(size_t n) {
    size_t c = 64;
    while (c < n * 2 + 64) c <<= 1;
    keys.assign(c, 0);
    state.assign(c, 0);
    mask = c - 1;
  }
  bool insert(u128 k) {
    uint64_t s = hash128(k) & mask;
    while (state[s] != 0) {
      if (keys[s] == k) return false;
      s = (s + 1) & mask;
    }
    keys[s] = k;
    state[s] = 1;
    return true;
  }
  bool remove(u128 k) {
    uint64_t s = hash128(k) & mask;
    while (state[s] != 0) {
      if (keys[s] == k) {
        if (state[s] == 1) { state[s] = 2; return true; }
        return false;
      }
      s = (s + 1) & mask;
    }
    return false;
  }
};

inline int code_of(char b) { return b == 'A' ? 0 : b == 'C' ? 1 : b == 'G' ? 2 : 3; }
inline char comp(char b) { return b == 'A' ? 'T' : b == 'C' ? 'G' : b == 'G' ? 'C' : 'A'; }

void revcomp(std::string& s) {
  std::reverse(s.begin(), s.end());
  for (char& c : s) c = comp(c);
}

u128 suffix_extension(const std::string& seq, int k, char base) {
  const u128 mask = k == 64 ? ~(u128)0 : (((u128)1 << (2 * k)) - 1);
  const int hs = 2 * (k - 1);
  u128 fwd = 0, rev = 0;
  for (size_t i = seq.size() - (size_t)(k - 1); i < seq.size(); i++) {
    const u128 b = (u128)code_of(seq[i]);
    fwd = ((fwd << 2) | b) & mask;
    rev = (rev >> 2) | ((b ^ 3) << hs);
  }
  const u128 b = (u128)code_of(base);
  fwd = ((fwd << 2) | b) & mask;
  rev = (rev >> 2) | ((b ^ 3) << hs);
  return fwd < rev ? fwd : rev;
}

void extend_forward(std::string& seq, int k, RemainingSet& rem) {
  static const char B[4] = {'A', 'C', 'G', 'T'};
  for (;;) {
    bool ext = false;
    for (char b : B) {
      if (rem.remove(suffix_extension(seq, k, b))) {
        seq.push_back(b);
        ext = true;
        break;
      }
    }
    if (!ext) return;
  }
}

}  // namespace

bool write_kff_records(const std::string& path, int k, int m, uint64_t x, int count_size, uint64_t n,
                       const uint8_t* rec, uint64_t rec_bytes, std::string* err) {
  File o(path);
  if (!o.f) {
    *err = "failed to create " + path;
    return false;
  }
  char fb[512];
  const int fbl = std::snprintf(fb, sizeof fb,
                                "producer=MC\nk=%d\nm=%d\nthreshold=%llu\nfilter=count>threshold\ncanonical=1\n", k, m,
                                (unsigned long long)x);
  o.put("KFF", 3);
  const uint8_t ver[5] = {1, 0, 0x1b, 1, 1};
  o.put(ver, 5);
  o.put_be((uint64_t)fbl, 4);
  o.put(fb, (size_t)fbl);
  o.put("v", 1);
  o.put_be(6, 8);
  const char* names[6] = {"k", "max", "data_size", "ordered", "m", "threshold"};
  const uint64_t vals[6] = {(uint64_t)k, 1, (uint64_t)count_size, 0, (uint64_t)m, x};
  for (int i = 0; i < 6; i++) {
    o.put(names[i], std::strlen(names[i]) + 1);
    o.put_be(vals[i], 8);
  }
  o.put("r", 1);
  o.put_be(n, 8);
  o.flush();
  if (o.f && rec_bytes && std::fwrite(rec, 1, rec_bytes, o.f) != rec_bytes) o.ok = false;
  o.put("KFF", 3);
  if (!o.close()) {
    *err = "failed to write " + path;
    return false;
  }
  return true;
}

namespace {

// decimal digits of v at p; returns the end
inline char* put_dec(char* p, uint64_t v) {
  char t[20];
  int n = 0;
  do {
    t[n++] = (char)('0' + v % 10);
    v /= 10;
  } while (v);
  while (n) *p++ = t[--n];
  return p;
}

// records [b, e) of the selected-k-mer FASTA into buf (enough room: 58 + k
// bytes a record: a header of at most 9 + 20 + 7 + 20 + 1, the bases and a
// newline); returns the bytes written
size_t format_kmer_records(char* buf, const uint64_t* lo, const uint64_t* hi, const uint64_t* count, uint64_t b,
                           uint64_t e, int k) {
  static const char B[4] = {'A', 'C', 'G', 'T'};
  char* p = buf;
  for (uint64_t i = b; i < e; i++) {
    std::memcpy(p, ">MC_kmer_", 9);
    p = put_dec(p + 9, i + 1);
    std::memcpy(p, " count=", 7);
    p = put_dec(p + 7, count[i]);
    *p++ = '\n';
    const u128 key = ((u128)(hi ? hi[i] : 0) << 64) | lo[i];
    for (int j = 0; j < k; j++) p[j] = B[(int)((key >> (2 * (k - 1 - j))) & 3)];
    p[k] = '\n';
    p += k + 1;
  }
  return (size_t)(p - buf);
}

}  // namespace

bool write_kmer_fasta(const std::string& path, const uint64_t* lo, const uint64_t* hi, const uint64_t* count,
                      uint64_t n, int k, std::string* err) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) {
    *err = "failed to create " + path;
    return false;
  }
  // blocks of records formatted on the host's threads, written in order
  const int threads = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  constexpr uint64_t PER = 1u << 17;  // records a thread formats per block
  const size_t cap = (size_t)PER * (58 + (size_t)k);
  std::vector<std::vector<char>> bufs((size_t)threads, std::vector<char>(n ? cap : 0));
  std::vector<size_t> len((size_t)threads);
  bool ok = true;
  for (uint64_t b0 = 0; b0 < n && ok; b0 += PER * (uint64_t)threads) {
    auto part = [&](int t) {
      const uint64_t b = std::min(n, b0 + PER * (uint64_t)t), e = std::min(n, b + PER);
      len[(size_t)t] = b < e ? format_kmer_records(bufs[(size_t)t].data(), lo, hi, count, b, e, k) : 0;
    };
    std::vector<std::thread> th;
    for (int t = 1; t < threads; t++) th.emplace_back(part, t);
    part(0);
    for (auto& x : th) x.join();
    for (int t = 0; t < threads && ok; t++)
      if (len[(size_t)t] && std::fwrite(bufs[(size_t)t].data(), 1, len[(size_t)t], f) != len[(size_t)t]) ok = false;
  }
  if (std::fclose(f) != 0) ok = false;
  if (!ok) {
    *err = "failed to write " + path;
    return false;
  }
  return true;
}

bool write_simplitig_file(const std::string& path, const HostRecords& r, int k, std::string* err) {
  File o(path);
  if (!o.f) {
    *err = "failed to create " + path;
    return false;
  }
  const size_t n = r.lo.size();
  RemainingSet rem(n);
  std::vector<u128> seeds;
  seeds.reserve(n);
  for (size_t i = 0; i < n; i++) {
    const u128 key = key_at(r, i);
    if (rem.insert(key)) seeds.push_back(key);
  }
  std::sort(seeds.begin(), seeds.end());
  static const char B[4] = {'A', 'C', 'G', 'T'};
  uint64_t idx = 0;
  std::string seq;
  char line[64];
  for (u128 seed : seeds) {
    if (!rem.remove(seed)) continue;
    seq.clear();
    for (int j = 0; j < k; j++) seq.push_back(B[(int)((seed >> (2 * (k - 1 - j))) & 3)]);
    extend_forward(seq, k, rem);
    revcomp(seq);
    extend_forward(seq, k, rem);
    revcomp(seq);
    idx++;
    const int l = std::snprintf(line, sizeof line, ">MC_simplitig_%llu kmers=%llu\n", (unsigned long long)idx,
                                (unsigned long long)(seq.size() - (size_t)k + 1));
    o.put(line, (size_t)l);
    for (size_t p = 0; p < seq.size(); p += 80) {
      const size_t len = std::min<size_t>(80, seq.size() - p);
      o.put(seq.data() + p, len);
      o.put_u8('\n');
    }
  }
  if (!o.close()) {
    *err = "failed to write " + path;
    return false;
  }
  return true;
}

void sorted_keys(const HostRecords& r, std::vector<uint64_t>* lo, std::vector<uint64_t>* hi, int threads) {
  const size_t n = r.lo.size();
  std::vector<u128> a(n), b(n);
  for (size_t i = 0; i < n; i++) a[i] = key_at(r, i);
  // chunks sorted in parallel, then merged pairwise (also in parallel)
  size_t parts = 1;
  while ((int)parts * 2 <= std::max(1, threads) && n / (parts * 2) >= (1u << 16)) parts *= 2;
  std::vector<size_t> cut(parts + 1);
  for (size_t p = 0; p <= parts; p++) cut[p] = n * p / parts;
  {
    std::vector<std::thread> th;
    for (size_t p = 0; p < parts; p++) th.emplace_back([&, p] { std::sort(a.begin() + cut[p], a.begin() + cut[p + 1]); });
    for (auto& t : th) t.join();
  }
  for (size_t w = 1; w < parts; w *= 2) {
    std::vector<std::thread> th;
    for (size_t p = 0; p < parts; p += 2 * w) {
      const size_t l = cut[p], m = cut[std::min(p + w, parts)], h = cut[std::min(p + 2 * w, parts)];
      th.emplace_back([&, l, m, h] { std::merge(a.begin() + l, a.begin() + m, a.begin() + m, a.begin() + h, b.begin() + l); });
    }
    for (auto& t : th) t.join();
    a.swap(b);
  }
  a.erase(std::unique(a.begin(), a.end()), a.end());
  lo->resize(a.size());
  hi->resize(a.size());
  for (size_t i = 0; i < a.size(); i++) {
    (*lo)[i] = (uint64_t)a[i];
    (*hi)[i] = (uint64_t)(a[i] >> 64);
  }
}

bool write_simplitig_walk(const std::string& path, const uint64_t* lo, const uint64_t* hi, uint64_t n, int k,
                          const uint32_t* ext, std::string* err) {
  File o(path);
  if (!o.f) {
    *err = "failed to create " + path;
    return false;
  }
  static const char B[4] = {'A', 'C', 'G', 'T'};
  std::vector<uint8_t> used_flags(n, 0);
  auto used = [&](uint64_t j) -> uint8_t& { return used_flags[j]; };
  std::string seq;
  char line[64];
  uint64_t idx = 0;
  // follows the extension table from (i, o), appending bases, marking k-mers used
  auto extend = [&](uint32_t i, uint32_t o) {
    for (;;) {
      const uint32_t* e = ext + (uint64_t)i * SIMPLITIG_STRIDE + o * 4;
      bool moved = false;
      for (int b = 0; b < 4; b++) {
        const uint32_t v = e[b];
        if (v == SIMPLITIG_NO_EXT) continue;
        const uint32_t j = v >> 1;
        if (used(j)) continue;
        used(j) = 1;
        seq.push_back(B[b]);
        i = j;
        o = v & 1u;
        moved = true;
        break;
      }
      if (!moved) return;
    }
  };
  for (uint64_t s = 0; s < n; s++) {
    if (used(s)) continue;
    used(s) = 1;
    const u128 seed = ((u128)hi[s] << 64) | lo[s];
    seq.clear();
    for (int j = 0; j < k; j++) seq.push_back(B[(int)((seed >> (2 * (k - 1 - j))) & 3)]);
    extend((uint32_t)s, 0);  // the path ends in the seed's canonical string
    revcomp(seq);
    extend((uint32_t)s, 1);  // reverse-complemented, it ends in the seed's reverse complement
    revcomp(seq);
    idx++;
    const int l = std::snprintf(line, sizeof line, ">MC_simplitig_%llu kmers=%llu\n", (unsigned long long)idx,
                                (unsigned long long)(seq.size() - (size_t)k + 1));
    o.put(line, (size_t)l);
    for (size_t p = 0; p < seq.size(); p += 80) {
      const size_t len = std::min<size_t>(80, seq.size() - p);
      o.put(seq.data() + p, len);
      o.put_u8('\n');
    }
  }
  if (!o.close()) {
    *err = "failed to write " + path;
    return false;
  }
  return true;
}

bool read_file(const std::string& path, std::vector<uint8_t>* out, std::string* err) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) {
    *err = "failed to open FASTA/FASTQ input " + path;
    return false;
  }
  out->clear();
  uint8_t buf[1 << 16];
  size_t got;
  while ((got = std::fread(buf, 1, sizeof buf, f)) > 0) out->insert(out->end(), buf, buf + got);
  const bool bad = std::ferror(f) != 0;
  std::fclose(f);
  if (bad) {
    *err = "failed to read " + path;
    return false;
  }
  return true;
}

}  // namespace mczi

extern "C" int32_t mczi_write_kmer_fasta(const char* path, const uint64_t* lo, const uint64_t* hi,
                                         const uint64_t* counts, uint64_t n, uint32_t k, char* err, uint64_t err_cap) {
  if (!path || k < 1 || k > 64 || (n && (!lo || !counts)) || (n && k > 32 && !hi)) return MCZI_ERR_INVALID_CONFIG;
  std::string e;
  if (!mczi::write_kmer_fasta(path, lo, k > 32 ? hi : nullptr, counts, n, (int)k, &e)) {
    if (err && err_cap) std::snprintf(err, err_cap, "%s", e.c_str());
    return MCZI_ERR_IO;
  }
  return MCZI_OK;
}
