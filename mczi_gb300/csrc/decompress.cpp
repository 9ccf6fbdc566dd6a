// decompress.cpp -- reading FASTA/FASTQ inputs that are gzip, xz or zstd
// compressed, for the path-based entry points.
//
// MC and ZI accept compressed inputs (the reference's readers go through
// flate2, liblzma and zstd: src/lib.rs:3127-3143, 3218-3226, 1436-1447).  The
// format is recognised by its magic bytes (gzip 1f 8b, xz fd '7zXZ' 00,
// zstd 28 b5 2f fd), so a misnamed file still reads; anything else is read
// as plain text.  The decoders are the system's own zlib, liblzma and
// libzstd, loaded at run time (dlopen) through their stable C APIs, so the
// library builds without their headers; a missing library is reported by
// name (MCZI_ERR_IO) instead of failing the build or the load.
//
// Concatenated members (multi-member gzip, several xz streams, several zstd
// frames) decode in sequence, as flate2's MultiGzDecoder and liblzma's
// LZMA_CONCATENATED do.  Several input files decode on parallel host threads.
// A gzip file whose members all carry their compressed size (BGZF) can
// instead be returned as it is (keep_sized_gzip) and decoded on the device
// (inflate.cu); the path-based entry points do that.
//
// The same libraries compress outputs (mczi_compress_output): MC's output
// writer picks gzip, xz or zstd by the output's extension.
#include "host_io.h"
#include "../../include/mczi_gpu.h"

#include <dlfcn.h>

#include <algorithm>
#include <atomic>
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <thread>

namespace mczi {

namespace {

// ------------------------------------------------------------ zlib (gzip)
// z_stream as declared by zlib's public header (LP64: uLong is 64 bits)
struct ZStream {
  const uint8_t* next_in;
  unsigned avail_in;
  unsigned long total_in;
  uint8_t* next_out;
  unsigned avail_out;
  unsigned long total_out;
  const char* msg;
  void* state;
  void* zalloc;
  void* zfree;
  void* opaque;
  int data_type;
  unsigned long adler;
  unsigned long reserved;
};
constexpr int Z_OK = 0, Z_STREAM_END = 1, Z_BUF_ERROR = -5, Z_NO_FLUSH = 0, Z_FINISH = 4, Z_DEFLATED = 8;

struct ZLib {
  bool ok = false;
  const char* (*version)() = nullptr;
  int (*init2)(ZStream*, int, const char*, int) = nullptr;
  int (*inflate)(ZStream*, int) = nullptr;
  int (*reset)(ZStream*) = nullptr;
  int (*end)(ZStream*) = nullptr;
  // encoder (outputs)
  bool enc = false;
  int (*dinit2)(ZStream*, int, int, int, int, int, const char*, int) = nullptr;
  int (*deflate)(ZStream*, int) = nullptr;
  int (*dend)(ZStream*) = nullptr;
};

// ------------------------------------------------------------ liblzma (xz)
// lzma_stream as declared by liblzma's public header (LZMA_STREAM_INIT is
// all zeros)
struct LzmaStream {
  const uint8_t* next_in;
  size_t avail_in;
  uint64_t total_in;
  uint8_t* next_out;
  size_t avail_out;
  uint64_t total_out;
  const void* allocator;
  void* internal;
  void* reserved_ptr[4];
  uint64_t reserved_int1, reserved_int2;
  size_t reserved_int3, reserved_int4;
  int reserved_enum1, reserved_enum2;
};
constexpr int LZMA_OK = 0, LZMA_STREAM_END = 1, LZMA_RUN = 0, LZMA_FINISH = 3;
constexpr uint32_t LZMA_CONCATENATED = 0x08;
constexpr int LZMA_CHECK_CRC64 = 4;

struct Lzma {
  bool ok = false;
  int (*stream_decoder)(LzmaStream*, uint64_t, uint32_t) = nullptr;
  int (*code)(LzmaStream*, int) = nullptr;
  void (*end)(LzmaStream*) = nullptr;
  int (*easy_encoder)(LzmaStream*, uint32_t, int) = nullptr;  // outputs
};

// ------------------------------------------------------------ libzstd
struct ZstdIn {
  const void* src;
  size_t size, pos;
};
struct ZstdOut {
  void* dst;
  size_t size, pos;
};
struct Zstd {
  bool ok = false;
  void* (*create)() = nullptr;
  size_t (*init)(void*) = nullptr;
  size_t (*decompress)(void*, ZstdOut*, ZstdIn*) = nullptr;
  size_t (*free_ds)(void*) = nullptr;
  unsigned (*is_error)(size_t) = nullptr;
  const char* (*error_name)(size_t) = nullptr;
  // one-shot encoder (outputs)
  size_t (*bound)(size_t) = nullptr;
  size_t (*compress)(void*, size_t, const void*, size_t, int) = nullptr;
};

void* open_any(const char* const* names) {
  for (int i = 0; names[i]; i++)
    if (void* h = dlopen(names[i], RTLD_NOW | RTLD_LOCAL)) return h;
  return nullptr;
}

template <class F>
bool sym(void* h, const char* name, F* out) {
  *out = reinterpret_cast<F>(dlsym(h, name));
  return *out != nullptr;
}

std::once_flag g_once;
ZLib g_z;
Lzma g_x;
Zstd g_zs;

void load_decoders() {
  static const char* zn[] = {"libz.so.1", "libz.so", nullptr};
  static const char* xn[] = {"liblzma.so.5", "liblzma.so", nullptr};
  static const char* sn[] = {"libzstd.so.1", "libzstd.so", nullptr};
  if (void* h = open_any(zn)) {
    g_z.ok = sym(h, "zlibVersion", &g_z.version) && sym(h, "inflateInit2_", &g_z.init2) &&
             sym(h, "inflate", &g_z.inflate) && sym(h, "inflateReset", &g_z.reset) && sym(h, "inflateEnd", &g_z.end);
    g_z.enc = g_z.ok && sym(h, "deflateInit2_", &g_z.dinit2) && sym(h, "deflate", &g_z.deflate) &&
              sym(h, "deflateEnd", &g_z.dend);
  }
  if (void* h = open_any(xn)) {
    g_x.ok = sym(h, "lzma_stream_decoder", &g_x.stream_decoder) && sym(h, "lzma_code", &g_x.code) &&
             sym(h, "lzma_end", &g_x.end);
    sym(h, "lzma_easy_encoder", &g_x.easy_encoder);
  }
  if (void* h = open_any(sn)) {
    g_zs.ok = sym(h, "ZSTD_createDStream", &g_zs.create) && sym(h, "ZSTD_initDStream", &g_zs.init) &&
              sym(h, "ZSTD_decompressStream", &g_zs.decompress) && sym(h, "ZSTD_freeDStream", &g_zs.free_ds) &&
              sym(h, "ZSTD_isError", &g_zs.is_error) && sym(h, "ZSTD_getErrorName", &g_zs.error_name);
    sym(h, "ZSTD_compressBound", &g_zs.bound);
    sym(h, "ZSTD_compress", &g_zs.compress);
  }
}

// output grows in steps; `hint` is an estimate of the decompressed size
void grow(std::vector<uint8_t>* out, size_t used, size_t hint) {
  if (out->size() - used >= (1u << 20)) return;
  size_t want = std::max<size_t>(out->size() + out->size() / 2, used + (4u << 20));
  want = std::max(want, hint);
  out->resize(want);
}

bool gunzip(const std::vector<uint8_t>& in, std::vector<uint8_t>* out, const std::string& path, std::string* err) {
  if (!g_z.ok) {
    *err = "gzip input " + path + " needs zlib (libz.so.1), which could not be loaded";
    return false;
  }
  ZStream zs;
  std::memset(&zs, 0, sizeof zs);
  // 15 + 32: 32 KiB window, gzip or zlib header detected
  if (g_z.init2(&zs, 15 + 32, g_z.version(), (int)sizeof(ZStream)) != Z_OK) {
    *err = "zlib could not start a decoder for " + path;
    return false;
  }
  // ISIZE (size mod 2^32 of the last member) as a first size estimate
  size_t hint = in.size() * 4;
  if (in.size() >= 4) {
    uint32_t isz;
    std::memcpy(&isz, in.data() + in.size() - 4, 4);
    if (isz > in.size()) hint = isz;
  }
  size_t used = 0, pos = 0;
  out->clear();
  bool ok = true;
  for (;;) {
    grow(out, used, hint);
    const size_t in_chunk = std::min<size_t>(in.size() - pos, 1u << 30);
    const size_t out_chunk = std::min<size_t>(out->size() - used, 1u << 30);
    zs.next_in = in.data() + pos;
    zs.avail_in = (unsigned)in_chunk;
    zs.next_out = out->data() + used;
    zs.avail_out = (unsigned)out_chunk;
    const int rc = g_z.inflate(&zs, Z_NO_FLUSH);
    pos += in_chunk - zs.avail_in;
    used += out_chunk - zs.avail_out;
    if (rc == Z_STREAM_END) {
      // another member may follow (trailing zero padding is skipped)
      while (pos < in.size() && in[pos] == 0) pos++;
      if (pos >= in.size()) break;
      g_z.reset(&zs);
      continue;
    }
    if (rc != Z_OK && rc != Z_BUF_ERROR) {
      *err = std::string("gzip input ") + path + " is corrupt: " + (zs.msg ? zs.msg : "inflate failed");
      ok = false;
      break;
    }
    if (zs.avail_out == 0) continue;  // more output pending: grow and go on
    if (pos >= in.size()) {
      *err = "gzip input " + path + " is truncated";
      ok = false;
      break;
    }
  }
  g_z.end(&zs);
  out->resize(used);
  return ok;
}

bool unxz(const std::vector<uint8_t>& in, std::vector<uint8_t>* out, const std::string& path, std::string* err) {
  if (!g_x.ok) {
    *err = "xz input " + path + " needs liblzma (liblzma.so.5), which could not be loaded";
    return false;
  }
  LzmaStream s;
  std::memset(&s, 0, sizeof s);
  if (g_x.stream_decoder(&s, UINT64_MAX, LZMA_CONCATENATED) != LZMA_OK) {
    *err = "liblzma could not start a decoder for " + path;
    return false;
  }
  s.next_in = in.data();
  s.avail_in = in.size();
  size_t used = 0;
  out->clear();
  bool ok = true;
  for (;;) {
    grow(out, used, in.size() * 5);
    s.next_out = out->data() + used;
    s.avail_out = out->size() - used;
    const size_t before = s.avail_out;
    const int rc = g_x.code(&s, s.avail_in ? LZMA_RUN : LZMA_FINISH);
    used += before - s.avail_out;
    if (rc == LZMA_STREAM_END) break;
    if (rc != LZMA_OK) {
      *err = "xz input " + path + " is corrupt or truncated (liblzma error " + std::to_string(rc) + ")";
      ok = false;
      break;
    }
  }
  g_x.end(&s);
  out->resize(used);
  return ok;
}

bool unzstd(const std::vector<uint8_t>& in, std::vector<uint8_t>* out, const std::string& path, std::string* err) {
  if (!g_zs.ok) {
    *err = "zstd input " + path + " needs libzstd (libzstd.so.1), which could not be loaded";
    return false;
  }
  void* ds = g_zs.create();
  if (!ds || g_zs.is_error(g_zs.init(ds))) {
    if (ds) g_zs.free_ds(ds);
    *err = "libzstd could not start a decoder for " + path;
    return false;
  }
  ZstdIn zi{in.data(), in.size(), 0};
  size_t used = 0, last = 0;
  out->clear();
  bool ok = true;
  while (zi.pos < zi.size) {
    grow(out, used, in.size() * 4);
    ZstdOut zo{out->data() + used, out->size() - used, 0};
    last = g_zs.decompress(ds, &zo, &zi);
    used += zo.pos;
    if (g_zs.is_error(last)) {
      *err = std::string("zstd input ") + path + " is corrupt: " + g_zs.error_name(last);
      ok = false;
      break;
    }
  }
  // flush what the decoder still holds for the last frame
  while (ok && last != 0) {
    grow(out, used, 0);
    ZstdOut zo{out->data() + used, out->size() - used, 0};
    const size_t before = zo.pos;
    last = g_zs.decompress(ds, &zo, &zi);
    used += zo.pos;
    if (g_zs.is_error(last)) {
      *err = std::string("zstd input ") + path + " is corrupt: " + g_zs.error_name(last);
      ok = false;
    } else if (last != 0 && zo.pos == before) {
      *err = "zstd input " + path + " is truncated";
      ok = false;
    }
  }
  g_zs.free_ds(ds);
  out->resize(used);
  return ok;
}

// ------------------------------------------------------------ outputs
// MC's output writer (src/lib.rs:1355-1405): gzip at the fast level, xz at
// preset 6 with a CRC64 check, zstd at level 1, chosen by the extension.
enum class OutputCodec { Plain, Gzip, Xz, Zstd };

OutputCodec output_codec(const std::string& path) {
  const size_t slash = path.find_last_of('/');
  const size_t dot = path.find_last_of('.');
  if (dot == std::string::npos || (slash != std::string::npos && dot < slash)) return OutputCodec::Plain;
  std::string ext = path.substr(dot + 1);
  for (char& c : ext) c = (char)std::tolower((unsigned char)c);
  if (ext == "gz" || ext == "gzip") return OutputCodec::Gzip;
  if (ext == "xz") return OutputCodec::Xz;
  if (ext == "zst" || ext == "zstd") return OutputCodec::Zstd;
  return OutputCodec::Plain;
}

bool gzip_encode(const std::vector<uint8_t>& in, std::vector<uint8_t>* out, std::string* err) {
  if (!g_z.enc) {
    *err = "gzip output needs zlib (libz.so.1), which could not be loaded";
    return false;
  }
  ZStream zs;
  std::memset(&zs, 0, sizeof zs);
  // level 1, 15 + 16: 32 KiB window with a gzip wrapper, memLevel 8, default strategy
  if (g_z.dinit2(&zs, 1, Z_DEFLATED, 15 + 16, 8, 0, g_z.version(), (int)sizeof(ZStream)) != Z_OK) {
    *err = "zlib could not start an encoder";
    return false;
  }
  size_t used = 0, pos = 0;
  out->clear();
  bool ok = true;
  for (;;) {
    grow(out, used, in.size() / 2);
    const size_t in_chunk = std::min<size_t>(in.size() - pos, 1u << 30);
    const size_t out_chunk = std::min<size_t>(out->size() - used, 1u << 30);
    zs.next_in = in.data() + pos;
    zs.avail_in = (unsigned)in_chunk;
    zs.next_out = out->data() + used;
    zs.avail_out = (unsigned)out_chunk;
    const int rc = g_z.deflate(&zs, pos + in_chunk == in.size() ? Z_FINISH : Z_NO_FLUSH);
    pos += in_chunk - zs.avail_in;
    used += out_chunk - zs.avail_out;
    if (rc == Z_STREAM_END) break;
    if (rc != Z_OK && rc != Z_BUF_ERROR) {
      *err = "zlib failed to compress (error " + std::to_string(rc) + ")";
      ok = false;
      break;
    }
  }
  g_z.dend(&zs);
  out->resize(used);
  return ok;
}

bool xz_encode(const std::vector<uint8_t>& in, std::vector<uint8_t>* out, std::string* err) {
  if (!g_x.ok || !g_x.easy_encoder) {
    *err = "xz output needs liblzma (liblzma.so.5), which could not be loaded";
    return false;
  }
  LzmaStream s;
  std::memset(&s, 0, sizeof s);
  if (g_x.easy_encoder(&s, 6, LZMA_CHECK_CRC64) != LZMA_OK) {
    *err = "liblzma could not start an encoder";
    return false;
  }
  s.next_in = in.data();
  s.avail_in = in.size();
  size_t used = 0;
  out->clear();
  bool ok = true;
  for (;;) {
    grow(out, used, in.size() / 3);
    s.next_out = out->data() + used;
    s.avail_out = out->size() - used;
    const size_t before = s.avail_out;
    const int rc = g_x.code(&s, LZMA_FINISH);  // all input is given: finish from the first call
    used += before - s.avail_out;
    if (rc == LZMA_STREAM_END) break;
    if (rc != LZMA_OK) {
      *err = "liblzma failed to compress (error " + std::to_string(rc) + ")";
      ok = false;
      break;
    }
  }
  g_x.end(&s);
  out->resize(used);
  return ok;
}

bool zstd_encode(const std::vector<uint8_t>& in, std::vector<uint8_t>* out, std::string* err) {
  if (!g_zs.ok || !g_zs.bound || !g_zs.compress) {
    *err = "zstd output needs libzstd (libzstd.so.1), which could not be loaded";
    return false;
  }
  out->resize(g_zs.bound(in.size()));
  const size_t n = g_zs.compress(out->data(), out->size(), in.data(), in.size(), 1);
  if (g_zs.is_error(n)) {
    *err = std::string("libzstd failed to compress: ") + g_zs.error_name(n);
    return false;
  }
  out->resize(n);
  return true;
}

}  // namespace

InputFormat input_format(const uint8_t* p, size_t n) {
  if (n >= 2 && p[0] == 0x1f && p[1] == 0x8b) return InputFormat::Gzip;
  if (n >= 6 && p[0] == 0xfd && p[1] == '7' && p[2] == 'z' && p[3] == 'X' && p[4] == 'Z' && p[5] == 0)
    return InputFormat::Xz;
  if (n >= 4 && p[0] == 0x28 && p[1] == 0xb5 && p[2] == 0x2f && p[3] == 0xfd) return InputFormat::Zstd;
  return InputFormat::Plain;
}

bool decompress_buffer(const std::vector<uint8_t>& in, std::vector<uint8_t>* out, const std::string& name,
                       std::string* err) {
  std::call_once(g_once, load_decoders);
  switch (input_format(in.data(), in.size())) {
    case InputFormat::Gzip: return gunzip(in, out, name, err);
    case InputFormat::Xz: return unxz(in, out, name, err);
    case InputFormat::Zstd: return unzstd(in, out, name, err);
    default: *out = in; return true;
  }
}

// RFC 1952 member layout: 10-byte header (magic, CM = 8, FLG, MTIME, XFL,
// OS), optional FEXTRA (XLEN, subfields SI1 SI2 SLEN data), FNAME and
// FCOMMENT (zero-terminated), FHCRC (2 bytes), the DEFLATE data, then CRC-32
// and ISIZE.  BGZF puts the member size minus one in subfield 'B' 'C'.
bool gzip_sized_members(const uint8_t* p, uint64_t n, std::vector<GzSpan>* members, uint64_t* out_total) {
  members->clear();
  uint64_t pos = 0, total = 0;
  auto u16 = [&](uint64_t at) { return (uint32_t)p[at] | ((uint32_t)p[at + 1] << 8); };
  auto u32 = [&](uint64_t at) { return u16(at) | (u16(at + 2) << 16); };
  while (pos < n) {
    if (p[pos] == 0) {  // zero padding after the last member
      for (uint64_t i = pos; i < n; i++)
        if (p[i] != 0) return false;
      break;
    }
    if (n - pos < 18 || p[pos] != 0x1f || p[pos + 1] != 0x8b || p[pos + 2] != 8) return false;
    const uint32_t flg = p[pos + 3];
    if (!(flg & 4u)) return false;  // no extra field: no size
    uint64_t h = pos + 10;
    const uint32_t xlen = u16(h);
    h += 2;
    if (h + xlen > n) return false;
    uint64_t bsize = 0;
    bool have = false;
    for (uint64_t f = h; f + 4 <= h + xlen;) {
      const uint32_t slen = u16(f + 2);
      if (f + 4 + slen > h + xlen) return false;
      if (p[f] == 'B' && p[f + 1] == 'C' && slen == 2) {
        bsize = u16(f + 4);
        have = true;
      }
      f += 4 + slen;
    }
    if (!have) return false;
    h += xlen;
    const uint64_t end = pos + bsize + 1;
    if (end > n) return false;
    for (uint32_t bit : {8u, 16u}) {  // FNAME, FCOMMENT
      if (flg & bit) {
        while (h < end && p[h] != 0) h++;
        h++;
      }
    }
    if (flg & 2u) h += 2;  // FHCRC
    if (h + 8 > end) return false;
    GzSpan m;
    m.in_off = h;
    m.in_len = (uint32_t)(end - 8 - h);
    m.crc = u32(end - 8);
    m.out_len = u32(end - 4);
    total += m.out_len;
    members->push_back(m);
    pos = end;
  }
  if (members->empty()) return false;
  *out_total = total;
  return true;
}

bool read_input_file(const std::string& path, std::vector<uint8_t>* out, std::string* err, bool keep_sized_gzip) {
  std::vector<uint8_t> raw;
  if (!read_file(path, &raw, err)) return false;
  const InputFormat f = input_format(raw.data(), raw.size());
  if (f == InputFormat::Plain) {
    out->swap(raw);
    return true;
  }
  if (keep_sized_gzip && f == InputFormat::Gzip) {
    std::vector<GzSpan> m;
    uint64_t total = 0;
    if (gzip_sized_members(raw.data(), raw.size(), &m, &total)) {
      out->swap(raw);
      return true;
    }
  }
  return decompress_buffer(raw, out, path, err);
}

bool read_input_files(const char* const* paths, size_t n, std::vector<std::vector<uint8_t>>* out,
                      std::string* err, bool keep_sized_gzip) {
  out->assign(n, {});
  std::vector<std::string> errs(n);
  std::vector<char> ok(n, 1);
  std::atomic<size_t> next{0};
  const size_t hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t nt = std::min(n, hw);
  auto work = [&]() {
    for (size_t i; (i = next.fetch_add(1)) < n;)
      ok[i] = read_input_file(paths[i], &(*out)[i], &errs[i], keep_sized_gzip) ? 1 : 0;
  };
  std::vector<std::thread> th;
  for (size_t t = 1; t < nt; t++) th.emplace_back(work);
  work();
  for (auto& t : th) t.join();
  for (size_t i = 0; i < n; i++)
    if (!ok[i]) {
      *err = errs[i];
      return false;
    }
  return true;
}

}  // namespace mczi

extern "C" {

int32_t mczi_read_input_file(const char* path, uint8_t** data, uint64_t* len, char* err, uint64_t err_cap) {
  if (!path || !data || !len) return MCZI_ERR_INVALID_CONFIG;
  *data = nullptr;
  *len = 0;
  std::vector<uint8_t> buf;
  std::string e;
  if (!mczi::read_input_file(path, &buf, &e)) {
    if (err && err_cap) std::snprintf(err, err_cap, "%s", e.c_str());
    return MCZI_ERR_IO;
  }
  uint8_t* p = static_cast<uint8_t*>(std::malloc(buf.size() ? buf.size() : 1));
  if (!p) return MCZI_ERR_OOM;
  if (!buf.empty()) std::memcpy(p, buf.data(), buf.size());
  *data = p;
  *len = buf.size();
  return MCZI_OK;
}

void mczi_free_input(uint8_t* data) { std::free(data); }

int32_t mczi_compress_output(const char* plain_path, const char* output_path, char* err, uint64_t err_cap) {
  if (!plain_path || !output_path) return MCZI_ERR_INVALID_CONFIG;
  std::call_once(mczi::g_once, mczi::load_decoders);
  std::string e;
  std::vector<uint8_t> plain, packed;
  auto fail = [&](const std::string& m) {
    if (err && err_cap) std::snprintf(err, err_cap, "%s", m.c_str());
    return MCZI_ERR_IO;
  };
  FILE* f = std::fopen(plain_path, "rb");
  if (!f) return fail(std::string("failed to open ") + plain_path);
  uint8_t buf[1 << 16];
  size_t got;
  while ((got = std::fread(buf, 1, sizeof buf, f)) > 0) plain.insert(plain.end(), buf, buf + got);
  const bool bad = std::ferror(f) != 0;
  std::fclose(f);
  if (bad) return fail(std::string("failed to read ") + plain_path);
  const std::vector<uint8_t>* data = &plain;
  bool ok = true;
  switch (mczi::output_codec(output_path)) {
    case mczi::OutputCodec::Gzip: ok = mczi::gzip_encode(plain, &packed, &e); data = &packed; break;
    case mczi::OutputCodec::Xz: ok = mczi::xz_encode(plain, &packed, &e); data = &packed; break;
    case mczi::OutputCodec::Zstd: ok = mczi::zstd_encode(plain, &packed, &e); data = &packed; break;
    case mczi::OutputCodec::Plain: break;
  }
  if (!ok) return fail(e);
  FILE* o = std::fopen(output_path, "wb");
  if (!o) return fail(std::string("failed to create ") + output_path);
  const bool wrote = data->empty() || std::fwrite(data->data(), 1, data->size(), o) == data->size();
  if (std::fclose(o) != 0 || !wrote) return fail(std::string("failed to compress ") + output_path);
  return MCZI_OK;
}

}  // extern "C"
