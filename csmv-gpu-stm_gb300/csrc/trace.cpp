// trace.cpp - on-disk bank streams and commit logs (include/csmv.h, csmv_stream_* / csmv_log_*),
// so a CPU run and a GPU run can replay identical inputs and a run's commit order can be kept
// and checked later. The reference keeps its generated keys as raw arrays in files named
// <name>_I<n>.bin without a header (memcachedGPU/keyGenAndCacheStore.cpp:151-182, storeArray /
// loadArray); these files carry a header and a checksum instead.
//
// Layout, all integers little-endian (written byte by byte, so the files are the same on every
// host):
//   stream  "CSMVSTRM" | u32 version = 1 | u32 n_txn | u64 n_addr | u64 checksum |
//           op[n_txn] u32 | off[n_txn] u32 | addr[n_addr] u32
//   log     "CSMVCLOG" | u32 version = 1 | u32 n_txn | u32 n_log | u32 base_ts | u64 checksum |
//           log_txn[n_log] u32 | outcome[n_txn] u32 | result[n_txn] i32
// The checksum is FNV-1a (64-bit) over the payload bytes. A file whose magic, version, size or
// checksum does not match is refused with CSMV_ERR_IO.
#include <cstdio>
#include <cstring>
#include <vector>

#include "common.h"

using namespace csmv;

namespace {

constexpr uint32_t kVersion = 1;
constexpr size_t kStreamHeader = 8 + 4 + 4 + 8 + 8;
constexpr size_t kLogHeader = 8 + 4 + 4 + 4 + 4 + 8;

struct Fnv {
  uint64_t h = 0xcbf29ce484222325ull;
  void add(const uint8_t* p, size_t n) {
    for (size_t i = 0; i < n; i++) {
      h ^= p[i];
      h *= 0x100000001b3ull;
    }
  }
};

void put32(uint8_t* p, uint32_t v) {
  for (int i = 0; i < 4; i++) p[i] = (uint8_t)(v >> (8 * i));
}
void put64(uint8_t* p, uint64_t v) {
  for (int i = 0; i < 8; i++) p[i] = (uint8_t)(v >> (8 * i));
}
uint32_t get32(const uint8_t* p) {
  uint32_t v = 0;
  for (int i = 0; i < 4; i++) v |= (uint32_t)p[i] << (8 * i);
  return v;
}
uint64_t get64(const uint8_t* p) {
  uint64_t v = 0;
  for (int i = 0; i < 8; i++) v |= (uint64_t)p[i] << (8 * i);
  return v;
}

struct File {
  std::FILE* f = nullptr;
  ~File() {
    if (f) std::fclose(f);
  }
};

csmv_status io_error(const char* what, const char* path) {
  set_error("%s: %s", what, path ? path : "(null)");
  return CSMV_ERR_IO;
}

// Writes `n` u32 words little-endian through a bounce buffer and folds them into the checksum.
bool write_words(std::FILE* f, const uint32_t* w, uint64_t n, Fnv* sum) {
  uint8_t buf[1 << 14];
  const uint64_t per = sizeof(buf) / 4;
  for (uint64_t i = 0; i < n; i += per) {
    const uint64_t k = n - i < per ? n - i : per;
    for (uint64_t j = 0; j < k; j++) put32(buf + 4 * j, w[i + j]);
    if (sum) sum->add(buf, 4 * k);
    if (f && std::fwrite(buf, 1, 4 * k, f) != 4 * k) return false;
  }
  return true;
}

bool read_words(std::FILE* f, uint32_t* w, uint64_t n, Fnv* sum) {
  uint8_t buf[1 << 14];
  const uint64_t per = sizeof(buf) / 4;
  for (uint64_t i = 0; i < n; i += per) {
    const uint64_t k = n - i < per ? n - i : per;
    if (std::fread(buf, 1, 4 * k, f) != 4 * k) return false;
    sum->add(buf, 4 * k);
    for (uint64_t j = 0; j < k; j++) w[i + j] = get32(buf + 4 * j);
  }
  return true;
}

long long file_size(std::FILE* f) {
  if (std::fseek(f, 0, SEEK_END) != 0) return -1;
  const long long n = std::ftell(f);
  if (std::fseek(f, 0, SEEK_SET) != 0) return -1;
  return n;
}

// Stream header checks (magic, version, size against the file's length).
csmv_status stream_header(std::FILE* f, const char* path, uint32_t* n_txn, uint64_t* n_addr,
                          uint64_t* sum) {
  uint8_t h[kStreamHeader];
  const long long size = file_size(f);
  if (size < (long long)kStreamHeader || std::fread(h, 1, kStreamHeader, f) != kStreamHeader)
    return io_error("not a stream file (too short)", path);
  if (std::memcmp(h, "CSMVSTRM", 8) != 0) return io_error("not a stream file (magic)", path);
  if (get32(h + 8) != kVersion) return io_error("stream file of another version", path);
  *n_txn = get32(h + 12);
  *n_addr = get64(h + 16);
  *sum = get64(h + 24);
  const unsigned long long want = kStreamHeader + 8ull * *n_txn + 4ull * *n_addr;
  if (*n_addr > (1ull << 40) || (unsigned long long)size != want)
    return io_error("stream file size does not match its header", path);
  return CSMV_OK;
}

csmv_status log_header(std::FILE* f, const char* path, uint32_t* n_txn, uint32_t* n_log,
                       uint32_t* base_ts, uint64_t* sum) {
  uint8_t h[kLogHeader];
  const long long size = file_size(f);
  if (size < (long long)kLogHeader || std::fread(h, 1, kLogHeader, f) != kLogHeader)
    return io_error("not a commit-log file (too short)", path);
  if (std::memcmp(h, "CSMVCLOG", 8) != 0) return io_error("not a commit-log file (magic)", path);
  if (get32(h + 8) != kVersion) return io_error("commit-log file of another version", path);
  *n_txn = get32(h + 12);
  *n_log = get32(h + 16);
  *base_ts = get32(h + 20);
  *sum = get64(h + 24);
  const unsigned long long want = kLogHeader + 4ull * *n_log + 8ull * *n_txn;
  if ((unsigned long long)size != want)
    return io_error("commit-log file size does not match its header", path);
  return CSMV_OK;
}

}  // namespace

extern "C" csmv_status csmv_stream_save(const char* path, const csmv_bank_stream* s) {
  if (!path || !s || (s->n_txn && (!s->op || !s->off)) || (s->n_addr && !s->addr))
    return CSMV_ERR_INVALID_ARG;
  Fnv sum;  // checksum first (one pass over the arrays), then the file
  write_words(nullptr, s->op, s->n_txn, &sum);
  write_words(nullptr, s->off, s->n_txn, &sum);
  write_words(nullptr, s->addr, s->n_addr, &sum);
  File f;
  if (!(f.f = std::fopen(path, "wb"))) return io_error("cannot create", path);
  uint8_t h[kStreamHeader];
  std::memcpy(h, "CSMVSTRM", 8);
  put32(h + 8, kVersion);
  put32(h + 12, s->n_txn);
  put64(h + 16, s->n_addr);
  put64(h + 24, sum.h);
  if (std::fwrite(h, 1, sizeof(h), f.f) != sizeof(h) || !write_words(f.f, s->op, s->n_txn, nullptr) ||
      !write_words(f.f, s->off, s->n_txn, nullptr) || !write_words(f.f, s->addr, s->n_addr, nullptr))
    return io_error("write failed", path);
  if (std::fclose(f.f) != 0) {
    f.f = nullptr;
    return io_error("write failed", path);
  }
  f.f = nullptr;
  return CSMV_OK;
}

extern "C" csmv_status csmv_stream_info(const char* path, uint32_t* n_txn, uint64_t* n_addr) {
  if (!path || !n_txn || !n_addr) return CSMV_ERR_INVALID_ARG;
  File f;
  if (!(f.f = std::fopen(path, "rb"))) return io_error("cannot open", path);
  uint64_t sum = 0;
  return stream_header(f.f, path, n_txn, n_addr, &sum);
}

extern "C" csmv_status csmv_stream_load(const char* path, uint32_t* op, uint32_t* off,
                                        uint32_t* addr, uint32_t n_txn_cap, uint64_t n_addr_cap) {
  if (!path) return CSMV_ERR_INVALID_ARG;
  File f;
  if (!(f.f = std::fopen(path, "rb"))) return io_error("cannot open", path);
  uint32_t n_txn = 0;
  uint64_t n_addr = 0, want = 0;
  csmv_status st = stream_header(f.f, path, &n_txn, &n_addr, &want);
  if (st != CSMV_OK) return st;
  if (n_txn > n_txn_cap || n_addr > n_addr_cap) {
    set_error("stream of %u transactions / %llu addresses; buffers hold %u / %llu", n_txn,
              (unsigned long long)n_addr, n_txn_cap, (unsigned long long)n_addr_cap);
    return CSMV_ERR_CAPACITY;
  }
  if ((n_txn && (!op || !off)) || (n_addr && !addr)) return CSMV_ERR_INVALID_ARG;
  Fnv sum;
  if (!read_words(f.f, op, n_txn, &sum) || !read_words(f.f, off, n_txn, &sum) ||
      !read_words(f.f, addr, n_addr, &sum))
    return io_error("read failed", path);
  if (sum.h != want) return io_error("stream file checksum mismatch", path);
  return CSMV_OK;
}

extern "C" csmv_status csmv_log_save(const char* path, uint32_t base_ts, const uint32_t* log_txn,
                                     uint32_t n_log, const uint32_t* outcome,
                                     const int32_t* result, uint32_t n_txn) {
  if (!path || (n_log && !log_txn) || (n_txn && (!outcome || !result))) return CSMV_ERR_INVALID_ARG;
  const uint32_t* res = reinterpret_cast<const uint32_t*>(result);
  Fnv sum;
  write_words(nullptr, log_txn, n_log, &sum);
  write_words(nullptr, outcome, n_txn, &sum);
  write_words(nullptr, res, n_txn, &sum);
  File f;
  if (!(f.f = std::fopen(path, "wb"))) return io_error("cannot create", path);
  uint8_t h[kLogHeader];
  std::memcpy(h, "CSMVCLOG", 8);
  put32(h + 8, kVersion);
  put32(h + 12, n_txn);
  put32(h + 16, n_log);
  put32(h + 20, base_ts);
  put64(h + 24, sum.h);
  if (std::fwrite(h, 1, sizeof(h), f.f) != sizeof(h) || !write_words(f.f, log_txn, n_log, nullptr) ||
      !write_words(f.f, outcome, n_txn, nullptr) || !write_words(f.f, res, n_txn, nullptr))
    return io_error("write failed", path);
  if (std::fclose(f.f) != 0) {
    f.f = nullptr;
    return io_error("write failed", path);
  }
  f.f = nullptr;
  return CSMV_OK;
}

extern "C" csmv_status csmv_log_info(const char* path, uint32_t* n_txn, uint32_t* n_log,
                                     uint32_t* base_ts) {
  if (!path || !n_txn || !n_log || !base_ts) return CSMV_ERR_INVALID_ARG;
  File f;
  if (!(f.f = std::fopen(path, "rb"))) return io_error("cannot open", path);
  uint64_t sum = 0;
  return log_header(f.f, path, n_txn, n_log, base_ts, &sum);
}

extern "C" csmv_status csmv_log_load(const char* path, uint32_t* log_txn, uint32_t n_log_cap,
                                     uint32_t* outcome, int32_t* result, uint32_t n_txn_cap) {
  if (!path) return CSMV_ERR_INVALID_ARG;
  File f;
  if (!(f.f = std::fopen(path, "rb"))) return io_error("cannot open", path);
  uint32_t n_txn = 0, n_log = 0, base = 0;
  uint64_t want = 0;
  csmv_status st = log_header(f.f, path, &n_txn, &n_log, &base, &want);
  if (st != CSMV_OK) return st;
  if (n_log > n_log_cap || n_txn > n_txn_cap) {
    set_error("commit log of %u timestamps / %u transactions; buffers hold %u / %u", n_log, n_txn,
              n_log_cap, n_txn_cap);
    return CSMV_ERR_CAPACITY;
  }
  if ((n_log && !log_txn) || (n_txn && (!outcome || !result))) return CSMV_ERR_INVALID_ARG;
  Fnv sum;
  if (!read_words(f.f, log_txn, n_log, &sum) || !read_words(f.f, outcome, n_txn, &sum) ||
      !read_words(f.f, reinterpret_cast<uint32_t*>(result), n_txn, &sum))
    return io_error("read failed", path);
  if (sum.h != want) return io_error("commit-log file checksum mismatch", path);
  return CSMV_OK;
}
