// Compressed row output: gzip members compressed in parallel on host threads.
//
// The reference writes its rows as plain text (cas-offinder.cpp:450).  High-hit
// searches produce GBs of rows, so the CLI (output name ending in ".gz") and
// library callers can write them gzip-compressed instead.  The input is cut
// into blocks; each block is deflated on its own thread into one complete gzip
// member (RFC 1952), and the members are written in order.  A file of several
// members is one gzip file to gunzip, zcat and zlib (they read members back to
// back).  zlib is loaded at run time (libz.so.1), so the library neither needs
// its headers to build nor links it; without it the calls report
// COF_ERR_UNSUPPORTED.
#include <dlfcn.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <deque>
#include <future>
#include <string>
#include <thread>

#include "../../include/cof.h"

namespace {

// zlib's stream state, as its public interface defines it (zlib 1.x).
struct ZStream {
  const unsigned char* next_in;
  unsigned avail_in;
  unsigned long total_in;
  unsigned char* next_out;
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

constexpr int kZOk = 0, kZStreamEnd = 1, kZFinish = 4, kZDeflated = 8, kZDefaultStrategy = 0;
constexpr int kGzipWindow = 15 + 16;  // 32 KiB window, gzip wrapper
constexpr size_t kBlock = 8u << 20;

struct Zlib {
  int (*init2)(ZStream*, int, int, int, int, int, const char*, int) = nullptr;
  int (*deflate)(ZStream*, int) = nullptr;
  int (*end)(ZStream*) = nullptr;
  unsigned long (*bound)(ZStream*, unsigned long) = nullptr;
  const char* (*version)() = nullptr;
  bool ok = false;
  Zlib() {
    void* h = dlopen("libz.so.1", RTLD_NOW | RTLD_LOCAL);
    if (!h) h = dlopen("libz.so", RTLD_NOW | RTLD_LOCAL);
    if (!h) return;
    init2 = (decltype(init2))dlsym(h, "deflateInit2_");
    deflate = (decltype(deflate))dlsym(h, "deflate");
    end = (decltype(end))dlsym(h, "deflateEnd");
    bound = (decltype(bound))dlsym(h, "deflateBound");
    version = (decltype(version))dlsym(h, "zlibVersion");
    ok = init2 && deflate && end && bound && version;
  }
};

const Zlib& zlib() {
  static Zlib z;
  return z;
}

// One block -> one gzip member; empty string on failure.
std::string deflate_member(const std::string& in, int level) {
  const Zlib& z = zlib();
  ZStream s;
  std::memset(&s, 0, sizeof s);
  if (z.init2(&s, level, kZDeflated, kGzipWindow, 8, kZDefaultStrategy, z.version(), (int)sizeof(ZStream)) != kZOk)
    return std::string();
  std::string out(z.bound(&s, in.size()) + 64, '\0');
  s.next_in = (const unsigned char*)in.data();
  s.avail_in = (unsigned)in.size();
  s.next_out = (unsigned char*)&out[0];
  s.avail_out = (unsigned)out.size();
  const int r = z.deflate(&s, kZFinish);
  const size_t n = out.size() - s.avail_out;
  z.end(&s);
  if (r != kZStreamEnd) return std::string();
  out.resize(n);
  return out;
}

}  // namespace

struct cof_gzip {
  FILE* f = nullptr;
  int level = 1;
  unsigned threads = 1;
  std::string block;
  std::deque<std::future<std::string>> inflight;
  cof_status status = COF_OK;
};

namespace {

// Writes finished members in order until at most `keep` are in flight.
void drain(cof_gzip* z, size_t keep) {
  while (z->inflight.size() > keep) {
    const std::string m = z->inflight.front().get();
    z->inflight.pop_front();
    if (z->status != COF_OK) continue;
    if (m.empty()) z->status = COF_ERR_NOMEM;  // deflate failed: out of memory
    else if (fwrite(m.data(), 1, m.size(), z->f) != m.size()) z->status = COF_ERR_IO;
  }
}

void submit(cof_gzip* z) {
  if (z->block.empty()) return;
  drain(z, z->threads - 1);
  const int level = z->level;
  z->inflight.push_back(std::async(std::launch::async, [blk = std::move(z->block), level]() {
    return deflate_member(blk, level);
  }));
  z->block = std::string();
  z->block.reserve(kBlock);
}

}  // namespace

extern "C" {

cof_status cof_gzip_open(const char* path, int level, int threads, cof_gzip** out) {
  if (!path || !out) return COF_ERR_ARG;
  *out = nullptr;
  if (!zlib().ok) return COF_ERR_UNSUPPORTED;
  FILE* f = std::strcmp(path, "-") == 0 ? stdout : std::fopen(path, "wb");
  if (!f) return COF_ERR_IO;
  cof_gzip* z = new cof_gzip();
  z->f = f;
  z->level = level < 1 ? 1 : level > 9 ? 9 : level;
  unsigned hw = std::thread::hardware_concurrency();
  z->threads = threads > 0 ? (unsigned)threads : (hw ? hw : 4);
  z->block.reserve(kBlock);
  *out = z;
  return COF_OK;
}

cof_status cof_gzip_write(cof_gzip* z, const char* data, size_t len) {
  if (!z || (!data && len)) return COF_ERR_ARG;
  while (len) {
    const size_t take = std::min(len, kBlock - z->block.size());
    z->block.append(data, take);
    data += take;
    len -= take;
    if (z->block.size() == kBlock) submit(z);
  }
  return z->status;
}

int cof_gzip_write_fn(void* ctx, const char* data, size_t len) {
  return cof_gzip_write((cof_gzip*)ctx, data, len) == COF_OK ? 0 : 1;
}

cof_status cof_gzip_close(cof_gzip* z) {
  if (!z) return COF_ERR_ARG;
  submit(z);
  drain(z, 0);
  cof_status st = z->status;
  if (z->f != stdout) {
    if (std::fclose(z->f) != 0 && st == COF_OK) st = COF_ERR_IO;
  } else if (std::fflush(stdout) != 0 && st == COF_OK) {
    st = COF_ERR_IO;
  }
  delete z;
  return st;
}

}  // extern "C"
