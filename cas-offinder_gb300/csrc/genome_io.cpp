// Genome loaders: FASTA and 2BIT files to resident-ready bit planes.
//
// Byte semantics follow the reference loaders exactly:
//   load_fasta   read_fasta (read_fasta.cpp:11-58): the first byte must be
//                '>'; a trailing '\r' is cut from each non-empty line; header
//                lines give record names (text after '>'); sequence lines are
//                upper-cased (soft mask dropped) and appended; a ';' separates
//                consecutive records; symlinks are resolved with readlink.
//   load_twobit  read_twobit (read_twobit.cpp:44-131): magic 0x1A412743,
//                N blocks become 'N', mask blocks are skipped, ';' between
//                records.  Beyond the reference (which reads host-order
//                version 0 files and ignores the index offsets, reading the
//                records back to back): each record is read at its index
//                offset (the same bytes for files laid out back to back),
//                version 1 files (64-bit offsets) and files of the other byte
//                order are accepted.
// 2BIT data is converted code for code (its T,C,A,G = 0..3 is the plane code),
// without expanding to one byte per base.
#include <unistd.h>

#include <climits>
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <thread>

#include "cof_internal.h"

namespace cof {

namespace {

// Per-byte plane bits: bit0 = lo, bit1 = hi, bit2 = ot, bit3 = exception.
struct CodeTable {
  uint8_t c[256];
  CodeTable() {
    for (int b = 0; b < 256; ++b) c[b] = 4 | 2 | 8;  // other byte: ot=1, (hi,lo)=10, exception
    c[(unsigned char)'T'] = 0;
    c[(unsigned char)'C'] = 1;
    c[(unsigned char)'A'] = 2;
    c[(unsigned char)'G'] = 3;
    c[(unsigned char)'N'] = 4;
    c[(unsigned char)';'] = 4 | 1;
  }
};
const CodeTable kCodes;

unsigned worker_count(uint64_t work) {
  unsigned hw = std::thread::hardware_concurrency();
  if (hw == 0) hw = 4;
  uint64_t cap = work / (1u << 20) + 1;  // at least ~1M items per thread
  return (unsigned)std::min<uint64_t>(hw, cap);
}

std::string resolve(const std::string& path) {
  char buf[PATH_MAX + 1];
  std::memset(buf, 0, sizeof buf);
  ssize_t n = readlink(path.c_str(), buf, PATH_MAX);
  return n >= 0 ? std::string(buf) : path;
}

}  // namespace

void pad_planes(uint64_t n, uint32_t* hi, uint32_t* lo, uint32_t* ot) {
  const uint64_t words = plane_words(n);
  for (uint64_t w = n / 32; w < words; ++w) {
    const uint64_t base = w * 32;
    const uint32_t keep = base >= n ? 0u : ((1u << (n - base)) - 1);  // 0 < n - base < 32 here
    hi[w] &= keep;
    lo[w] = (lo[w] & keep) | ~keep;
    ot[w] = (ot[w] & keep) | ~keep;
  }
}

void pack_text(const char* seq, uint64_t n, uint32_t* hi, uint32_t* lo, uint32_t* ot, std::vector<uint64_t>* exc_pos,
               std::vector<uint8_t>* exc_byte) {
  const uint64_t full = n / 32 + ((n & 31) ? 1 : 0);
  const unsigned T = worker_count(full * 32);
  std::vector<std::vector<uint64_t>> epos(T);
  std::vector<std::vector<uint8_t>> ebyte(T);
  auto work = [&](unsigned t) {
    const uint64_t w0 = full * t / T, w1 = full * (t + 1) / T;
    for (uint64_t w = w0; w < w1; ++w) {
      uint32_t h = 0, l = 0, o = 0, e = 0;
      const uint64_t base = w * 32;
      const unsigned m = (unsigned)std::min<uint64_t>(32, n - base);
      for (unsigned b = 0; b < m; ++b) {
        const uint8_t c = kCodes.c[(unsigned char)seq[base + b]];
        l |= (uint32_t)(c & 1) << b;
        h |= (uint32_t)((c >> 1) & 1) << b;
        o |= (uint32_t)((c >> 2) & 1) << b;
        e |= (uint32_t)((c >> 3) & 1) << b;
      }
      hi[w] = h;
      lo[w] = l;
      ot[w] = o;
      while (e) {
        const unsigned b = __builtin_ctz(e);
        e &= e - 1;
        epos[t].push_back(base + b);
        ebyte[t].push_back((uint8_t)seq[base + b]);
      }
    }
  };
  std::vector<std::thread> pool;
  for (unsigned t = 1; t < T; ++t) pool.emplace_back(work, t);
  work(0);
  for (auto& th : pool) th.join();
  for (uint64_t w = full; w < plane_words(n); ++w) hi[w] = lo[w] = ot[w] = 0;
  pad_planes(n, hi, lo, ot);
  if (exc_pos) {
    exc_pos->clear();
    exc_byte->clear();
    for (unsigned t = 0; t < T; ++t) {
      exc_pos->insert(exc_pos->end(), epos[t].begin(), epos[t].end());
      exc_byte->insert(exc_byte->end(), ebyte[t].begin(), ebyte[t].end());
    }
  }
}

int load_fasta(const std::string& path, PackedGenome& g) {
  FILE* f = fopen(resolve(path).c_str(), "rb");
  if (!f) return 1;
  int first = fgetc(f);
  if (first != '>') {
    fclose(f);
    return 1;
  }
  rewind(f);
  g = PackedGenome();
  std::string text;
  {
    fseek(f, 0, SEEK_END);
    long sz = ftell(f);
    rewind(f);
    if (sz > 0) text.reserve((size_t)sz);
  }
  // Line splitting on '\n' over large blocks; `line` carries a partial line.
  std::vector<char> buf(1 << 24);
  std::string line;
  auto flush_line = [&](const char* p, size_t len) {
    if (len == 0) return;
    if (p[len - 1] == '\r') --len;
    if (len > 0 && p[0] == '>') {
      g.names.emplace_back(p + 1, len - 1);
      if (!g.starts.empty()) text.push_back(';');
      g.starts.push_back(text.size());
    } else {
      const size_t at = text.size();
      text.append(p, len);
      for (size_t i = at; i < text.size(); ++i) {
        const unsigned char c = (unsigned char)text[i];
        if (c >= 'a' && c <= 'z') text[i] = (char)(c - 32);
      }
    }
  };
  size_t got;
  while ((got = fread(buf.data(), 1, buf.size(), f)) > 0) {
    const char* p = buf.data();
    const char* end = p + got;
    while (p < end) {
      const char* nl = (const char*)memchr(p, '\n', (size_t)(end - p));
      if (!nl) {
        line.append(p, (size_t)(end - p));
        break;
      }
      if (line.empty()) {
        flush_line(p, (size_t)(nl - p));
      } else {
        line.append(p, (size_t)(nl - p));
        flush_line(line.data(), line.size());
        line.clear();
      }
      p = nl + 1;
    }
  }
  if (!line.empty()) flush_line(line.data(), line.size());
  fclose(f);
  g.n = text.size();
  const uint64_t W = plane_words(g.n);
  g.hi.assign(W, 0);
  g.lo.assign(W, 0);
  g.ot.assign(W, 0);
  pack_text(text.data(), g.n, g.hi.data(), g.lo.data(), g.ot.data(), &g.exc_pos, &g.exc_byte);
  return 0;
}

namespace {

// One 2BIT byte (4 bases, first in the top bits) as 4 hi and 4 lo plane bits.
struct TwoBitTable {
  uint8_t hi[256], lo[256];
  TwoBitTable() {
    for (int b = 0; b < 256; ++b) {
      hi[b] = lo[b] = 0;
      for (int k = 0; k < 4; ++k) {
        const int code = (b >> (6 - 2 * k)) & 3;
        hi[b] |= (uint8_t)(((code >> 1) & 1) << k);
        lo[b] |= (uint8_t)((code & 1) << k);
      }
    }
  }
};
const TwoBitTable kTwoBit;

// Sets plane bits [p, p+cnt) to ot=1, (hi,lo) = (0, sep).
void mark_other(PackedGenome& g, uint64_t p, uint64_t cnt, bool sep) {
  for (uint64_t q = p; q < p + cnt;) {
    const uint64_t w = q >> 5;
    const unsigned b = q & 31;
    const unsigned take = (unsigned)std::min<uint64_t>(32 - b, p + cnt - q);
    const uint32_t m = (take == 32 ? 0xFFFFFFFFu : ((1u << take) - 1)) << b;
    g.ot[w] |= m;
    g.hi[w] &= ~m;
    if (sep) g.lo[w] |= m;
    else g.lo[w] &= ~m;
    q += take;
  }
}

}  // namespace

int load_twobit(const std::string& path, PackedGenome& g) {
  FILE* f = fopen(resolve(path).c_str(), "rb");
  if (!f) return 1;
  bool swap = false;  // file written on a machine of the other byte order
  auto u32 = [&](uint32_t& v) {
    if (fread(&v, 4, 1, f) != 1) return false;
    if (swap) v = __builtin_bswap32(v);
    return true;
  };
  uint32_t magic = 0, version = 2, count = 0, reserved = 0;
  if (!u32(magic) || (magic != 0x1A412743u && magic != 0x4327411Au)) {
    fclose(f);
    return 1;
  }
  swap = magic == 0x4327411Au;
  if (!u32(version) || version > 1) {
    fclose(f);
    return 1;
  }
  g = PackedGenome();
  u32(count);
  u32(reserved);
  // Index: name and file offset of each record (32-bit in version 0, 64-bit
  // in version 1).  The reference reads records back to back after the index
  // and knows version 0 only; honouring the offsets reads the same bytes for
  // files laid out that way and the right ones for any other layout.
  std::vector<uint64_t> offset(count, 0);
  for (uint32_t i = 0; i < count; ++i) {
    unsigned char nlen = 0;
    char name[256];
    if (fread(&nlen, 1, 1, f) != 1) nlen = 0;
    const size_t got = fread(name, 1, nlen, f);
    g.names.emplace_back(name, got);
    uint32_t lo32 = 0, hi32 = 0;
    u32(lo32);
    if (version == 1) {
      u32(hi32);
      if (swap) std::swap(lo32, hi32);
    }
    offset[i] = ((uint64_t)hi32 << 32) | lo32;
  }
  struct Rec {
    uint32_t len;
    std::vector<uint32_t> nstart, nsize;
    std::vector<uint8_t> packed;
  };
  // First pass: read every record (lengths are needed to size the planes).
  std::vector<Rec> recs(count);
  uint64_t total = 0;
  for (uint32_t r = 0; r < count; ++r) {
    Rec& R = recs[r];
    if (offset[r] && fseeko(f, (off_t)offset[r], SEEK_SET) != 0) break;
    uint32_t nb = 0, mb = 0;
    R.len = 0;
    u32(R.len);
    u32(nb);
    R.nstart.resize(nb);
    R.nsize.resize(nb);
    for (auto& v : R.nstart) u32(v);
    for (auto& v : R.nsize) u32(v);
    u32(mb);
    fseeko(f, (off_t)mb * 8 + 4, SEEK_CUR);
    R.packed.assign(((uint64_t)R.len + 3) / 4, 0);
    const size_t got = fread(R.packed.data(), 1, R.packed.size(), f);
    (void)got;  // a short file leaves zeros (T), like the reference's unread buffer
    total += R.len + (r + 1 < count ? 1 : 0);
  }
  fclose(f);
  g.n = total;
  const uint64_t W = plane_words(g.n);
  g.hi.assign(W, 0);
  g.lo.assign(W, 0);
  g.ot.assign(W, 0);
  uint64_t p = 0;
  for (uint32_t r = 0; r < count; ++r) {
    Rec& R = recs[r];
    if (r == 0) g.starts.push_back(0);
    // Bases: 4 per byte, first base in the two most significant bits.  Eight
    // bytes make 32 positions, placed at any bit offset of the planes.
    for (uint64_t i = 0; i < R.len; i += 32) {
      uint32_t hw = 0, lw = 0;
      const uint64_t b0 = i >> 2, b1 = std::min<uint64_t>(b0 + 8, R.packed.size());
      for (uint64_t b = b0; b < b1; ++b) {
        hw |= (uint32_t)kTwoBit.hi[R.packed[b]] << (4 * (b - b0));
        lw |= (uint32_t)kTwoBit.lo[R.packed[b]] << (4 * (b - b0));
      }
      const uint64_t take = std::min<uint64_t>(32, R.len - i);
      if (take < 32) {
        hw &= (1u << take) - 1;
        lw &= (1u << take) - 1;
      }
      const uint64_t q = p + i;
      const unsigned s = q & 31;
      g.hi[q >> 5] |= hw << s;
      g.lo[q >> 5] |= lw << s;
      if (s) {
        g.hi[(q >> 5) + 1] |= hw >> (32 - s);
        g.lo[(q >> 5) + 1] |= lw >> (32 - s);
      }
    }
    for (size_t b = 0; b < R.nstart.size(); ++b) {
      const uint64_t s = R.nstart[b];
      if (s >= R.len) continue;
      const uint64_t e = std::min<uint64_t>((uint64_t)R.len, s + R.nsize[b]);
      mark_other(g, p + s, e - s, false);
    }
    p += R.len;
    if (r + 1 < count) {
      mark_other(g, p, 1, true);
      ++p;
      g.starts.push_back(p);
    }
  }
  pad_planes(g.n, g.hi.data(), g.lo.data(), g.ot.data());
  return 0;
}

}  // namespace cof

// Test hook (include/cof_tools.h): the reference's genome string as the
// loaders produce it, decoded back from the planes.
extern "C" int cofx_genome_text(const char* path, char* out, uint64_t cap, uint64_t* n) {
  cof::PackedGenome g;
  const std::string p = path ? path : "";
  if (cof::load_fasta(p, g) != 0 && cof::load_twobit(p, g) != 0) return 1;
  if (n) *n = g.n;
  if (!out || cap < g.n) return 0;
  size_t e = 0;
  for (uint64_t q = 0; q < g.n; ++q) {
    const unsigned b = q & 31;
    const unsigned h = (g.hi[q >> 5] >> b) & 1, l = (g.lo[q >> 5] >> b) & 1, o = (g.ot[q >> 5] >> b) & 1;
    char c;
    if (!o) c = "TCAG"[h * 2 + l];
    else if (!h) c = l ? ';' : 'N';
    else {
      while (e < g.exc_pos.size() && g.exc_pos[e] < q) ++e;
      c = (e < g.exc_pos.size() && g.exc_pos[e] == q) ? (char)g.exc_byte[e] : 'N';
    }
    out[q] = c;
  }
  return 0;
}
