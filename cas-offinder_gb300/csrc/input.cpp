// Input-file parsing, compare-variant expansion and output row shapes.
//
// Semantics follow the reference exactly, quirks included:
//   parse_job     Cas_OFFinder::parseInput (cas-offinder.cpp:590-694) with
//                 parseLine (:570-583) and add_compare (:14-18)
//   build_shapes  the row surgery of Cas_OFFinder::compareAll
//                 (cas-offinder.cpp:394-455), evaluated once per
//                 (variant, bulge record, strand) on a symbolic window
//   mismatch      the IUPAC test of cas-offinder.cl:30-43 / cas-offinder.cpp:302-315
//   complement_byte  set_complementary_sequence (cas-offinder.cpp:35-58)
#include <algorithm>
#include <cstdlib>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "cof_internal.h"

namespace cof {

bool mismatch(unsigned char p, unsigned char g) {
  // Allowed-base sets as 4-bit masks over (A, C, G, T); concrete bases
  // mismatch every byte but themselves, degenerate codes only the bases
  // outside their set, anything else (N included) nothing.
  unsigned set;
  switch (p) {
    case 'A': return g != 'A';
    case 'C': return g != 'C';
    case 'G': return g != 'G';
    case 'T': return g != 'T';
    case 'R': set = 0x5; break;  // A G
    case 'Y': set = 0xA; break;  // C T
    case 'K': set = 0xC; break;  // G T
    case 'M': set = 0x3; break;  // A C
    case 'W': set = 0x9; break;  // A T
    case 'S': set = 0x6; break;  // C G
    case 'H': set = 0xB; break;  // A C T
    case 'B': set = 0xE; break;  // C G T
    case 'V': set = 0x7; break;  // A C G
    case 'D': set = 0xD; break;  // A G T
    default: return false;
  }
  unsigned bit;
  switch (g) {
    case 'A': bit = 1; break;
    case 'C': bit = 2; break;
    case 'G': bit = 4; break;
    case 'T': bit = 8; break;
    default: return false;
  }
  return (set & bit) == 0;
}

unsigned char complement_byte(unsigned char c) {
  static const char from[] = "ATGCRYMKHDBV";
  static const char to[] = "TACGYRKMDHVB";
  for (int i = 0; i < 12; ++i)
    if (c == (unsigned char)from[i]) return (unsigned char)to[i];
  return c;
}

namespace {

struct ParseError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

std::string to_upper(std::string s) {
  std::transform(s.begin(), s.end(), s.begin(), [](char c) { return (char)toupper((unsigned char)c); });
  return s;
}

std::vector<std::string> tokens(const std::string& line) {
  std::vector<std::string> t;
  std::istringstream is(line);
  for (std::string w; is >> w;) t.push_back(w);
  return t;
}

// parseLine: a required line after end of file throws; a failed read returns
// false with `line` cleared; a trailing '\r' is removed.
bool next_line(std::istream& is, std::string& line, bool required) {
  if (required && is.eof()) throw ParseError("Unexpected end of file.");
  if (!std::getline(is, line)) return false;
  if (!line.empty() && line.back() == '\r') line.pop_back();
  return true;
}

bool is_decimal(const std::string& s) { return s.find_first_not_of("0123456789") == std::string::npos; }

}  // namespace

bool parse_job(const char* text, size_t len, Job& job, std::string& err) {
  job = Job();
  std::istringstream is(std::string(text, len));
  std::map<std::string, Variant> table;
  auto insert = [&](const std::string& key, const std::string& id, uint16_t thr, BulgeRecord b) {
    auto it = table.find(key);
    if (it != table.end()) {
      it->second.bulges.push_back(std::move(b));
      return;
    }
    Variant v;
    v.key = key;
    v.id = id;
    v.threshold = thr;
    v.bulges.push_back(std::move(b));
    v.order = (uint32_t)table.size();
    table.emplace(key, std::move(v));
  };
  try {
    std::string line;
    next_line(is, job.genome_path, true);
    next_line(is, line, true);
    std::vector<std::string> t = tokens(line);
    if (t.size() != 1 && t.size() != 3) throw ParseError("Malformed input file.");
    if (t.size() == 3) {
      job.dna = (unsigned)atoi(t[1].c_str());
      job.rna = (unsigned)atoi(t[2].c_str());
    }
    job.pam5 = t[0][0] != 'N';  // tested before upper-casing, as the reference does
    const std::string pad(job.dna, 'N');
    job.pattern = to_upper(job.pam5 ? t[0] + pad : pad + t[0]);

    size_t guide_line = 0, tokens_per_line = 0;
    while (next_line(is, line, false)) {
      if (line.empty()) break;
      t = tokens(line);
      if (t.size() != 2 && t.size() != 3) throw ParseError("Malformed input file.");
      if (t[0].size() + job.dna != job.pattern.size())
        throw ParseError("The length of target sequences should match with the length of pattern sequence.");
      const std::string guide = to_upper(t[0]);
      const uint16_t thr = (uint16_t)atoi(t[1].c_str());
      const std::string id = t.size() == 3 ? t[2] : std::to_string(guide_line);
      const size_t lo = guide.find_first_not_of('N'), hi = guide.find_last_not_of('N');

      if (job.dna == 0) {
        insert(guide, id, thr, BulgeRecord{"0", 0});
      } else if (lo != std::string::npos) {
        // DNA bulges: i extra genome bases, modelled as i 'N's inserted into
        // the guide before guide position j, for j in [lo, hi + 1].
        const std::string plain = job.pam5 ? guide + pad : pad + guide;
        for (unsigned i = 1; i <= job.dna; ++i) {
          const std::string fill(job.dna - i, 'N'), gap(i, 'N');
          for (size_t j = lo; j <= hi + 1; ++j) {
            std::string key = job.pam5 ? guide.substr(0, j) + gap + guide.substr(j) + fill
                                       : fill + guide.substr(0, j) + gap + guide.substr(j);
            const int at = job.pam5 ? -(int)j : (int)j;
            const std::string what = key == plain ? std::string("0") : std::to_string(i);
            insert(key, id, thr, BulgeRecord{what, at});
          }
        }
      }
      // RNA bulges: i guide bases with no genome partner, modelled as the
      // guide with guide[j, j+i) deleted, for j in [lo, hi + 1 - i).
      for (unsigned i = 1; i <= job.rna; ++i) {
        // The reference computes hi + 1 - i in size_t; when that wraps (no
        // non-N byte, or fewer than i) its substr throws out_of_range.
        if (lo == std::string::npos || hi + 1 < i) throw ParseError("basic_string::substr");
        const std::string fill(job.dna + i, 'N');
        for (size_t j = lo; j + i < hi + 1; ++j) {
          std::string key = job.pam5 ? guide.substr(0, j) + guide.substr(j + i) + fill
                                     : fill + guide.substr(0, j) + guide.substr(j + i);
          insert(key, id, thr, BulgeRecord{guide.substr(j, i), job.pam5 ? -(int)j : (int)j});
        }
      }
      if (tokens_per_line == 0) tokens_per_line = t.size();
      else if (tokens_per_line != t.size())
        throw ParseError("The number of entries below 2nd line should be consistent.");
      ++guide_line;
    }
  } catch (const std::exception& e) {
    err = e.what();
    return false;
  }
  job.variants.reserve(table.size());
  for (auto& kv : table) job.variants.push_back(std::move(kv.second));
  return true;
}

// One row shape of compareAll (cas-offinder.cpp:401-450) for compare string
// `comp`, bulge record `b` and strand `minus`; `win` is the symbolic oriented
// window (window byte k written as 0x80 + k).
static RowShape shape_of(const Job& job, const Variant& v, const BulgeRecord& b, bool minus, const std::string& win) {
  const std::string& comp = v.key;
  const size_t dna = job.dna;
  const bool flipped = b.index < 0 || minus;
  const size_t at = (size_t)(b.index < 0 ? -(long)b.index : (long)b.index);
  RowShape r;
  std::string crrna, seq = win;
  if (is_decimal(b.what)) {
    r.bulge_size = (unsigned)std::stoi(b.what);
    const size_t sz = r.bulge_size;
    if (flipped) {
      r.offset = 0;
      crrna = comp.substr(0, at) + std::string(sz, '-') + comp.substr(at + sz);
    } else {
      const size_t off = dna - sz;
      r.offset = (int64_t)off;
      crrna = comp.substr(off, at) + std::string(sz, '-') + comp.substr(off + at + sz);
      seq = seq.substr(off);
    }
    if (sz == 0) {
      r.type = "X";
      if (flipped) {
        crrna = crrna.substr(0, crrna.size() - dna);
        seq = seq.substr(0, seq.size() - dna);
      }
    } else {
      r.type = "DNA";
    }
  } else {
    r.bulge_size = (unsigned)b.what.size();
    const size_t sz = r.bulge_size;
    if (flipped) {
      r.offset = 0;
      crrna = comp.substr(0, at) + b.what + comp.substr(at);
      seq = seq.substr(0, at) + std::string(sz, '-') + seq.substr(at);
      crrna = crrna.substr(0, crrna.size() - dna - sz);
      seq = seq.substr(0, seq.size() - dna - sz);
    } else {
      const size_t off = dna + sz;
      r.offset = (int64_t)off;
      crrna = comp.substr(off, at) + b.what + comp.substr(off + at);
      seq = seq.substr(off, at) + std::string(sz, '-') + seq.substr(off + at);
    }
    r.type = "RNA";
  }
  r.head = v.id + "\t" + r.type + "\t" + crrna + "\t";
  r.dna = seq;
  r.tail = std::to_string(r.bulge_size) + "\n";
  return r;
}

bool build_shapes(Job& job, std::string& err) {
  const size_t L = job.pattern.size();
  const size_t V = job.variants.size();
  std::string win(L, '\0');
  for (size_t k = 0; k < L; ++k) win[k] = (char)(0x80 + k);
  for (int s = 0; s < 2; ++s) job.shapes[s].assign(V, {});
  // Variants are independent: large inputs are split over a few threads.
  // The first failure in variant order is the one reported.
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t T = V < 4096 ? 1 : std::min<size_t>(std::min<unsigned>(hw, 8u), V / 2048);
  std::vector<size_t> bad(T, V);
  std::vector<std::string> why(T);
  auto work = [&](size_t t) {
    for (size_t v = V * t / T; v < V * (t + 1) / T; ++v)
      for (int s = 0; s < 2; ++s)
        for (const BulgeRecord& b : job.variants[v].bulges) {
          try {
            job.shapes[s][v].push_back(shape_of(job, job.variants[v], b, s == 1, win));
          } catch (const std::exception& e) {
            bad[t] = v;
            why[t] = e.what();
            return;
          }
        }
  };
  if (T == 1) {
    work(0);
  } else {
    std::vector<std::thread> th;
    for (size_t t = 0; t < T; ++t) th.emplace_back(work, t);
    for (std::thread& x : th) x.join();
  }
  for (size_t t = 0; t < T; ++t)
    if (bad[t] < V) {
      err = "row construction failed: " + why[t];
      return false;
    }
  return true;
}

}  // namespace cof
