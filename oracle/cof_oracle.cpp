/*
 * cof-oracle: CPU restatement of Cas-OFFinder 3.0.0's search path.
 *
 * TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg run this program, and only as the checker or the timed CPU
 * baseline.  The product never links or calls it.
 *
 * It restates, function by function, what the reference computes:
 *   parse_input         cas-offinder.cpp:590-694 (+ add_compare :14-18,
 *                       parseLine :570-583, isnumeric cas-offinder.h:20-22)
 *   revcomp             cas-offinder.cpp:35-58  (set_complementary_sequence)
 *   non_n_index         cas-offinder.cpp:60-70  (set_seq_flags)
 *   mism                cas-offinder.cl:30-43   (IUPAC mismatch predicate)
 *   find_candidates     cas-offinder.cl:157-213 (finder_cpu)
 *   compare_all         cas-offinder.cl:214-286 (comparer_cpu, every variant)
 *   format_hits         cas-offinder.cpp:394-455 (compareAll's row surgery)
 *   read_fasta          read_fasta.cpp:11-58
 *   read_twobit         read_twobit.cpp:44-131
 *   write_summary       cas-offinder.cpp:471-500
 *   main                main.cpp:72-157 (argv contract, directory walk)
 * The whole file is searched as one chunk.  With a single chunk the reference
 * emits rows variant by variant (std::map key order), hits of a variant in
 * work-item order, and every bulge record of a hit in insertion order; this
 * program emits exactly that sequential order, so its output equals the
 * reference's run with one OpenMP thread byte for byte.  OpenMP threads here
 * only split loops whose results are merged back in sequential order.
 *
 * Usage: cof-oracle [--summary f] {input|-} {C|G|A}[ids] {output|-}
 *        cof-oracle --mismatch-table out.bin   (the predicate, 256x256 bytes)
 * Environment: OMP_NUM_THREADS sets the thread count.
 */
#include <dirent.h>
#include <sys/stat.h>
#include <sys/time.h>
#include <unistd.h>

#include <algorithm>
#include <climits>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------- sequences
unsigned char g_mism[256][256];  // g_mism[pattern char][genome char]

// cas-offinder.cl:30-43: a concrete base mismatches every other byte; a
// degenerate code mismatches only the concrete bases outside its set; N and
// every other byte never mismatch.
bool mism_slow(unsigned char p, unsigned char g) {
  switch (p) {
    case 'A': return g != 'A';
    case 'C': return g != 'C';
    case 'G': return g != 'G';
    case 'T': return g != 'T';
    case 'R': return g == 'C' || g == 'T';
    case 'Y': return g == 'A' || g == 'G';
    case 'K': return g == 'A' || g == 'C';
    case 'M': return g == 'G' || g == 'T';
    case 'W': return g == 'C' || g == 'G';
    case 'S': return g == 'A' || g == 'T';
    case 'H': return g == 'G';
    case 'B': return g == 'A';
    case 'V': return g == 'T';
    case 'D': return g == 'C';
    default: return false;
  }
}

void init_tables() {
  for (int p = 0; p < 256; ++p)
    for (int g = 0; g < 256; ++g) g_mism[p][g] = mism_slow((unsigned char)p, (unsigned char)g) ? 1 : 0;
}

inline bool mism(char p, char g) { return g_mism[(unsigned char)p][(unsigned char)g] != 0; }

char complement(char c) {
  switch (c) {
    case 'A': return 'T';
    case 'T': return 'A';
    case 'G': return 'C';
    case 'C': return 'G';
    case 'R': return 'Y';
    case 'Y': return 'R';
    case 'M': return 'K';
    case 'K': return 'M';
    case 'H': return 'D';
    case 'D': return 'H';
    case 'B': return 'V';
    case 'V': return 'B';
    default: return c;
  }
}

std::string revcomp(const std::string& s) {
  std::string r(s.rbegin(), s.rend());
  for (char& c : r) c = complement(c);
  return r;
}

// Positions of the bytes that are not 'N' (cas-offinder.cpp:60-70).  The
// reference's kernels stop at the -1 terminator, i.e. they visit exactly these.
std::vector<int> non_n_index(const std::string& s) {
  std::vector<int> v;
  for (size_t i = 0; i < s.size(); ++i)
    if (s[i] != 'N') v.push_back((int)i);
  return v;
}

std::string upper(std::string s) {
  for (char& c : s) c = (char)toupper((unsigned char)c);
  return s;
}

std::vector<std::string> split_ws(const std::string& line) {
  std::istringstream is(line);
  std::vector<std::string> out;
  std::string t;
  while (is >> t) out.push_back(t);
  return out;
}

bool all_digits(const std::string& s) { return s.find_first_not_of("0123456789") == std::string::npos; }

// ---------------------------------------------------------------- input file
struct Bulge {
  std::string what;  // decimal DNA-bulge size ("0" = none) or the deleted RNA bases
  int index;         // insertion point; negated when the PAM is at the 5' end
};
struct Variant {
  std::string id;
  uint16_t threshold;
  std::vector<Bulge> bulges;
};

struct Input {
  std::string genome_path;
  std::string pattern;
  unsigned dna = 0, rna = 0;
  std::map<std::string, Variant> variants;  // keyed by the full compare string
};

[[noreturn]] void critical(const std::string& what) {
  std::cerr << "Critical error! " << what << std::endl;
  std::exit(1);
}

// parseLine (cas-offinder.cpp:570-583): a required line at end of file is an
// error; otherwise a failed read returns false (and leaves `line` empty), and a
// trailing '\r' is dropped.
bool read_line(std::istream& in, std::string& line, bool required) {
  if (required && in.eof()) critical("Unexpected end of file.");
  if (!std::getline(in, line)) return false;
  if (!line.empty() && line.back() == '\r') line.pop_back();
  return true;
}

void add_variant(Input& in, const std::string& key, const std::string& id, uint16_t thr, const Bulge& b) {
  auto it = in.variants.find(key);
  if (it == in.variants.end()) in.variants.emplace(key, Variant{id, thr, {b}});
  else it->second.bulges.push_back(b);  // first inserter keeps id and threshold
}

Input parse_input(std::istream& is) {
  Input in;
  std::string line;
  if (!is.good()) critical("Cannot read input file.");
  read_line(is, in.genome_path, true);  // the reference ignores a failed read here
  read_line(is, line, true);
  std::vector<std::string> tok = split_ws(line);
  if (tok.size() != 1 && tok.size() != 3) critical("Malformed input file.");
  if (tok.size() == 3) {
    in.dna = (unsigned)atoi(tok[1].c_str());
    in.rna = (unsigned)atoi(tok[2].c_str());
  }
  // The PAM side is decided on the raw first byte, before upper-casing.
  const bool pam5 = tok[0][0] != 'N';
  in.pattern = upper(pam5 ? tok[0] + std::string(in.dna, 'N') : std::string(in.dna, 'N') + tok[0]);

  size_t guide_no = 0, ntok_first = 0;
  while (read_line(is, line, false)) {
    if (line.empty()) break;
    tok = split_ws(line);
    if (tok.size() != 2 && tok.size() != 3) critical("Malformed input file.");
    if (tok[0].size() + in.dna != in.pattern.size())
      critical("The length of target sequences should match with the length of pattern sequence.");
    const std::string g = upper(tok[0]);
    const uint16_t thr = (uint16_t)atoi(tok[1].c_str());  // stored as cl_ushort
    const std::string id = tok.size() == 3 ? tok[2] : std::to_string(guide_no);
    const size_t first = g.find_first_not_of('N');
    const size_t last = g.find_last_not_of('N');
    if (in.dna == 0) {
      add_variant(in, g, id, thr, Bulge{"0", 0});
    } else if (first != std::string::npos) {
      const std::string unbulged = pam5 ? g + std::string(in.dna, 'N') : std::string(in.dna, 'N') + g;
      for (unsigned i = 1; i <= in.dna; ++i) {
        const unsigned pad = in.dna - i;
        for (size_t j = first; j < last + 2; ++j) {
          const std::string gap(i, 'N');
          const std::string key = pam5 ? g.substr(0, j) + gap + g.substr(j) + std::string(pad, 'N')
                                       : std::string(pad, 'N') + g.substr(0, j) + gap + g.substr(j);
          const int idx = pam5 ? -(int)j : (int)j;
          add_variant(in, key, id, thr, Bulge{key == unbulged ? "0" : std::to_string(i), idx});
        }
      }
    }
    for (unsigned i = 1; i <= in.rna; ++i) {
      // The reference's loop bound is size_t arithmetic; when it wraps the
      // loop walks off the guide and std::string::substr throws.
      if (first == std::string::npos || last + 1 < i) critical("basic_string::substr");
      const unsigned pad = in.dna + i;
      for (size_t j = first; j < last + 1 - i; ++j) {
        const std::string key = pam5 ? g.substr(0, j) + g.substr(j + i) + std::string(pad, 'N')
                                     : std::string(pad, 'N') + g.substr(0, j) + g.substr(j + i);
        add_variant(in, key, id, thr, Bulge{g.substr(j, i), pam5 ? -(int)j : (int)j});
      }
    }
    if (ntok_first == 0) ntok_first = tok.size();
    else if (ntok_first != tok.size()) critical("The number of entries below 2nd line should be consistent.");
    ++guide_no;
  }
  return in;
}

// ---------------------------------------------------------------- genome files
struct Genome {
  std::vector<std::string> names;
  std::string seq;                  // records joined with ';'
  std::vector<unsigned long long> starts;
};

std::string resolve_link(const std::string& path) {
  char buf[PATH_MAX + 1];
  memset(buf, 0, sizeof(buf));
  ssize_t n = readlink(path.c_str(), buf, PATH_MAX);
  return n >= 0 ? std::string(buf) : path;
}

// read_fasta.cpp:11-58.  Returns false when the first byte is not '>'.
bool read_fasta(const std::string& path, Genome& gn) {
  std::ifstream f(resolve_link(path));
  gn = Genome();
  char c = 0;
  if (!f.get(c) || c != '>') return false;
  f.seekg(0);
  std::string line;
  while (std::getline(f, line)) {
    if (line.empty()) continue;
    if (line.back() == '\r') line.pop_back();
    if (!line.empty() && line[0] == '>') {
      gn.names.push_back(line.substr(1));
      if (!gn.starts.empty()) gn.seq.push_back(';');
      gn.starts.push_back(gn.seq.size());
    } else {
      for (char& ch : line) ch = (char)toupper((unsigned char)ch);
      gn.seq += line;
    }
  }
  return true;
}

// read_twobit.cpp:44-131: host-order magic, version 0, index offsets ignored
// (records are read back to back), 2-bit codes T,C,A,G = 0..3 from the most
// significant bits, N blocks written as 'N', soft-mask blocks skipped.
bool read_twobit(const std::string& path, Genome& gn) {
  FILE* f = fopen(resolve_link(path).c_str(), "rb");
  if (!f) return false;
  auto u32 = [&](uint32_t& v) { return fread(&v, 4, 1, f) == 1; };
  uint32_t magic = 0, version = 1, count = 0, reserved = 0;
  if (!u32(magic) || magic != 0x1A412743u || !u32(version) || version != 0) {
    fclose(f);
    return false;
  }
  u32(count);
  u32(reserved);
  for (uint32_t i = 0; i < count; ++i) {
    unsigned char len = 0;
    char name[256];
    if (fread(&len, 1, 1, f) != 1) break;
    size_t got = fread(name, 1, len, f);
    name[got] = 0;
    gn.names.push_back(name);
    uint32_t off;
    u32(off);
  }
  static const char kBase[4] = {'T', 'C', 'A', 'G'};
  gn.starts.push_back(0);
  for (uint32_t r = 0; r < count; ++r) {
    uint32_t len = 0, nblocks = 0, mblocks = 0;
    u32(len);
    u32(nblocks);
    std::vector<uint32_t> nstart(nblocks), nsize(nblocks);
    for (auto& v : nstart) u32(v);
    for (auto& v : nsize) u32(v);
    u32(mblocks);
    fseek(f, (long)mblocks * 8 + 4, SEEK_CUR);
    std::vector<unsigned char> packed((len + 3) / 4);
    size_t got = fread(packed.data(), 1, packed.size(), f);
    (void)got;
    std::string s(len, 'N');
    for (uint32_t p = 0; p < len; ++p) s[p] = kBase[(packed[p >> 2] >> (6 - 2 * (p & 3))) & 3];
    for (uint32_t b = 0; b < nblocks; ++b)
      for (uint32_t p = nstart[b]; p < nstart[b] + nsize[b] && p < len; ++p) s[p] = 'N';
    gn.seq += s;
    if (r + 1 < count) {
      gn.seq.push_back(';');
      gn.starts.push_back(gn.seq.size());
    }
  }
  fclose(f);
  return true;
}

// ---------------------------------------------------------------- search
// A candidate start and its finder flag packed in one word: pos << 2 | flag.
// flag 0: both strands, 1: forward only, 2: reverse only.
struct Candidate {
  uint64_t v;
  uint64_t pos() const { return v >> 2; }
  char flag() const { return (char)(v & 3); }
};
struct Hit {
  uint64_t pos;
  uint16_t mm;
  char dir;
};

int nthreads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
int thread_id() {
#ifdef _OPENMP
  return omp_get_thread_num();
#else
  return 0;
#endif
}

// finder_cpu (cas-offinder.cl:157-213) over positions [0, n-L], in order.
std::vector<Candidate> find_candidates(const std::string& chr, const std::string& pat) {
  const size_t L = pat.size();
  std::vector<Candidate> out;
  if (chr.size() < L || L == 0) return out;
  const std::string rpat = revcomp(pat);
  const std::vector<int> fi = non_n_index(pat), ri = non_n_index(rpat);
  const uint64_t npos = chr.size() - L + 1;
  const int T = nthreads();
  std::vector<std::vector<Candidate>> part(T);
  const char* g = chr.data();
#pragma omp parallel
  {
    std::vector<Candidate>& mine = part[thread_id()];
#pragma omp for schedule(static)
    for (long long ii = 0; ii < (long long)npos; ++ii) {
      const uint64_t i = (uint64_t)ii;
      char flag = 0;
      for (size_t j = 0; j < fi.size(); ++j) {
        if (mism(pat[fi[j]], g[i + fi[j]])) flag |= 2;
        if (mism(rpat[ri[j]], g[i + ri[j]])) flag |= 1;
        if (flag == 3) break;
      }
      if (flag == 3) continue;
      if (memchr(g + i, ';', L)) continue;
      mine.push_back(Candidate{i << 2 | (uint64_t)flag});
    }
  }
  size_t total = 0;
  for (auto& p : part) total += p.size();
  out.reserve(total);
  for (auto& p : part) {  // static schedule: thread t holds the t-th range, so this keeps position order
    out.insert(out.end(), p.begin(), p.end());
    std::vector<Candidate>().swap(p);
  }
  return out;
}

// Mismatches of `comp` at its non-N positions against chr[pos..].  The
// reference stops counting once the count passes the threshold and then
// drops the candidate (cas-offinder.cl:241-243); this counts every position.
// Both keep a candidate exactly when the full count is <= the threshold, and
// then the two counts are equal, so the hits and their counts are the same.
// Counting without the data-dependent exit avoids a mispredicted branch per
// position, which made the early-exit loop several times slower.
inline unsigned count_mm(const char* g, const char* comp, const int* idx, size_t n) {
  unsigned c = 0;
  for (size_t j = 0; j < n; ++j) c += g_mism[(unsigned char)comp[idx[j]]][(unsigned char)g[idx[j]]];
  return c;
}

// One compare variant as comparer_cpu sees it (cas-offinder.cpp:360-370 sets
// its arguments): the compare string and its reverse complement, with the
// non-N index lists of both, and the threshold.
struct CompareArgs {
  std::string comp, rcomp;
  std::vector<int> fi, ri;
  unsigned thr;
};

// comparer_cpu (cas-offinder.cl:214-286) for every variant: hits[v] holds
// variant v's hits in work-item order ('+' before '-' for one candidate).
// The candidates are cut into blocks that threads take in any order; a block
// is tested against every variant while its windows are in cache, and the
// per-block hit lists are joined in block order, so every variant's list is
// the one a single sequential pass over all candidates gives.
std::vector<std::vector<Hit>> compare_all(const std::string& chr, const std::vector<Candidate>& cands,
                                          const std::vector<CompareArgs>& vs) {
  const size_t V = vs.size();
  std::vector<std::vector<Hit>> hits(V);
  if (cands.empty() || V == 0) return hits;
  const size_t B = 2048, nb = (cands.size() + B - 1) / B;
  std::vector<std::vector<Hit>> blk_hits(nb);
  std::vector<std::vector<uint32_t>> blk_off(nb);  // variant v's hits of block b: [off[v], off[v+1])
#pragma omp parallel for schedule(dynamic, 4)
  for (long long bb = 0; bb < (long long)nb; ++bb) {
    const size_t c0 = (size_t)bb * B, c1 = std::min(cands.size(), c0 + B);
    std::vector<Hit>& H = blk_hits[bb];
    std::vector<uint32_t>& off = blk_off[bb];
    off.resize(V + 1);
    for (size_t v = 0; v < V; ++v) {
      off[v] = (uint32_t)H.size();
      const CompareArgs& a = vs[v];
      for (size_t c = c0; c < c1; ++c) {
        const uint64_t pos = cands[c].pos();
        const char flag = cands[c].flag();
        const char* g = chr.data() + pos;
        if (flag == 0 || flag == 1) {
          const unsigned m = count_mm(g, a.comp.data(), a.fi.data(), a.fi.size());
          if (m <= a.thr) H.push_back(Hit{pos, (uint16_t)m, '+'});
        }
        if (flag == 0 || flag == 2) {
          const unsigned m = count_mm(g, a.rcomp.data(), a.ri.data(), a.ri.size());
          if (m <= a.thr) H.push_back(Hit{pos, (uint16_t)m, '-'});
        }
      }
    }
    off[V] = (uint32_t)H.size();
  }
  for (size_t v = 0; v < V; ++v)
    for (size_t b = 0; b < nb; ++b)
      hits[v].insert(hits[v].end(), blk_hits[b].begin() + blk_off[b][v], blk_hits[b].begin() + blk_off[b][v + 1]);
  return hits;
}

// compareAll's per-hit row construction (cas-offinder.cpp:394-455).
void format_hits(std::ostream& os, const Genome& gn, const Input& in, const std::string& comp, const Variant& v,
                 const std::vector<Hit>& hits, std::map<std::string, unsigned>* summary) {
  const size_t L = in.pattern.size();
  std::string window;
  for (const Hit& h : hits) {
    window = gn.seq.substr(h.pos, L);
    if (h.dir == '-') window = revcomp(window);
    for (size_t k = 0; k < L; ++k)
      if (mism(comp[k], window[k])) window[k] = (char)(window[k] + 32);
    size_t rec = 0;
    for (size_t j = 0; j < gn.starts.size() && h.pos >= gn.starts[j]; ++j) rec = j;
    for (const Bulge& b : v.bulges) {
      const bool flipped = b.index < 0 || h.dir == '-';
      const size_t at = (size_t)(b.index < 0 ? -b.index : b.index);
      std::string crrna, dna = window, type;
      unsigned size;
      long offset;
      if (all_digits(b.what)) {
        size = (unsigned)std::stoi(b.what);
        if (flipped) {
          offset = 0;
          crrna = comp.substr(0, at) + std::string(size, '-') + comp.substr(at + size);
        } else {
          offset = (long)in.dna - (long)size;
          crrna = comp.substr(offset, at) + std::string(size, '-') + comp.substr(offset + at + size);
          dna = dna.substr(offset);
        }
        if (size == 0) {
          type = "X";
          if (flipped) {
            crrna = crrna.substr(0, crrna.size() - in.dna);
            dna = dna.substr(0, dna.size() - in.dna);
          }
        } else {
          type = "DNA";
        }
      } else {
        size = (unsigned)b.what.size();
        if (flipped) {
          offset = 0;
          crrna = comp.substr(0, at) + b.what + comp.substr(at);
          dna = dna.substr(0, at) + std::string(size, '-') + dna.substr(at);
          crrna = crrna.substr(0, crrna.size() - in.dna - size);
          dna = dna.substr(0, dna.size() - in.dna - size);
        } else {
          offset = (long)in.dna + (long)size;
          crrna = comp.substr(offset, at) + b.what + comp.substr(offset + at);
          dna = dna.substr(offset, at) + std::string(size, '-') + dna.substr(offset + at);
        }
        type = "RNA";
      }
      os << v.id << '\t' << type << '\t' << crrna << '\t' << dna << '\t' << gn.names[rec] << '\t'
         << (unsigned long long)(h.pos - gn.starts[rec] + (unsigned long long)offset) << '\t' << h.dir << '\t'
         << h.mm << '\t' << size << '\n';
      if (summary) {
        char key[10000];
        snprintf(key, sizeof key, "%s,%s,%d,%d", v.id.c_str(), type.c_str(), (int)size, (int)h.mm);
        ++(*summary)[key];
      }
    }
  }
}

// writeSummaryTable (cas-offinder.cpp:471-500).
void write_summary(const std::string& path, const std::map<std::string, unsigned>& table) {
  static const char* kHead[4] = {"Id", "Bulge Type", "Bulge Size", "Mismatches"};
  std::ofstream file;
  std::ostream* os = &std::cout;
  if (path != "-") {
    file.open(path, std::ios::out);
    os = &file;
  }
  for (const auto& kv : table) {
    std::string key = kv.first;
    size_t cut, col = 0;
    *os << "##";
    while ((cut = key.find(',')) != std::string::npos && col < 3) {
      *os << kHead[col++] << "=" << key.substr(0, cut) << ";";
      key.erase(0, cut + 1);
    }
    *os << kHead[col] << "=" << key << ";";
    *os << "Number of Found Targets=" << kv.second << std::endl;
  }
}

void search_file(const std::string& path, const Input& in, std::ostream& os, const std::string& summary_path,
                 std::map<std::string, unsigned>& summary) {
  Genome gn;
  std::cerr << "Reading " << path << "..." << std::endl;
  if (!read_fasta(path, gn)) {
    gn = Genome();
    if (!read_twobit(path, gn)) {
      std::cerr << "Skipping non-acceptable file " << path << "..." << std::endl;
      return;
    }
  }
  const bool want_summary = !summary_path.empty();
  const std::vector<Candidate> cands = find_candidates(gn.seq, in.pattern);
  // compareAll (cas-offinder.cpp:356) walks the variants in std::map key order.
  std::vector<CompareArgs> args;
  std::vector<const std::pair<const std::string, Variant>*> order;
  for (const auto& kv : in.variants) {
    CompareArgs a;
    a.comp = kv.first;
    a.rcomp = revcomp(kv.first);
    a.fi = non_n_index(a.comp);
    a.ri = non_n_index(a.rcomp);
    a.thr = kv.second.threshold;
    args.push_back(std::move(a));
    order.push_back(&kv);
  }
  const std::vector<std::vector<Hit>> hits = compare_all(gn.seq, cands, args);
  for (size_t v = 0; v < order.size(); ++v)
    format_hits(os, gn, in, order[v]->first, order[v]->second, hits[v], want_summary ? &summary : nullptr);
  os.flush();
  if (want_summary) write_summary(summary_path, summary);
}

}  // namespace

int main(int argc, char** argv) {
  init_tables();
  if (argc == 3 && std::string(argv[1]) == "--mismatch-table") {  // the predicate as 256x256 bytes
    FILE* f = fopen(argv[2], "wb");
    if (!f) return 1;
    for (int p = 0; p < 256; ++p) fwrite(g_mism[p], 1, 256, f);
    fclose(f);
    return 0;
  }
  struct timeval t0, t1;
  gettimeofday(&t0, nullptr);
  std::vector<std::string> pos;
  std::string summary_path;
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    if (a.size() > 2 && a[0] == '-' && a[1] == '-') {
      if (a == "--summary" && i + 1 < argc) summary_path = argv[++i];
      else {
        std::cout << "Usage: cof-oracle [--summary f] {input|-} {C|G|A}[ids] {output|-}" << std::endl;
        return 0;
      }
    } else {
      pos.push_back(a);
    }
  }
  if (pos.size() < 3) {
    std::cout << "Usage: cof-oracle [--summary f] {input|-} {C|G|A}[ids] {output|-}" << std::endl;
    return 0;
  }
  if (pos[1].empty() || (pos[1][0] != 'C' && pos[1][0] != 'G' && pos[1][0] != 'A')) {
    std::cerr << "Unknown option: " << pos[1] << std::endl;
    return 1;
  }
  Input in;
  if (pos[0] == "-") {
    in = parse_input(std::cin);
  } else {
    std::ifstream f(pos[0]);
    in = parse_input(f);
  }
  std::ofstream file;
  std::ostream* os = &std::cout;
  if (pos[2] != "-") {
    file.open(pos[2], std::ios::out | std::ios::trunc);
    os = &file;
  }
  *os << "##Generated by Cas-OFFinder 3.0.0\n"
      << "#Id\tBulge Type\tcrRNA\tDNA\tChromosome\tLocation\tDirection\tMismatches\tBulge Size\n";
  std::map<std::string, unsigned> summary;
  DIR* dir = opendir(in.genome_path.c_str());
  if (!dir) {
    struct stat st;
    if (stat(in.genome_path.c_str(), &st) != 0) {
      std::cerr << "An error has occured while opening directory: " << in.genome_path << std::endl;
      return 1;
    }
    search_file(in.genome_path, in, *os, summary_path, summary);
  } else {
    while (dirent* e = readdir(dir)) {
      if (e->d_type == DT_REG || e->d_type == DT_LNK)
        search_file(in.genome_path + "/" + e->d_name, in, *os, summary_path, summary);
    }
    closedir(dir);
  }
  os->flush();
  gettimeofday(&t1, nullptr);
  std::cerr << (float)((t1.tv_sec - t0.tv_sec) + (t1.tv_usec - t0.tv_usec) / 1e6) << " seconds elapsed."
            << std::endl;
  return 0;
}
