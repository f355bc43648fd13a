// cof-synth: writes a synthetic genome file (FASTA or 2BIT) from the record
// generator of synth.cpp, without loading libcasoff.so or touching a GPU.
//
//   cof-synth [--limit P] OUT SEED GC GC_DRIFT WINDOW N_FRAC RUN_MIN RUN_MAX NAME:LEN...
//
// Record k of the list is record k of the generator (cofx_synth_record with
// the given parameters), so a list of the leading records of a genome writes
// byte for byte that genome's prefix.  --limit P writes only the first P
// positions of the genome string (records joined by one separator each): the
// record that reaches P is cut there (it is still generated at its full
// length, because its N runs depend on that length) and later records are
// left out.  OUT ending in ".2bit" gives a UCSC
// 2BIT file (version 0, little-endian, non-ACGT bytes as N blocks, no mask
// blocks); anything else gives FASTA with 60 bases per line.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/cof_tools.h"

namespace {

struct Record {
  std::string name;
  uint64_t len;
};

bool put_u32(FILE* f, uint32_t v) {
  const unsigned char b[4] = {(unsigned char)v, (unsigned char)(v >> 8), (unsigned char)(v >> 16),
                              (unsigned char)(v >> 24)};
  return fwrite(b, 1, 4, f) == 4;
}

bool write_fasta_record(FILE* f, const Record& r, const std::vector<char>& seq) {
  if (fprintf(f, ">%s\n", r.name.c_str()) < 0) return false;
  for (uint64_t p = 0; p < r.len; p += 60) {
    const uint64_t k = r.len - p < 60 ? r.len - p : 60;
    if (fwrite(seq.data() + p, 1, k, f) != k || fputc('\n', f) == EOF) return false;
  }
  return true;
}

int code_of(char c) {
  switch (c) {
    case 'T': return 0;
    case 'C': return 1;
    case 'A': return 2;
    case 'G': return 3;
    default: return -1;
  }
}

// One 2BIT record: dnaSize, N blocks (runs of non-ACGT bytes), no mask
// blocks, reserved word, then 2-bit codes four to a byte, first base in the
// most significant bits.
bool write_twobit_record(FILE* f, const Record& r, const std::vector<char>& seq) {
  std::vector<uint32_t> starts, sizes;
  for (uint64_t p = 0; p < r.len;) {
    if (code_of(seq[p]) >= 0) {
      ++p;
      continue;
    }
    uint64_t q = p;
    while (q < r.len && code_of(seq[q]) < 0) ++q;
    starts.push_back((uint32_t)p);
    sizes.push_back((uint32_t)(q - p));
    p = q;
  }
  bool ok = put_u32(f, (uint32_t)r.len) && put_u32(f, (uint32_t)starts.size());
  for (uint32_t v : starts) ok = ok && put_u32(f, v);
  for (uint32_t v : sizes) ok = ok && put_u32(f, v);
  ok = ok && put_u32(f, 0) && put_u32(f, 0);
  std::vector<unsigned char> packed((r.len + 3) / 4, 0);
  for (uint64_t p = 0; p < r.len; ++p) {
    const int c = code_of(seq[p]);
    packed[p >> 2] |= (unsigned char)((c < 0 ? 0 : c) << (6 - 2 * (p & 3)));
  }
  return ok && fwrite(packed.data(), 1, packed.size(), f) == packed.size();
}

}  // namespace

int main(int argc, char** argv) {
  uint64_t limit = ~0ull;
  if (argc > 2 && strcmp(argv[1], "--limit") == 0) {
    limit = strtoull(argv[2], nullptr, 10);
    argc -= 2;
    argv += 2;
  }
  if (argc < 10) {
    fprintf(stderr, "usage: cof-synth [--limit P] OUT SEED GC GC_DRIFT WINDOW N_FRAC RUN_MIN RUN_MAX NAME:LEN...\n");
    return 2;
  }
  const std::string out = argv[1];
  const uint64_t seed = strtoull(argv[2], nullptr, 10);
  const double gc = atof(argv[3]), drift = atof(argv[4]);
  const uint32_t window = (uint32_t)strtoul(argv[5], nullptr, 10);
  const double nfrac = atof(argv[6]);
  const uint32_t run_min = (uint32_t)strtoul(argv[7], nullptr, 10), run_max = (uint32_t)strtoul(argv[8], nullptr, 10);
  std::vector<Record> recs;
  for (int i = 9; i < argc; ++i) {
    const char* colon = strrchr(argv[i], ':');
    if (!colon || colon == argv[i]) {
      fprintf(stderr, "cof-synth: bad record %s (want NAME:LEN)\n", argv[i]);
      return 2;
    }
    recs.push_back(Record{std::string(argv[i], colon - argv[i]), strtoull(colon + 1, nullptr, 10)});
  }
  // Records past the limit are dropped; the one that reaches it is cut when written.
  std::vector<uint64_t> keep;  // written length of each record
  for (uint64_t pos = 0, k = 0; k < recs.size() && (k == 0 || pos < limit); ++k) {
    const uint64_t room = limit > pos ? limit - pos : 0;
    keep.push_back(recs[k].len < room ? recs[k].len : room);
    pos += recs[k].len + 1;
  }
  if (keep.size() < recs.size()) recs.resize(keep.size());
  const bool twobit = out.size() > 5 && out.compare(out.size() - 5, 5, ".2bit") == 0;
  FILE* f = fopen(out.c_str(), "wb");
  if (!f) {
    perror(out.c_str());
    return 1;
  }
  bool ok = true;
  long index_pos = 0;
  if (twobit) {
    ok = put_u32(f, 0x1A412743u) && put_u32(f, 0) && put_u32(f, (uint32_t)recs.size()) && put_u32(f, 0);
    index_pos = ftell(f);
    for (const Record& r : recs) {  // offsets are filled in once the records are written
      const unsigned char n = (unsigned char)r.name.size();
      ok = ok && fwrite(&n, 1, 1, f) == 1 && fwrite(r.name.data(), 1, n, f) == n && put_u32(f, 0);
    }
  }
  std::vector<uint32_t> offsets;
  std::vector<char> seq;
  for (size_t k = 0; ok && k < recs.size(); ++k) {
    seq.assign(recs[k].len, 'N');
    if (recs[k].len)
      cofx_synth_record(seed, (uint32_t)k, recs[k].len, gc, drift, window, nfrac, run_min, run_max, seq.data());
    const Record cut{recs[k].name, keep[k]};
    offsets.push_back((uint32_t)ftell(f));
    ok = twobit ? write_twobit_record(f, cut, seq) : write_fasta_record(f, cut, seq);
  }
  if (ok && twobit) {
    ok = fseek(f, index_pos, SEEK_SET) == 0;
    for (size_t k = 0; ok && k < recs.size(); ++k) {
      const unsigned char n = (unsigned char)recs[k].name.size();
      ok = fseek(f, 1 + n, SEEK_CUR) == 0 && put_u32(f, offsets[k]);
    }
  }
  if (fclose(f) != 0) ok = false;
  if (!ok) {
    fprintf(stderr, "cof-synth: write failed: %s\n", out.c_str());
    return 1;
  }
  return 0;
}
