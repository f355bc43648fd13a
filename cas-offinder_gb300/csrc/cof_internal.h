// Internal host-side types shared by the input parser, the genome loaders and
// the CUDA engine of libcasoff.so.  Not part of the public ABI (include/cof.h).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace cof {

// ---------------------------------------------------------------- genome planes
// Every genome byte is one position; position p lives in bit (p & 31) of word
// (p >> 5) of three planes:
//   ot = 0: a base, (hi, lo) = the 2BIT code  T=00 C=01 A=10 G=11
//   ot = 1: not a base, (hi, lo) = 00 'N' | 01 ';' (record separator) |
//           10 another byte, kept in the exception list (position, byte).
// With this code the complement of a base flips `hi` only.  Positions past
// the end of the genome read as separators, so no window crosses the end.
constexpr uint64_t kPlanePadWords = 4;  // words of separators after the last position

inline uint64_t plane_words(uint64_t n) { return (n + 31) / 32 + kPlanePadWords; }

struct PackedGenome {
  uint64_t n = 0;                         // positions (bytes of the reference string)
  std::vector<uint32_t> hi, lo, ot;       // plane_words(n) each
  std::vector<uint64_t> exc_pos;          // ascending
  std::vector<uint8_t> exc_byte;
  std::vector<std::string> names;         // record names (m_chrnames)
  std::vector<uint64_t> starts;           // record start offsets (m_chrpos)
};

// Packs the reference's genome string.  Multi-threaded over words.
void pack_text(const char* seq, uint64_t n, uint32_t* hi, uint32_t* lo, uint32_t* ot,
               std::vector<uint64_t>* exc_pos, std::vector<uint8_t>* exc_byte);
// Marks [n, plane_words(n)*32) as separators.
void pad_planes(uint64_t n, uint32_t* hi, uint32_t* lo, uint32_t* ot);

// Loaders.  Return 0 on success, 1 when the file is not of that format.
int load_fasta(const std::string& path, PackedGenome& g);
int load_twobit(const std::string& path, PackedGenome& g);

// ---------------------------------------------------------------- input file
struct BulgeRecord {
  std::string what;  // DNA-bulge size in decimal ("0": none) or the deleted RNA bases
  int index;         // gap position in the guide; negative when the PAM is 5'
};

struct Variant {
  std::string key;       // the compare string (length L)
  std::string id;        // id of the first guide that produced the key
  uint16_t threshold;    // its mismatch limit (the reference stores cl_ushort)
  std::vector<BulgeRecord> bulges;
  uint32_t order = 0;    // rank of its first insertion among the file's variants
};

// One output row shape for (variant, bulge record, strand).  `head` is
// "id\ttype\tcrRNA\t"; `dna` is the DNA column where bytes >= 0x80 stand for
// oriented window position (byte - 0x80) and other bytes are literal; `tail`
// is "size\n".  Location = hit position - record start + offset.
struct RowShape {
  std::string head, dna, tail;
  int64_t offset;
  std::string type;      // "X", "DNA" or "RNA" (summary table key)
  unsigned bulge_size;
};

struct Job {
  std::string genome_path;
  std::string pattern;        // with DNA-bulge padding, upper case
  unsigned dna = 0, rna = 0;
  bool pam5 = false;          // PAM written first (first pattern byte not 'N')
  std::vector<Variant> variants;                // std::map key order
  // shapes[v][s] lists variant v's rows for strand s (0 '+', 1 '-') in bulge order.
  std::vector<std::vector<RowShape>> shapes[2];
};

// Parses an input file (the whole text).  On error returns false and sets
// `err` to the reference's message.
bool parse_job(const char* text, size_t len, Job& job, std::string& err);
// Builds the row shapes of every variant.  False (and `err`) if the
// reference's string surgery would throw.
bool build_shapes(Job& job, std::string& err);

// IUPAC mismatch predicate of the reference (pattern byte p vs genome byte g).
bool mismatch(unsigned char p, unsigned char g);
unsigned char complement_byte(unsigned char c);

}  // namespace cof
