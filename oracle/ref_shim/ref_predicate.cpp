/*
 * Dumps the reference's IUPAC mismatch predicate as a 256x256 table.
 *
 * TEST INFRASTRUCTURE.  Compiles the reference's comparer_cpu kernel
 * (cas-offinder.cl:214-286) as C++, exactly as cl_host_emulator.cpp does,
 * and runs it on a one-byte compare string p against a chunk that holds every
 * byte value g once, forward strand only, with a threshold that keeps every
 * candidate.  The mismatch count it returns for position g is the predicate
 * mism(p, g) (cas-offinder.cl:30-43).  Output: 65536 bytes, row p, column g.
 * Usage: ref-predicate out.bin
 */
#include <atomic>
#include <cstdio>
#include <cstring>
#include <vector>

namespace refcl {
static thread_local size_t g_global_id = 0;
static inline size_t get_global_id(unsigned) { return g_global_id; }
static inline size_t get_group_id(unsigned) { return 0; }
static inline size_t get_local_size(unsigned) { return 1; }
static inline void barrier(int) {}
static inline unsigned int atomic_inc(unsigned int* p) { return (*p)++; }
#define CLK_LOCAL_MEM_FENCE 1
#define __kernel static
#define __global
#define __constant
#define __local
#pragma GCC diagnostic push
#pragma GCC diagnostic ignored "-Wunknown-pragmas"
#pragma GCC diagnostic ignored "-Wsign-compare"
#pragma GCC diagnostic ignored "-Wunused-function"
#include COF_REFERENCE_KERNELS
#pragma GCC diagnostic pop
}  // namespace refcl

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  std::vector<unsigned char> table(65536, 0);
  char chr[256];
  for (int g = 0; g < 256; ++g) chr[g] = (char)g;
  std::vector<unsigned int> loci(256), mm_loci(512);
  std::vector<char> flag(256, 1);  // forward strand only
  std::vector<unsigned short> mm_count(512);
  std::vector<char> direction(512);
  for (int g = 0; g < 256; ++g) loci[g] = (unsigned)g;
  for (int p = 0; p < 256; ++p) {
    char comp[2] = {(char)p, (char)p};       // compare string and its (unused) reverse complement
    int comp_index[2] = {p == 'N' ? -1 : 0, p == 'N' ? -1 : 0};  // set_seq_flags of a 1-byte string
    unsigned int count = 0;
    for (size_t i = 0; i < 256; ++i) {
      refcl::g_global_id = i;
      refcl::comparer_cpu(chr, loci.data(), mm_loci.data(), comp, comp_index, 1u, (unsigned short)1, flag.data(),
                          mm_count.data(), direction.data(), &count);
    }
    if (count != 256) return 3;
    for (unsigned int e = 0; e < count; ++e) table[p * 256 + mm_loci[e]] = (unsigned char)mm_count[e];
  }
  FILE* f = fopen(argv[1], "wb");
  if (!f) return 4;
  fwrite(table.data(), 1, table.size(), f);
  fclose(f);
  return 0;
}
