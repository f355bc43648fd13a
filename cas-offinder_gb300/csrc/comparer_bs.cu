// Bit-sliced comparer: host dispatch (launch_comparer_bs) and the shared
// table geometry.  The kernels are in comparer_bs.cuh, instantiated by
// comparer_bs_inst.cu.
#include "kernels.cuh"

namespace cof {
namespace bs {
// Launches the instance for `slots` (8..32); false when none fits.
template <int ROW, int NK, bool CONC>
bool dispatch_s(int slots, const GenomeView& g, const uint32_t* queue, const uint32_t* qcount, uint64_t seg_pos0,
                const uint32_t* prog, const uint32_t* pgid, uint32_t chunks, uint32_t m, uint32_t L,
                uint32_t* tile_ctr, uint64_t* hits, unsigned long long* hit_count, uint64_t hit_cap, int sm_count,
                cudaStream_t stream);
}  // namespace bs
using bs::dispatch_s;

int bs_slots_for(int max_positions) {
  if (max_positions > 32) return 0;
  int s = max_positions < 8 ? 8 : ((max_positions + 3) / 4) * 4;
  return s;
}

int bs_row_for(uint32_t L) { return L <= 36 ? 36 : 68; }

uint32_t bs_class_of(unsigned char p) {
  switch (p) {
    case 'T': return 1;
    case 'C': return 2;
    case 'A': return 3;
    case 'G': return 4;
    case 'V': return 5;
    case 'D': return 6;
    case 'B': return 7;
    case 'H': return 8;
    case 'R': return 9;
    case 'Y': return 10;
    case 'K': return 11;
    case 'M': return 12;
    case 'W': return 13;
    case 'S': return 14;
    default: return 0;
  }
}

bool launch_comparer_bs(const GenomeView& g, const uint32_t* queue, const uint32_t* qcount, uint64_t seg_pos0,
                        const uint32_t* prog, const uint32_t* pgid, uint32_t chunks, uint32_t m, int slots,
                        uint32_t L, bool concrete_only, uint32_t* tile_ctr, uint64_t* hits,
                        unsigned long long* hit_count, uint64_t hit_cap, int sm_count, cudaStream_t stream) {
  if (chunks == 0) return true;
  if (seg_pos0 & 31) return false;  // the kernels address windows from the segment's first plane word
#define COF_BS_ROW(ROWV, NKV)                                                                                       \
  return concrete_only ? dispatch_s<ROWV, NKV, true>(slots, g, queue, qcount, seg_pos0, prog, pgid, chunks, m, L,  \
                                                      tile_ctr, hits, hit_count, hit_cap, sm_count, stream)         \
                       : dispatch_s<ROWV, NKV, false>(slots, g, queue, qcount, seg_pos0, prog, pgid, chunks, m, L, \
                                                       tile_ctr, hits, hit_count, hit_cap, sm_count, stream);
  if (L <= 32) COF_BS_ROW(36, 1)
  if (L <= 36) COF_BS_ROW(36, 2)
  if (L <= 64) COF_BS_ROW(68, 2)
#undef COF_BS_ROW
  return false;
}

}  // namespace cof
