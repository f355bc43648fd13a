// Bit-sliced comparer: host dispatch (launch_comparer_bs) and the shared
// table geometry.  The kernels are in comparer_bs.cuh, instantiated by
// comparer_bs_inst.cu.
#include "kernels.cuh"

namespace cof {
namespace bs {
// Launches the instance for `slots` (8..32); false when none fits.
template <int ROW, int NK, bool CONC>
bool dispatch_s(int slots, const GenomeView& g, const uint32_t* queue, const uint32_t* qcount, uint64_t seg_pos0,
                const uint32_t* prog, const uint32_t* pgid, uint32_t chunks, uint32_t m, bool narrow, uint32_t L,
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

namespace {
// LOP3-class instructions of CountTree<N, LEV, NB> (comparer_bs.cuh) that
// survive dead-code elimination: a level's sums (xor3 / xor) only while LEV <
// NB, its carries (maj3 / and) only while LEV + 1 < NB.
int tree_ops(int N, int LEV, int NB) {
  if (N <= 1) return 0;
  const int fa = N >= 3 ? (N - 1) / 2 : 0, left = N - 2 * fa, carry = fa + (left == 2 ? 1 : 0);
  const int per = (LEV < NB ? 1 : 0) + (LEV + 1 < NB ? 1 : 0);
  return (fa + (left == 2 ? 1 : 0)) * per + tree_ops(carry, LEV + 1, NB);
}
int width_of(int s) { return s <= 1 ? 1 : 1 + width_of(s >> 1); }
}  // namespace

double bs_lane_lop3(int slots, uint32_t m, bool narrow) {
  const int NB = width_of(slots);
  double ops = 2.0 * tree_ops(slots, 0, NB);  // full count of the first variant, groups a and b
  if (m <= 1) return ops + 2.0 * NB;          // carry of count + bias, per group
  const int NP = narrow ? NB : NB + 1;        // count planes (launch_bs: narrow only for m > 1)
  ops += 2.0 * (NB + NP - 1);                 // add_bias: xor3 per plane, maj3 per carry kept, per group
  const uint32_t ns = m - 1;
  ops += (double)ns * 2 * (2 * NP);           // step_update: t = a ^ b, NP xors, NP - 1 lop3, per group
  ops += (double)(ns / 2) * 3 + (ns & 1);     // votes: t0, t1, t0 & t1 per pair of steps; one for a lone step
  return ops;
}

bool bs_narrow_ok(int slots, const uint32_t* thresholds, const uint32_t* positions, size_t n) {
  const uint32_t half = 1u << (width_of(slots) - 1);
  for (size_t i = 0; i < n; ++i)
    if (thresholds[i] >= half || positions[i] > thresholds[i] + half) return false;
  return true;
}

bool launch_comparer_bs(const GenomeView& g, const uint32_t* queue, const uint32_t* qcount, uint64_t seg_pos0,
                        const uint32_t* prog, const uint32_t* pgid, uint32_t chunks, uint32_t m, int slots,
                        bool narrow, uint32_t L, bool concrete_only, uint32_t* tile_ctr, uint64_t* hits,
                        unsigned long long* hit_count, uint64_t hit_cap, int sm_count, cudaStream_t stream) {
  if (chunks == 0) return true;
  if (seg_pos0 & 31) return false;  // the kernels address windows from the segment's first plane word
#define COF_BS_ROW(ROWV, NKV)                                                                                       \
  return concrete_only ? dispatch_s<ROWV, NKV, true>(slots, g, queue, qcount, seg_pos0, prog, pgid, chunks, m, narrow, L,  \
                                                      tile_ctr, hits, hit_count, hit_cap, sm_count, stream)         \
                       : dispatch_s<ROWV, NKV, false>(slots, g, queue, qcount, seg_pos0, prog, pgid, chunks, m, narrow, L, \
                                                       tile_ctr, hits, hit_count, hit_cap, sm_count, stream);
  if (L <= 32) COF_BS_ROW(36, 1)
  if (L <= 36) COF_BS_ROW(36, 2)
  if (L <= 64) COF_BS_ROW(68, 2)
#undef COF_BS_ROW
  return false;
}

}  // namespace cof
