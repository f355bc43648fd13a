// Bit-sliced comparer: replaces comparer/comparer_cpu (cas-offinder.cl:73-155,
// :214-286) for compare variants with at most 32 positions that can mismatch.
//
// Work unit: a tile of 32*W strand-oriented candidates (W groups of 32, one
// per warp; W = ceil(variants / 32), at most 8) against every compare variant.
//  1. Build: warp w takes group w.  Lane c extracts candidate c's oriented
//     window from the genome planes (prefetched one tile ahead); three 32x32
//     bit transposes (shuffles) turn the 32 windows into per-position words
//     whose bit c is candidate c.  Lane k then writes, for window position k,
//     the 14 "class words": for each kind of pattern byte (concrete base,
//     3-base code, 2-base code), the 32-candidate bit mask of mismatches at
//     that position.  One LOP3 each.  Groups 2p and 2p+1 share one uint2 slot,
//     so one 64-bit shared load serves 64 candidates (an odd last group is
//     counted alone).  Two table buffers: tile t+1 is built while tile t is
//     counted, one barrier per tile.
//  2. Count: each lane owns one compare variant, described by the list of its
//     positions that can mismatch as shared-memory offsets of the matching
//     class word (N positions are skipped).  For a group pair, the lane loads
//     one uint2 per listed position and adds the words bit-sliced with a
//     carry-save full-adder tree (2 LOP3 per word), so the candidates'
//     mismatch counts come out as 5-6 bit planes.  A carry chain against the
//     variant's threshold gives the hit mask; hits (rare) decode their exact
//     count from the planes.
// Per lane and 64 candidates: S loads + ~4S LOP3 + ~12 for 64 variant tests.
#include <algorithm>
#include <type_traits>

#include "kernels.cuh"

namespace cof {

namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr int kGroups = 8;    // groups of 32 candidates per tile, at most
constexpr int kMaxWarps = 8;  // warps per block (one group each)

// One LOP3 with truth table LUT over (a, b, c) = (0xF0, 0xCC, 0xAA).
template <uint32_t LUT>
__device__ __forceinline__ uint32_t lop3(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t d;
  asm("lop3.b32 %0, %1, %2, %3, %4;" : "=r"(d) : "r"(a), "r"(b), "r"(c), "n"(LUT));
  return d;
}
__device__ __forceinline__ uint32_t maj3(uint32_t a, uint32_t b, uint32_t c) { return lop3<0xE8>(a, b, c); }
__device__ __forceinline__ uint32_t xor3(uint32_t a, uint32_t b, uint32_t c) { return lop3<0x96>(a, b, c); }

// 32x32 bit transpose across the warp: lane i holds row i; afterwards lane i
// holds column i (bit j = bit i of row j).
__device__ __forceinline__ uint32_t warp_transpose(uint32_t x, unsigned lane) {
#pragma unroll
  for (int j = 16; j > 0; j >>= 1) {
    const uint32_t m = j == 16 ? 0x0000FFFFu : j == 8 ? 0x00FF00FFu : j == 4 ? 0x0F0F0F0Fu : j == 2 ? 0x33333333u
                                                                                                    : 0x55555555u;
    const bool upper = (lane & j) != 0;
    const uint32_t y = __shfl_xor_sync(kFull, x, j);
    // upper lanes take the partner's bits shifted down, lower lanes shifted up;
    // a rotate moves them in both cases without touching the kept half.
    const uint32_t r = __funnelshift_l(y, y, upper ? 32 - j : j);
    const uint32_t keep = upper ? ~m : m;
    x = lop3<0xE2>(x, keep, r);  // (x & keep) | (r & ~keep)
  }
  return x;
}



// Reduces N bit-sliced one-bit inputs of weight 2^LEV to binary planes.
template <int N, int LEV, int NB>
struct CountTree {
  static constexpr int kFA = N >= 3 ? (N - 1) / 2 : 0;
  static constexpr int kLeft = N - 2 * kFA;
  static constexpr int kCarry = kFA + (kLeft == 2 ? 1 : 0);
  __device__ __forceinline__ static void run(const uint32_t* v, uint32_t* bits) {
    uint32_t c[kCarry > 0 ? kCarry : 1];
    uint32_t acc = v[0];
#pragma unroll
    for (int f = 0; f < kFA; ++f) {
      const uint32_t a = v[1 + 2 * f], b = v[2 + 2 * f];
      c[f] = maj3(acc, a, b);
      acc = xor3(acc, a, b);
    }
    if (kLeft == 2) {
      c[kFA] = acc & v[N - 1];
      acc ^= v[N - 1];
    }
    if (LEV < NB) bits[LEV] = acc;
    CountTree<kCarry, LEV + 1, NB>::run(c, bits);
  }
};
template <int LEV, int NB>
struct CountTree<1, LEV, NB> {
  __device__ __forceinline__ static void run(const uint32_t* v, uint32_t* bits) {
    if (LEV < NB) bits[LEV] = v[0];
#pragma unroll
    for (int i = LEV + 1; i < NB; ++i) bits[i] = 0;
  }
};
template <int LEV, int NB>
struct CountTree<0, LEV, NB> {
  __device__ __forceinline__ static void run(const uint32_t*, uint32_t* bits) {
#pragma unroll
    for (int i = LEV; i < NB; ++i) bits[i] = 0;
  }
};

__host__ __device__ constexpr int bit_width(int s) { return s <= 1 ? 1 : 1 + bit_width(s >> 1); }

// Raw genome words of one candidate window, loaded one tile ahead.
template <int NK>
struct RawWindow {
  uint32_t e;
  uint32_t h[NK + 1], l[NK + 1], o[NK + 1];
};

template <int NK>
__device__ __forceinline__ void load_raw(RawWindow<NK>& r, const uint32_t* __restrict__ hi,
                                         const uint32_t* __restrict__ lo, const uint32_t* __restrict__ ot,
                                         const uint32_t* __restrict__ queue, uint32_t idx, uint32_t n,
                                         uint64_t seg_pos0) {
  r.e = 0xFFFFFFFFu;  // no candidate
#pragma unroll
  for (int i = 0; i <= NK; ++i) r.h[i] = r.l[i] = r.o[i] = 0;
  if (idx < n) {
    r.e = queue[idx];
    const uint64_t w = (seg_pos0 + (r.e >> 1)) >> 5;
#pragma unroll
    for (int i = 0; i <= NK; ++i) {
      r.h[i] = hi[w + i];
      r.l[i] = lo[w + i];
      r.o[i] = ot[w + i];
    }
  }
}

// Builds group g of a tile: oriented windows of 32 candidates (from `raw`),
// transposed, expanded to class words in `pair_table` (.x for even g, .y for
// odd g) and candidate entries in `ents`.  `concrete_only`: the variants use
// only A/C/G/T (and N), so the ten degenerate-code rows are not needed.
template <int NK, int ROW>
__device__ __forceinline__ void build_group(const RawWindow<NK>& raw, uint64_t seg_pos0, uint32_t L, unsigned lane,
                                            uint2* pair_table, unsigned half, uint32_t* ents, bool concrete_only) {
  uint32_t hw[NK], lw[NK], ow[NK];
  const bool have = raw.e != 0xFFFFFFFFu;
  const unsigned r = have ? (unsigned)((seg_pos0 + (raw.e >> 1)) & 31) : 0u;
#pragma unroll
  for (int i = 0; i < NK; ++i) {
    hw[i] = __funnelshift_r(raw.h[i], raw.h[i + 1], r);
    lw[i] = __funnelshift_r(raw.l[i], raw.l[i + 1], r);
    ow[i] = __funnelshift_r(raw.o[i], raw.o[i + 1], r);
  }
  if (have && (raw.e & 1)) {
    // Reverse complement: reverse the L positions, flip hi of bases.
    if (NK == 1) {
      const unsigned sh = 32 - L;
      hw[0] = ~(__brev(hw[0]) >> sh) & (0xFFFFFFFFu >> sh);
      lw[0] = __brev(lw[0]) >> sh;
      ow[0] = __brev(ow[0]) >> sh;
    } else {
      const unsigned sh = 64 - L;
      const uint64_t mask = ~0ull >> sh;
      const uint64_t H = ~(__brevll(((uint64_t)hw[NK - 1] << 32) | hw[0]) >> sh) & mask;
      const uint64_t Lo = __brevll(((uint64_t)lw[NK - 1] << 32) | lw[0]) >> sh;
      const uint64_t O = __brevll(((uint64_t)ow[NK - 1] << 32) | ow[0]) >> sh;
      hw[0] = (uint32_t)H;
      hw[NK - 1] = (uint32_t)(H >> 32);
      lw[0] = (uint32_t)Lo;
      lw[NK - 1] = (uint32_t)(Lo >> 32);
      ow[0] = (uint32_t)O;
      ow[NK - 1] = (uint32_t)(O >> 32);
    }
  }
  ents[lane] = raw.e;
  uint32_t* tg = (uint32_t*)pair_table + half;
#pragma unroll
  for (int i = 0; i < NK; ++i) {
    const uint32_t h = warp_transpose(hw[i], lane);
    const uint32_t l = warp_transpose(lw[i], lane);
    const uint32_t o = warp_transpose(ow[i], lane);
    const unsigned k = i * 32 + lane;
    if (k < (unsigned)ROW) {
      // One LOP3 of (h, l, o) each; truth tables over (0xF0, 0xCC, 0xAA).
      tg[2 * (1 * ROW + k)] = lop3<0xFE>(h, l, o);  // T: h | l | o (mismatch unless T)
      tg[2 * (2 * ROW + k)] = lop3<0xFB>(h, l, o);  // C: h | ~l | o
      tg[2 * (3 * ROW + k)] = lop3<0xEF>(h, l, o);  // A: ~h | l | o
      tg[2 * (4 * ROW + k)] = lop3<0xBF>(h, l, o);  // G: ~h | ~l | o
      if (!concrete_only) {
        tg[2 * (5 * ROW + k)] = lop3<0x01>(h, l, o);   // V: ~h & ~l & ~o (mismatch only T)
        tg[2 * (6 * ROW + k)] = lop3<0x04>(h, l, o);   // D: ~h & l & ~o (only C)
        tg[2 * (7 * ROW + k)] = lop3<0x10>(h, l, o);   // B: h & ~l & ~o (only A)
        tg[2 * (8 * ROW + k)] = lop3<0x40>(h, l, o);   // H: h & l & ~o (only G)
        tg[2 * (9 * ROW + k)] = lop3<0x05>(h, l, o);   // R: ~h & ~o (C or T)
        tg[2 * (10 * ROW + k)] = lop3<0x50>(h, l, o);  // Y: h & ~o (A or G)
        tg[2 * (11 * ROW + k)] = lop3<0x14>(h, l, o);  // K: (h ^ l) & ~o (A or C)
        tg[2 * (12 * ROW + k)] = lop3<0x41>(h, l, o);  // M: ~(h ^ l) & ~o (G or T)
        tg[2 * (13 * ROW + k)] = lop3<0x44>(h, l, o);  // W: l & ~o (C or G)
        tg[2 * (14 * ROW + k)] = lop3<0x11>(h, l, o);  // S: ~l & ~o (A or T)
      }
    }
  }
}

// The compare variant of a lane: its slot offsets (two u16 per word), the
// carry constant of its threshold test and its id (inactive lanes get no hits).
template <int S>
__device__ __forceinline__ void load_variant(const uint32_t* __restrict__ voff, const uint32_t* __restrict__ vthr,
                                             const uint32_t* __restrict__ vgid, uint32_t nvar, uint32_t v,
                                             uint32_t (&packed)[S / 2], uint32_t& kadd, uint32_t& gid, bool& active) {
  constexpr int NB = bit_width(S);
  active = v < nvar;
#pragma unroll
  for (int s = 0; s < S / 2; ++s) packed[s] = active ? voff[(size_t)v * (S / 2) + s] : 0u;
  // count > thr  <=>  count + (2^NB - 1 - thr) carries out of NB bits.
  const uint32_t thr = active ? min(vthr[v], (uint32_t)((1u << NB) - 1)) : 0u;
  kadd = (1u << NB) - 1 - thr;
  gid = active ? vgid[v] : 0u;
}

// Counts one lane's variant against the G groups of a tile and appends hits.
template <int S, int ROW>
__device__ __forceinline__ void count_tile(const uint32_t (&packed)[S / 2], uint32_t kadd, uint32_t gid, bool active,
                                           const uint2* table, const uint32_t* ents, uint32_t ntile, unsigned G,
                                           const uint32_t (&gvalid)[kGroups], uint64_t seg_pos0,
                                           uint64_t* __restrict__ hits, unsigned long long* __restrict__ hit_count,
                                           uint64_t hit_cap) {
  constexpr int NB = bit_width(S);
  constexpr int kPairWords = 16 * ROW;
  uint32_t kmask[NB];  // bit i of the threshold constant as an all-ones / all-zeros word
#pragma unroll
  for (int i = 0; i < NB; ++i) kmask[i] = 0u - ((kadd >> i) & 1u);
  const uint32_t lane_on = active ? kFull : 0u;
  uint32_t off[S];
#pragma unroll
  for (int s = 0; s < S; s += 2) {
    off[s] = packed[s / 2] & 0xFFFFu;
    off[s + 1] = packed[s / 2] >> 16;
  }
#pragma unroll
  for (int p = 0; p < kGroups / 2; ++p) {
    if ((unsigned)(2 * p) >= G || (uint32_t)p * 64 >= ntile) break;
    const char* base = (const char*)(table + p * kPairWords);
    if ((unsigned)(2 * p + 1) == G) {  // odd last group: counted alone
      uint32_t xa[S];
#pragma unroll
      for (int s = 0; s < S; ++s) xa[s] = *(const uint32_t*)(base + off[s]);
      uint32_t ba[NB];
      CountTree<S, 0, NB>::run(xa, ba);
      uint32_t ca = 0;
#pragma unroll
      for (int i = 0; i < NB; ++i) ca = maj3(ba[i], kmask[i], ca);
      uint32_t hm = ~ca & gvalid[2 * p] & lane_on;
      while (hm) {
        const unsigned c = __ffs(hm) - 1;
        hm &= hm - 1;
        uint32_t mm = 0;
#pragma unroll
        for (int i = 0; i < NB; ++i) mm |= ((ba[i] >> c) & 1u) << i;
        const uint32_t e = ents[2 * p * 32 + c];
        const unsigned long long at = atomicAdd(hit_count, 1ull);
        if (at < hit_cap) hits[at] = make_hit(gid, seg_pos0 + (e >> 1), e & 1, mm);
      }
      break;
    }
    uint32_t xa[S], xb[S];
#pragma unroll
    for (int s = 0; s < S; ++s) {
      const uint2 w2 = *(const uint2*)(base + off[s]);
      xa[s] = w2.x;
      xb[s] = w2.y;
    }
    uint32_t ba[NB], bb[NB];
    CountTree<S, 0, NB>::run(xa, ba);
    CountTree<S, 0, NB>::run(xb, bb);
    uint32_t ca = 0, cb = 0;
#pragma unroll
    for (int i = 0; i < NB; ++i) {
      ca = maj3(ba[i], kmask[i], ca);
      cb = maj3(bb[i], kmask[i], cb);
    }
    const uint32_t hita = ~ca & gvalid[2 * p] & lane_on, hitb = ~cb & gvalid[2 * p + 1] & lane_on;
    if (hita | hitb) {
#pragma unroll
      for (int half = 0; half < 2; ++half) {
        uint32_t hm = half ? hitb : hita;
        const uint32_t* bp = half ? bb : ba;
        while (hm) {
          const unsigned c = __ffs(hm) - 1;
          hm &= hm - 1;
          uint32_t mm = 0;
#pragma unroll
          for (int i = 0; i < NB; ++i) mm |= ((bp[i] >> c) & 1u) << i;
          const uint32_t e = ents[(2 * p + half) * 32 + c];
          const unsigned long long at = atomicAdd(hit_count, 1ull);
          if (at < hit_cap) hits[at] = make_hit(gid, seg_pos0 + (e >> 1), e & 1, mm);
        }
      }
    }
  }
}

template <int S, int ROW, int NK>
__global__ void __launch_bounds__(32 * kMaxWarps, (S <= 20 ? 4 : S <= 28 ? 3 : 2)) comparer_bs_kernel(
    const uint32_t* __restrict__ hi, const uint32_t* __restrict__ lo, const uint32_t* __restrict__ ot,
    const uint32_t* __restrict__ queue, const uint32_t* __restrict__ qcount, uint64_t seg_pos0,
    const uint32_t* __restrict__ voff, const uint32_t* __restrict__ vthr, const uint32_t* __restrict__ vgid,
    uint32_t nvar, uint32_t L, bool concrete_only, uint64_t* __restrict__ hits,
    unsigned long long* __restrict__ hit_count, uint64_t hit_cap) {
  constexpr int NB = bit_width(S);          // planes of a count in [0, S]
  constexpr int kPairWords = 16 * ROW;      // uint2 elements per group pair
  constexpr int kBufWords = (kGroups / 2) * kPairWords;
  extern __shared__ uint2 smem2[];
  uint2* tables = smem2;                                        // [2 buffers][4 pairs][16][ROW]
  uint32_t* ents_all = (uint32_t*)(smem2 + 2 * kBufWords);      // [2 buffers][kGroups * 32]
  const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned G = blockDim.x >> 5;  // groups per tile = warps
  const unsigned tile_n = G * 32;

  // Rows 0 and 15 (pattern bytes that never mismatch) stay zero in both buffers.
  for (unsigned i = threadIdx.x; i < 2 * (kGroups / 2) * ROW; i += blockDim.x) {
    const unsigned p = i / ROW, k = i % ROW;
    tables[p * kPairWords + k] = make_uint2(0, 0);
    tables[p * kPairWords + 15 * ROW + k] = make_uint2(0, 0);
  }

  const uint32_t n = *qcount;
  const uint32_t ntiles = (n + tile_n - 1) / tile_n;
  uint32_t t = blockIdx.x;
  // With at most one variant per thread the lane's variant stays in registers
  // for the whole kernel.
  const bool one_chunk = nvar <= blockDim.x;
  uint32_t packed0[S / 2], kadd0 = 0, gid0 = 0;
  bool active0 = false;
  if (one_chunk) load_variant<S>(voff, vthr, vgid, nvar, warp * 32 + lane, packed0, kadd0, gid0, active0);
  RawWindow<NK> raw0;
  load_raw<NK>(raw0, hi, lo, ot, queue, t * tile_n + warp * 32 + lane, n, seg_pos0);
  if (t < ntiles)
    build_group<NK, ROW>(raw0, seg_pos0, L, lane, tables + (warp >> 1) * kPairWords, warp & 1, ents_all + warp * 32,
                         concrete_only);
  __syncthreads();
  // One tile per step; the step for buffer B counts from buffer B and builds
  // the next tile into buffer B^1.  Unrolled by two so that both buffers'
  // shared-memory addresses are compile-time constants.
  auto step = [&](auto bufc) {
    constexpr unsigned B = decltype(bufc)::value;
    // Loads of the next tile's windows are in flight during the count.
    const uint32_t tn = t + gridDim.x;
    load_raw<NK>(raw0, hi, lo, ot, queue, tn * tile_n + warp * 32 + lane, n, seg_pos0);
    const uint2* table = tables + B * kBufWords;
    const uint32_t* ents = ents_all + B * (kGroups * 32);
    const uint32_t ntile = min(tile_n, n - t * tile_n);
    uint32_t gvalid[kGroups];  // candidates present in each group of the tile
#pragma unroll
    for (int g = 0; g < kGroups; ++g) {
      const uint32_t have = ntile > (uint32_t)g * 32 ? ntile - (uint32_t)g * 32 : 0u;
      gvalid[g] = have >= 32 ? kFull : ((1u << have) - 1);
    }
    for (uint32_t vb = warp * 32; vb < nvar; vb += blockDim.x) {
      if (!one_chunk) load_variant<S>(voff, vthr, vgid, nvar, vb + lane, packed0, kadd0, gid0, active0);
      count_tile<S, ROW>(packed0, kadd0, gid0, active0, table, ents, ntile, G, gvalid, seg_pos0, hits, hit_count,
                         hit_cap);
    }
    if (tn < ntiles)
      build_group<NK, ROW>(raw0, seg_pos0, L, lane, tables + (B ^ 1) * kBufWords + (warp >> 1) * kPairWords, warp & 1,
                           ents_all + (B ^ 1) * (kGroups * 32) + warp * 32, concrete_only);
    __syncthreads();
  };
  while (t < ntiles) {
    step(std::integral_constant<unsigned, 0>());
    t += gridDim.x;
    if (t >= ntiles) break;
    step(std::integral_constant<unsigned, 1>());
    t += gridDim.x;
  }
}

template <int S, int ROW, int NK>
void launch_bs(const GenomeView& g, const uint32_t* queue, const uint32_t* qcount, uint64_t seg_pos0,
               const uint32_t* voff, const uint32_t* vthr, const uint32_t* vgid, uint32_t nvar, uint32_t L,
               bool concrete_only, uint64_t* hits, unsigned long long* hit_count, uint64_t hit_cap, int sm_count,
               cudaStream_t stream) {
  // Warps per block: enough lanes for every variant (so few lanes idle), at most 8.
  const int warps = (int)std::min<uint32_t>(kMaxWarps, (nvar + 31) / 32);
  const int threads = 32 * warps;
  const size_t smem = 2 * ((size_t)(kGroups / 2) * 16 * ROW * sizeof(uint2) + kGroups * 32 * 4);  // two buffers
  cudaFuncSetAttribute(comparer_bs_kernel<S, ROW, NK>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, comparer_bs_kernel<S, ROW, NK>, threads, smem) !=
          cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  comparer_bs_kernel<S, ROW, NK><<<sm_count * per_sm, threads, smem, stream>>>(
      g.hi, g.lo, g.ot, queue, qcount, seg_pos0, voff, vthr, vgid, nvar, L, concrete_only, hits, hit_count, hit_cap);
}

template <int ROW, int NK>
bool dispatch_s(int slots, const GenomeView& g, const uint32_t* queue, const uint32_t* qcount, uint64_t seg_pos0,
                const uint32_t* voff, const uint32_t* vthr, const uint32_t* vgid, uint32_t nvar, uint32_t L,
                bool concrete_only, uint64_t* hits, unsigned long long* hit_count, uint64_t hit_cap, int sm_count,
                cudaStream_t stream) {
#define COF_BS_CASE(SV)                                                                                       \
  case SV:                                                                                                    \
    launch_bs<SV, ROW, NK>(g, queue, qcount, seg_pos0, voff, vthr, vgid, nvar, L, concrete_only, hits,      \
                           hit_count, hit_cap, sm_count, stream);                                             \
    return true;
  switch (slots) {
    COF_BS_CASE(8)
    COF_BS_CASE(12)
    COF_BS_CASE(16)
    COF_BS_CASE(20)
    COF_BS_CASE(24)
    COF_BS_CASE(28)
    COF_BS_CASE(32)
    default:
      return false;
  }
#undef COF_BS_CASE
}

}  // namespace

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
                        const uint32_t* voff, const uint32_t* vthr, const uint32_t* vgid, uint32_t nvar, int slots,
                        uint32_t L, bool concrete_only, uint64_t* hits, unsigned long long* hit_count,
                        uint64_t hit_cap, int sm_count, cudaStream_t stream) {
  if (nvar == 0) return true;
  if (L <= 32) return dispatch_s<36, 1>(slots, g, queue, qcount, seg_pos0, voff, vthr, vgid, nvar, L, concrete_only,
                                        hits, hit_count, hit_cap, sm_count, stream);
  if (L <= 36) return dispatch_s<36, 2>(slots, g, queue, qcount, seg_pos0, voff, vthr, vgid, nvar, L, concrete_only,
                                        hits, hit_count, hit_cap, sm_count, stream);
  if (L <= 64) return dispatch_s<68, 2>(slots, g, queue, qcount, seg_pos0, voff, vthr, vgid, nvar, L, concrete_only,
                                        hits, hit_count, hit_cap, sm_count, stream);
  return false;
}

}  // namespace cof
