// Bit-sliced comparer: replaces comparer/comparer_cpu (cas-offinder.cl:73-155,
// :214-286) for compare variants with at most 32 positions that can mismatch.
//
// Work unit: a tile of 64*W strand-oriented candidates (W pairs of
// 32-candidate groups, W = warps per CTA, at most 8) against every compare
// variant of the pattern group.  CTAs are persistent: two tiles each, then
// tiles claimed from a per-launch counter.
//  1. Build: warp w builds pair w.  The pair's window words are copied into
//     shared memory one tile ahead (stage_pair: one 32-word span per plane
//     when the 64 windows lie within it, else each lane's own words).  Each
//     lane aligns its two windows to their first position, 32x32 bit
//     transposes (shuffles) turn the windows of a group into per-position
//     words whose bit c is candidate c, and the group's '-' strand windows
//     are turned into reverse complements in that form.  Lane k then writes,
//     for window position k, the class words: for each kind of pattern byte
//     (concrete base, 3-base code, 2-base code) the mismatch mask of the two
//     groups as one uint2 (one LOP3 each), so one 64-bit shared load serves
//     64 candidates.  Variants that use only A/C/G/T (and N) need 4 class
//     rows instead of 14, and the table shrinks to match.  Two table
//     buffers: tile t+1 is built while tile t is counted, one barrier per
//     tile.
//  2. Count: each lane runs a lane program (a chain of up to m compare
//     variants, built on the host, layout in kernels.cuh) on every pair of
//     the tile.  Its first variant is counted in full: one uint2 per
//     position that can mismatch ([register + immediate] shared addresses),
//     summed bit-sliced by a carry-save full-adder tree (explicit LOP3), plus
//     a bias so that the top plane is clear exactly where count <=
//     threshold.  Each later variant is reached by steps that add one class
//     word and remove one (an up/down ripple, 2 LOP3 per plane), two steps
//     per loop with one hit vote.  Hits (rare) decode their exact count from
//     the planes; entries past the end of the queue are dropped there, so
//     full and partial tiles run the same code.
//
// Kernel templates; comparer_bs_inst.cu instantiates them, once per
// (ROW, NK, CONC) object, so the instances compile in parallel.
#pragma once
#include <algorithm>
#include <type_traits>

#include "kernels.cuh"

namespace cof {
namespace bs {

namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;
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
// holds column i (bit j = bit i of row j).  Each stage j swaps j-bit blocks
// with lane i ^ j.  The 16- and 8-bit stages move whole bytes, so one byte
// permute of (x, partner) does the merge there (lower lanes keep their low
// blocks and take the partner's low blocks above them, upper lanes the
// reverse); the 4-, 2- and 1-bit stages rotate the partner's word and merge
// under a mask.
__device__ __forceinline__ uint32_t warp_transpose(uint32_t x, unsigned lane) {
  {
    const uint32_t y = __shfl_xor_sync(kFull, x, 16);
    x = __byte_perm(x, y, (lane & 16) ? 0x3276u : 0x5410u);
  }
  {
    const uint32_t y = __shfl_xor_sync(kFull, x, 8);
    x = __byte_perm(x, y, (lane & 8) ? 0x3715u : 0x6240u);
  }
#pragma unroll
  for (int j = 4; j > 0; j >>= 1) {
    const uint32_t m = j == 4 ? 0x0F0F0F0Fu : j == 2 ? 0x33333333u : 0x55555555u;
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

// Queue entry `idx` (0xFFFFFFFF past the end), loaded two tiles ahead.
__device__ __forceinline__ uint32_t load_entry(const uint32_t* __restrict__ queue, uint32_t idx, uint32_t n) {
  return idx < n ? queue[idx] : 0xFFFFFFFFu;
}

// Staging of window words in shared memory: per thread, two candidates x
// three planes x (NK + 1) words, slot-major ([slot][thread], slot stride =
// threads per block).
template <int NK>
struct Stage {
  static constexpr int kSlots = 3 * (NK + 1);  // per candidate
};

// 4-byte asynchronous global -> shared copy; `bytes` 0 writes a zero without
// reading the source.
__device__ __forceinline__ void cp_async4(uint32_t dst, const uint32_t* src, uint32_t bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(dst), "l"(src), "r"(bytes));
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Starts the copy of entry `e`'s window words (planes hi, lo, ot; NK + 1 words
// each) into the staging slots at shared address `dst` (slot stride kS
// bytes); a missing entry stages zeros.
template <int NK>
__device__ __forceinline__ void stage_planes(uint32_t dst, uint32_t kS, const uint32_t* __restrict__ hi,
                                             const uint32_t* __restrict__ lo, const uint32_t* __restrict__ ot,
                                             uint32_t e, uint32_t seg_w0) {
  const bool have = e != 0xFFFFFFFFu;
  const uint32_t w = have ? seg_w0 + (e >> 6) : 0u;
  const uint32_t bytes = have ? 4u : 0u;
#pragma unroll
  for (int i = 0; i <= NK; ++i) {
    cp_async4(dst + (0 * (NK + 1) + i) * kS, hi + w + i, bytes);
    cp_async4(dst + (1 * (NK + 1) + i) * kS, lo + w + i, bytes);
    cp_async4(dst + (2 * (NK + 1) + i) * kS, ot + w + i, bytes);
  }
}

// Reads back a staged window (after cp_async_wait_all); slot stride kS words.
template <int NK>
__device__ __forceinline__ void unstage(RawWindow<NK>& r, const uint32_t* st, uint32_t kS, uint32_t e) {
  r.e = e;
#pragma unroll
  for (int i = 0; i <= NK; ++i) {
    r.h[i] = st[(0 * (NK + 1) + i) * kS];
    r.l[i] = st[(1 * (NK + 1) + i) * kS];
    r.o[i] = st[(2 * (NK + 1) + i) * kS];
  }
}

// Window words of one pair (entry ea -> group a, eb -> group b), copied into
// shared memory asynchronously.  The 64 entries are consecutive in the queue,
// which the finder fills in genome order, so their windows nearly always lie
// within a few plane words: when every window lies in [w0, w0 + 32), lane l
// copies word w0 + l of each plane (three copies of consecutive words per
// warp; a gather of each lane's own words would copy the same few words many
// times over, one L1 wavefront per distinct word) and `meta` records w0.
// Otherwise -- a pair where two finder warps' queue ranges meet, or windows
// spread out around a run of N -- each lane copies its own candidates' words
// into its slots and `meta` records kNoWindow.  Only the words the windows
// cover are read.  The same warp reads `meta` back after the copies land.
constexpr uint32_t kNoWindow = 0xFFFFFFFFu;
constexpr int kWindowWords = 32;  // per plane
constexpr int kCoopWords = 4 * kWindowWords;  // per warp: three planes, then meta

// The pair's entries go to `ents` (its 64 entry slots), where unstage_pair
// reads them back, so they hold no registers while the current tile is
// counted.
template <int NK>
__device__ __forceinline__ void stage_pair(uint32_t coop, uint32_t* meta, uint32_t dst_a, uint32_t dst_b, uint32_t kS,
                                           const uint32_t* __restrict__ hi, const uint32_t* __restrict__ lo,
                                           const uint32_t* __restrict__ ot, uint32_t ea, uint32_t eb,
                                           uint32_t seg_w0, unsigned lane, uint32_t* ents) {
  ents[lane] = ea;
  ents[32 + lane] = eb;
  // Plane word of each window's first position (< 2^31 for genomes below 2^36 positions).
  const bool ha = ea != 0xFFFFFFFFu, hb = eb != 0xFFFFFFFFu;
  const uint32_t wa = seg_w0 + (ea >> 6), wb = seg_w0 + (eb >> 6);
  const uint32_t w0 = __reduce_min_sync(kFull, min(ha ? wa : 0xFFFFFFFFu, hb ? wb : 0xFFFFFFFFu));
  const uint32_t w1 = __reduce_max_sync(kFull, max(ha ? wa : 0u, hb ? wb : 0u)) + NK;  // last word read
  if (w0 != 0xFFFFFFFFu && w1 - w0 < (uint32_t)kWindowWords) {  // warp-uniform
    const uint32_t w = w0 + lane;
    const uint32_t bytes = w <= w1 ? 4u : 0u;
    const uint32_t ws = bytes ? w : w0;
    cp_async4(coop + (0 * kWindowWords + lane) * 4, hi + ws, bytes);
    cp_async4(coop + (1 * kWindowWords + lane) * 4, lo + ws, bytes);
    cp_async4(coop + (2 * kWindowWords + lane) * 4, ot + ws, bytes);
    if (lane == 0) *meta = w0;
  } else {
    stage_planes<NK>(dst_a, kS, hi, lo, ot, ea, seg_w0);
    stage_planes<NK>(dst_b, kS, hi, lo, ot, eb, seg_w0);
    if (lane == 0) *meta = kNoWindow;
  }
}

// Reads back the pair staged by stage_pair (call after cp_async_wait_all):
// each lane waited for its own copies; the warp barrier makes the other
// lanes' copies and `meta` visible.  Entries past the end of the queue read
// word w0 (their windows are never reported).
template <int NK>
__device__ __forceinline__ void unstage_pair(RawWindow<NK>& ra, RawWindow<NK>& rb, const uint32_t* coop_w,
                                             const uint32_t* meta, const uint32_t* st, uint32_t kS,
                                             const uint32_t* ents, unsigned lane, uint32_t seg_w0) {
  __syncwarp();
  const uint32_t w0 = *meta;
  const uint32_t ea = ents[lane], eb = ents[32 + lane];
  if (w0 != kNoWindow) {
    const uint32_t ia = ea != 0xFFFFFFFFu ? seg_w0 + (ea >> 6) - w0 : 0u;
    const uint32_t ib = eb != 0xFFFFFFFFu ? seg_w0 + (eb >> 6) - w0 : 0u;
    ra.e = ea;
    rb.e = eb;
#pragma unroll
    for (int i = 0; i <= NK; ++i) {
      ra.h[i] = coop_w[0 * kWindowWords + ia + i];
      ra.l[i] = coop_w[1 * kWindowWords + ia + i];
      ra.o[i] = coop_w[2 * kWindowWords + ia + i];
      rb.h[i] = coop_w[0 * kWindowWords + ib + i];
      rb.l[i] = coop_w[1 * kWindowWords + ib + i];
      rb.o[i] = coop_w[2 * kWindowWords + ib + i];
    }
  } else {
    unstage<NK>(ra, st, kS, ea);
    unstage<NK>(rb, st + Stage<NK>::kSlots * kS, kS, eb);
  }
}

// The window of one candidate: positions 0..L-1 in bits 0..L-1 of (h, l, o)
// words (a segment starts on a plane word, so the window's first position is
// bit (e >> 1) & 31 of its first word).  NK > 1: a '-' strand window is turned
// into its reverse complement here; NK == 1 windows are turned after the
// transpose (build_pair), for the whole group at once.
template <int NK>
__device__ __forceinline__ void orient(const RawWindow<NK>& raw, uint32_t L, uint32_t (&hw)[NK], uint32_t (&lw)[NK],
                                       uint32_t (&ow)[NK]) {
  const bool have = raw.e != 0xFFFFFFFFu;
  const unsigned r = (raw.e >> 1) & 31;
#pragma unroll
  for (int i = 0; i < NK; ++i) {
    hw[i] = __funnelshift_r(raw.h[i], raw.h[i + 1], r);
    lw[i] = __funnelshift_r(raw.l[i], raw.l[i + 1], r);
    ow[i] = __funnelshift_r(raw.o[i], raw.o[i + 1], r);
  }
  if (NK > 1 && have && (raw.e & 1)) {
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
}

// Class rows of the shared table: 0 never mismatches (padding slots), 1-4 the
// concrete bases, 5-14 the degenerate codes.
template <bool CONC>
struct TableRows {
  static constexpr int kRows = CONC ? 5 : 15;
};

// Builds pair p of a tile from two groups of candidates (`ra` -> .x, `rb` ->
// .y): oriented windows, transposed, expanded to class words in `pt` (the
// pair's table, [row][ROW] uint2).  The pair's entries are already in its
// entry slots (stage_pair).
template <int NK, int ROW, bool CONC>
__device__ __forceinline__ void build_pair(const RawWindow<NK>& ra, const RawWindow<NK>& rb, uint32_t L,
                                           unsigned lane, uint2* pt) {
  uint32_t ha[NK], la[NK], oa[NK], hb[NK], lb[NK], ob[NK];
  orient<NK>(ra, L, ha, la, oa);
  orient<NK>(rb, L, hb, lb, ob);
  // NK == 1: after the transpose lane k holds position k of every window of
  // the group; a '-' window (bit c of the strand ballot) takes position
  // L - 1 - k instead, complemented in the hi plane, from lane L - 1 - k.
  // Lanes k >= L hold positions no compare variant reads.
  const uint32_t ma = NK == 1 ? __ballot_sync(kFull, ra.e & 1) : 0u;
  const uint32_t mb = NK == 1 ? __ballot_sync(kFull, rb.e & 1) : 0u;
  const int src = (int)((L - 1 - lane) & 31);
#pragma unroll
  for (int i = 0; i < NK; ++i) {
    uint32_t h0 = warp_transpose(ha[i], lane), h1 = warp_transpose(hb[i], lane);
    uint32_t l0 = warp_transpose(la[i], lane), l1 = warp_transpose(lb[i], lane);
    // Windows holding a non-base byte (N, a separator, another byte) are rare:
    // most pairs skip the third plane's transposes.
    uint32_t o0 = 0, o1 = 0;
    const bool any_o = __any_sync(kFull, oa[i] | ob[i]);
    if (any_o) {
      o0 = warp_transpose(oa[i], lane);
      o1 = warp_transpose(ob[i], lane);
    }
    if (NK == 1 && (ma | mb)) {  // warp-uniform
      // (x & ~m) | (~y & m) and (x & ~m) | (y & m) over (x, y, m) = (0xF0, 0xCC, 0xAA).
      h0 = lop3<0x72>(h0, __shfl_sync(kFull, h0, src), ma);
      h1 = lop3<0x72>(h1, __shfl_sync(kFull, h1, src), mb);
      l0 = lop3<0xD8>(l0, __shfl_sync(kFull, l0, src), ma);
      l1 = lop3<0xD8>(l1, __shfl_sync(kFull, l1, src), mb);
      if (any_o) {
        o0 = lop3<0xD8>(o0, __shfl_sync(kFull, o0, src), ma);
        o1 = lop3<0xD8>(o1, __shfl_sync(kFull, o1, src), mb);
      }
    }
    const unsigned k = i * 32 + lane;
    if (k < (unsigned)ROW) {
      // One LOP3 of (h, l, o) each; truth tables over (0xF0, 0xCC, 0xAA).
      // Row r holds position k at column (k + r) mod ROW: classes rotate across
      // the banks, so lanes reading different classes at nearby positions
      // conflict less.
#define COF_ROW(r, LUT)                                                           \
  pt[(r) * ROW + (k + (r) < (unsigned)ROW ? k + (r) : k + (r) - ROW)] =           \
      make_uint2(lop3<LUT>(h0, l0, o0), lop3<LUT>(h1, l1, o1))
      COF_ROW(1, 0xFE);  // T: h | l | o (mismatch unless T)
      COF_ROW(2, 0xFB);  // C: h | ~l | o
      COF_ROW(3, 0xEF);  // A: ~h | l | o
      COF_ROW(4, 0xBF);  // G: ~h | ~l | o
      if (!CONC) {
        COF_ROW(5, 0x01);   // V: ~h & ~l & ~o (mismatch only T)
        COF_ROW(6, 0x04);   // D: ~h & l & ~o (only C)
        COF_ROW(7, 0x10);   // B: h & ~l & ~o (only A)
        COF_ROW(8, 0x40);   // H: h & l & ~o (only G)
        COF_ROW(9, 0x05);   // R: ~h & ~o (C or T)
        COF_ROW(10, 0x50);  // Y: h & ~o (A or G)
        COF_ROW(11, 0x14);  // K: (h ^ l) & ~o (A or C)
        COF_ROW(12, 0x41);  // M: ~(h ^ l) & ~o (G or T)
        COF_ROW(13, 0x44);  // W: l & ~o (C or G)
        COF_ROW(14, 0x11);  // S: ~l & ~o (A or T)
      }
#undef COF_ROW
    }
  }
}

// 64-bit shared-memory load at a shared-window byte address plus a constant.
template <uint32_t IMM>
__device__ __forceinline__ void lds64(uint32_t addr, uint32_t& x, uint32_t& y) {
  asm volatile("ld.shared.v2.u32 {%0, %1}, [%2+%3];" : "=r"(x), "=r"(y) : "r"(addr), "n"(IMM));
}

// A lane program's first variant (program layout in kernels.cuh): the shared
// addresses of its slots' class words (pair 0 of the buffer at `tbase`), the
// carry masks of its threshold bias and whether it is a real variant.
// NARROW: the bias is lowered by 2^(NB-1) so that NB count planes suffice
// (the top plane, 2^(NB-1), is then set exactly where count > threshold).
template <int S, bool NARROW>
__device__ __forceinline__ void load_program(const uint32_t* __restrict__ pr, uint32_t tbase, uint32_t (&addr)[S],
                                             uint32_t (&kmask)[bit_width(S)], uint32_t& kadd, uint32_t& first_on) {
  constexpr int NB = bit_width(S);
  const uint32_t h = __ldg(pr);
#pragma unroll
  for (int s = 0; s < S; s += 2) {
    const uint32_t pk = __ldg(pr + (1 + s / 2) * 32);
    addr[s] = tbase + (pk & 0xFFFFu);
    addr[s + 1] = tbase + (pk >> 16);
  }
  kadd = h & 0xFFu;
  if (NARROW) kadd -= 1u << (NB - 1);  // the bias for NB planes (the host checked kadd >= 2^(NB-1))
#pragma unroll
  for (int i = 0; i < NB; ++i) kmask[i] = 0u - ((kadd >> i) & 1u);
  first_on = (h & 0x100u) ? kFull : 0u;
}

// Appends the hits of one group: mask `hm`, count planes `bits` holding
// count + `bias`.  Entries past the end of the queue (0xFFFFFFFF) are not
// candidates.
template <int NP>
__device__ __forceinline__ void emit_hits(uint32_t hm, const uint32_t (&bits)[NP], uint32_t bias,
                                          const uint32_t* ents, uint32_t gid, uint64_t seg_pos0,
                                          uint64_t* __restrict__ hits, unsigned long long* __restrict__ hit_count,
                                          uint64_t hit_cap) {
  while (hm) {
    const unsigned c = __ffs(hm) - 1;
    hm &= hm - 1;
    const uint32_t e = ents[c];
    if (e == 0xFFFFFFFFu) continue;
    uint32_t v = 0;
#pragma unroll
    for (int i = 0; i < NP; ++i) v |= ((bits[i] >> c) & 1u) << i;
    const unsigned long long at = atomicAdd(hit_count, 1ull);
    if (at < hit_cap) hits[at] = make_hit(gid, seg_pos0 + (e >> 1), e & 1, v - bias);
  }
}

// Count planes + a per-lane constant (bit i of it as the all-ones / all-zeros
// word kmask[i]): NP planes out, NB + 1 (the carry out of the top count plane
// kept) or NB (the sum taken modulo 2^NB, exact when it stays below 2^NB).
template <int NB, int NP>
__device__ __forceinline__ void add_bias(const uint32_t (&b)[NB], const uint32_t (&kmask)[NB], uint32_t (&p)[NP]) {
  static_assert(NP == NB || NP == NB + 1, "NB or NB + 1 planes");
  uint32_t c = 0;
#pragma unroll
  for (int i = 0; i < NB; ++i) {
    p[i] = xor3(b[i], kmask[i], c);
    if (i + 1 < NP) c = maj3(b[i], kmask[i], c);
  }
  if constexpr (NP > NB) p[NP - 1] = c;
}

// One update step of bit-sliced counters: + a - b (one bit each per
// candidate).  Where exactly one of a, b is set the counter moves by one:
// up (carry = p & t) when a is set, down (borrow = ~p & t) otherwise.
template <int NP>
__device__ __forceinline__ void step_update(uint32_t (&p)[NP], uint32_t a, uint32_t b) {
  uint32_t t = a ^ b;
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    // The next carry first, so the plane's new value can take its register.
    const uint32_t tn = i + 1 < NP ? lop3<0x90>(t, p[i], a) : 0u;  // t & ~(p ^ a)
    p[i] ^= t;
    t = tn;
  }
}

// Registers per thread: 80 lets 25 one-warp CTAs (or three 256-thread CTAs)
// share an SM; wider slot lists get more.  (A 72-register budget, 28 one-warp
// CTAs, spilled once both steps of a pair were loaded ahead and measured
// slower.)
template <int S, int NK>
struct MaxRegs {
  static constexpr int value = S <= 20 ? 80 : S <= 28 ? 96 : 104;
};

// The full count of a lane program's first variant on pair P: its S class
// words summed into NB bit planes.  P is a compile-time constant so that every
// load is [register + immediate] (`addr` points at pair 0 of the buffer).
template <int P, int S, int ROW, bool CONC>
__device__ __forceinline__ void full_count(const uint32_t (&addr)[S], uint32_t (&ba)[bit_width(S)],
                                           uint32_t (&bb)[bit_width(S)]) {
  constexpr int NB = bit_width(S);
  constexpr uint32_t kImm = P * TableRows<CONC>::kRows * ROW * 8;
  uint32_t xa[S], xb[S];
#pragma unroll
  for (int s = 0; s < S; ++s) lds64<kImm>(addr[s], xa[s], xb[s]);
  CountTree<S, 0, NB>::run(xa, ba);
  CountTree<S, 0, NB>::run(xb, bb);
}

// Runs one lane program on pair P of the current tile (`addr` points at pair
// 0 of the current buffer, `tbase` is that buffer's base).  Only the full
// count is compiled once per pair index; the steps, which address their words
// from the pair's base, run from one copy of the code for every pair (one
// copy per pair made the loop of an eight-warp CTA larger than the
// instruction cache).
template <int S, int ROW, int NK, bool CONC, bool NARROW>
__device__ __forceinline__ void run_pair(unsigned P, const uint32_t (&addr)[S], const uint32_t (&kmask)[bit_width(S)],
                                         uint32_t kadd, uint32_t first_on, const uint2* __restrict__ steps,
                                         const uint32_t* __restrict__ gids, uint32_t m, uint32_t tbase,
                                         const uint32_t* ents, uint64_t seg_pos0, uint64_t* __restrict__ hits,
                                         unsigned long long* __restrict__ hit_count, uint64_t hit_cap) {
  constexpr int NB = bit_width(S);
  constexpr int NP = NARROW ? NB : NB + 1;  // count planes
  constexpr uint32_t kPairBytes = TableRows<CONC>::kRows * ROW * 8;
  static_assert(kMaxWarps == 8, "one full_count case per pair index");
  {
    uint32_t ba[NB], bb[NB];
    switch (P) {
      case 0: full_count<0, S, ROW, CONC>(addr, ba, bb); break;
      case 1: full_count<1, S, ROW, CONC>(addr, ba, bb); break;
      case 2: full_count<2, S, ROW, CONC>(addr, ba, bb); break;
      case 3: full_count<3, S, ROW, CONC>(addr, ba, bb); break;
      case 4: full_count<4, S, ROW, CONC>(addr, ba, bb); break;
      case 5: full_count<5, S, ROW, CONC>(addr, ba, bb); break;
      case 6: full_count<6, S, ROW, CONC>(addr, ba, bb); break;
      default: full_count<7, S, ROW, CONC>(addr, ba, bb); break;
    }
    const uint32_t* pe = ents + P * 64;
    const uint32_t pbase = tbase + P * kPairBytes;  // this pair's class words
    if (m == 1) {
      // One variant per lane: only the carry out of count + bias matters.
      uint32_t ca = 0, cb = 0;
#pragma unroll
      for (int i = 0; i < NB; ++i) {
        ca = maj3(ba[i], kmask[i], ca);
        cb = maj3(bb[i], kmask[i], cb);
      }
      const uint32_t hita = ~ca & first_on, hitb = ~cb & first_on;
      if (__any_sync(kFull, hita | hitb)) {
        const uint32_t gid = __ldg(gids);
        emit_hits<NB>(hita, ba, 0u, pe, gid, seg_pos0, hits, hit_count, hit_cap);
        emit_hits<NB>(hitb, bb, 0u, pe + 32, gid, seg_pos0, hits, hit_count, hit_cap);
      }
      return;
    }
    // Biased counters (count + bias in NP planes): a variant passes
    // while the top plane is clear.
    uint32_t pa[NP], pb[NP];
    add_bias<NB, NP>(ba, kmask, pa);
    add_bias<NB, NP>(bb, kmask, pb);
    const uint32_t hita = ~pa[NP - 1] & first_on, hitb = ~pb[NP - 1] & first_on;
    if (__any_sync(kFull, hita | hitb)) {
      const uint32_t gid = __ldg(gids);
      emit_hits<NP>(hita, pa, kadd, pe, gid, seg_pos0, hits, hit_count, hit_cap);
      emit_hits<NP>(hitb, pb, kadd, pe + 32, gid, seg_pos0, hits, hit_count, hit_cap);
    }
    // Step st tests its variant when it emits (bit 15); the variant's id is
    // entry st + 1 of the lane's id list.  A candidate passes while the top
    // plane is clear, so a step has hits when the flag is set and some
    // candidate of the pair has that plane clear.
    auto emit_step = [&](bool any, uint32_t st) {
      const uint32_t on = any ? kFull : 0u;
      const uint32_t ha = ~pa[NP - 1] & on, hb = ~pb[NP - 1] & on;
      const uint32_t gid = any ? __ldg(gids + (st + 1) * 32) : 0u;
      emit_hits<NP>(ha, pa, kadd, pe, gid, seg_pos0, hits, hit_count, hit_cap);
      emit_hits<NP>(hb, pb, kadd, pe + 32, gid, seg_pos0, hits, hit_count, hit_cap);
    };
    auto step = [&](uint32_t w, uint32_t st, uint32_t a0, uint32_t a1, uint32_t b0, uint32_t b1) {
      step_update<NP>(pa, a0, b0);
      step_update<NP>(pb, a1, b1);
      const bool any = (w & 0x8000u) && (pa[NP - 1] & pb[NP - 1]) != kFull;
      if (__any_sync(kFull, any)) emit_step(any, st);
    };
    // Steps come in pairs (one 64-bit load), the next pair loaded ahead.
    // Both steps' class words are loaded before the first is applied (four
    // shared loads in flight instead of two), and the pair's two steps share
    // one vote: t0 & t1 (the top planes after each step) has a clear bit
    // exactly when some candidate passed either step.  In that rare case the
    // second step is undone (+b - a is the exact inverse of +a - b) to report
    // the first step's hits, then redone.
    // A program of up to m variants has at most m - 1 steps: (m - 1) / 2
    // pairs, then one step alone when m - 1 is odd (the pair layout's last
    // slot is padding then).
    const uint32_t ns = m - 1, sp = ns / 2;
    uint2 wn = make_uint2(0u, 0u);
    if (ns) wn = __ldg(steps);
    for (uint32_t j = 0; j < sp; ++j) {
      const uint2 w2 = wn;
      if (2 * (j + 1) < ns) wn = __ldg(steps + (j + 1) * 32);
      uint32_t a0, a1, b0, b1, c0, c1, d0, d1;
      lds64<0>(pbase + (w2.x & 0x7FFFu), a0, a1);
      lds64<0>(pbase + (w2.x >> 16), b0, b1);
      lds64<0>(pbase + (w2.y & 0x7FFFu), c0, c1);
      lds64<0>(pbase + (w2.y >> 16), d0, d1);
      step_update<NP>(pa, a0, b0);
      step_update<NP>(pb, a1, b1);
      const uint32_t t0 = pa[NP - 1] & pb[NP - 1];
      step_update<NP>(pa, c0, d0);
      step_update<NP>(pb, c1, d1);
      const uint32_t t1 = pa[NP - 1] & pb[NP - 1];
      if (__any_sync(kFull, (t0 & t1) != kFull)) {
        const bool e0 = (w2.x & 0x8000u) && t0 != kFull;
        const bool e1 = (w2.y & 0x8000u) && t1 != kFull;
        if (__any_sync(kFull, e0)) {
          step_update<NP>(pa, d0, c0);
          step_update<NP>(pb, d1, c1);
          emit_step(e0, 2 * j);
          step_update<NP>(pa, c0, d0);
          step_update<NP>(pb, c1, d1);
        }
        if (__any_sync(kFull, e1)) emit_step(e1, 2 * j + 1);
      }
    }
    if (ns & 1) {
      uint32_t a0, a1, b0, b1;
      lds64<0>(pbase + (wn.x & 0x7FFFu), a0, a1);
      lds64<0>(pbase + (wn.x >> 16), b0, b1);
      step(wn.x, ns - 1, a0, a1, b0, b1);
    }
  }
}

// 128-bit shared-memory load (four step addresses).
__device__ __forceinline__ uint4 lds128(uint32_t addr) {
  uint4 r;
  asm volatile("ld.shared.v4.u32 {%0, %1, %2, %3}, [%4];" : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w) : "r"(addr));
  return r;
}

// One-warp CTAs: the lane's program on the tile's only pair, read from table
// buffer CUR (a compile-time constant; a buffer is one pair).  Every class
// word address is a register holding the word's shared address in buffer 0
// -- the full count's `addr`, the steps' four addresses per pair of steps in
// `steps` (uint4 per lane, lane stride 32) -- plus the buffer's offset as the
// load's immediate, so no address arithmetic runs per tile.  `emask` (the
// lane's word in shared memory) has bit s set when step s ends a variant; it
// is read only when some candidate passed.
template <int CUR, int S, int ROW, int NK, bool CONC, bool NARROW>
__device__ __forceinline__ void run_one(const uint32_t (&addr)[S], const uint32_t (&kmask)[bit_width(S)],
                                        uint32_t kadd, uint32_t first_on, uint32_t steps, const uint32_t* emask,
                                        const uint32_t* __restrict__ gids, uint32_t m, const uint32_t* pe,
                                        uint64_t seg_pos0, uint64_t* __restrict__ hits,
                                        unsigned long long* __restrict__ hit_count, uint64_t hit_cap) {
  constexpr int NB = bit_width(S);
  constexpr int NP = NARROW ? NB : NB + 1;  // count planes
  constexpr uint32_t kBuf = CUR * TableRows<CONC>::kRows * ROW * 8;
  uint32_t ba[NB], bb[NB];
  full_count<CUR, S, ROW, CONC>(addr, ba, bb);  // pair CUR of buffer 0 = buffer CUR's pair
  if (m == 1) {
    uint32_t ca = 0, cb = 0;
#pragma unroll
    for (int i = 0; i < NB; ++i) {
      ca = maj3(ba[i], kmask[i], ca);
      cb = maj3(bb[i], kmask[i], cb);
    }
    const uint32_t hita = ~ca & first_on, hitb = ~cb & first_on;
    if (__any_sync(kFull, hita | hitb)) {
      const uint32_t gid = __ldg(gids);
      emit_hits<NB>(hita, ba, 0u, pe, gid, seg_pos0, hits, hit_count, hit_cap);
      emit_hits<NB>(hitb, bb, 0u, pe + 32, gid, seg_pos0, hits, hit_count, hit_cap);
    }
    return;
  }
  uint32_t pa[NP], pb[NP];
  add_bias<NB, NP>(ba, kmask, pa);
  add_bias<NB, NP>(bb, kmask, pb);
  const uint32_t hita = ~pa[NP - 1] & first_on, hitb = ~pb[NP - 1] & first_on;
  if (__any_sync(kFull, hita | hitb)) {
    const uint32_t gid = __ldg(gids);
    emit_hits<NP>(hita, pa, kadd, pe, gid, seg_pos0, hits, hit_count, hit_cap);
    emit_hits<NP>(hitb, pb, kadd, pe + 32, gid, seg_pos0, hits, hit_count, hit_cap);
  }
  auto emit_step = [&](bool any, uint32_t st) {
    const uint32_t on = any ? kFull : 0u;
    const uint32_t ha = ~pa[NP - 1] & on, hb = ~pb[NP - 1] & on;
    const uint32_t gid = any ? __ldg(gids + (st + 1) * 32) : 0u;
    emit_hits<NP>(ha, pa, kadd, pe, gid, seg_pos0, hits, hit_count, hit_cap);
    emit_hits<NP>(hb, pb, kadd, pe + 32, gid, seg_pos0, hits, hit_count, hit_cap);
  };
  // The same schedule as run_pair: pairs of steps, the next pair's addresses
  // loaded ahead, one vote per pair, the second step undone to report the
  // first step's hits.
  const uint32_t ns = m - 1, sp = ns / 2;
  uint4 wn = make_uint4(0u, 0u, 0u, 0u);
  if (ns) wn = lds128(steps);
  for (uint32_t j = 0; j < sp; ++j) {
    const uint4 w = wn;
    if (2 * (j + 1) < ns) wn = lds128(steps + (j + 1) * 32 * 16);
    uint32_t a0, a1, b0, b1, c0, c1, d0, d1;
    lds64<kBuf>(w.x, a0, a1);
    lds64<kBuf>(w.y, b0, b1);
    lds64<kBuf>(w.z, c0, c1);
    lds64<kBuf>(w.w, d0, d1);
    step_update<NP>(pa, a0, b0);
    step_update<NP>(pb, a1, b1);
    const uint32_t t0 = pa[NP - 1] & pb[NP - 1];
    step_update<NP>(pa, c0, d0);
    step_update<NP>(pb, c1, d1);
    const uint32_t t1 = pa[NP - 1] & pb[NP - 1];
    if (__any_sync(kFull, (t0 & t1) != kFull)) {
      const uint32_t em = *emask >> (2 * j);
      const bool e0 = (em & 1u) && t0 != kFull;
      const bool e1 = (em & 2u) && t1 != kFull;
      if (__any_sync(kFull, e0)) {
        step_update<NP>(pa, d0, c0);
        step_update<NP>(pb, d1, c1);
        emit_step(e0, 2 * j);
        step_update<NP>(pa, c0, d0);
        step_update<NP>(pb, c1, d1);
      }
      if (__any_sync(kFull, e1)) emit_step(e1, 2 * j + 1);
    }
  }
  if (ns & 1) {
    uint32_t a0, a1, b0, b1;
    lds64<kBuf>(wn.x, a0, a1);
    lds64<kBuf>(wn.y, b0, b1);
    step_update<NP>(pa, a0, b0);
    step_update<NP>(pb, a1, b1);
    const bool any = ((*emask >> (ns - 1)) & 1u) && (pa[NP - 1] & pb[NP - 1]) != kFull;
    if (__any_sync(kFull, any)) emit_step(any, ns - 1);
  }
}

// Runs one lane program on pairs 0 .. W-1 of the current tile (CTAs of
// several warps; one-warp CTAs use run_one).
template <int S, int ROW, int NK, bool CONC, bool NARROW>
__device__ __forceinline__ void run_program(const uint32_t (&addr)[S], const uint32_t (&kmask)[bit_width(S)],
                                            uint32_t kadd, uint32_t first_on, const uint2* __restrict__ steps,
                                            const uint32_t* __restrict__ gids, uint32_t m, uint32_t tbase, unsigned W,
                                            const uint32_t* ents, uint64_t seg_pos0, uint64_t* __restrict__ hits,
                                            unsigned long long* __restrict__ hit_count, uint64_t hit_cap) {
#pragma unroll 1
  for (unsigned P = 0; P < W; ++P)
    run_pair<S, ROW, NK, CONC, NARROW>(P, addr, kmask, kadd, first_on, steps, gids, m, tbase, ents, seg_pos0, hits, hit_count,
                               hit_cap);
}

// Shared memory of a CTA of W warps: two table buffers of W pairs, their
// candidate entries, the per-thread staging slots and the per-warp window
// copies (with their meta word); one-warp CTAs add their program's step
// addresses (m / 2 pairs of steps per lane, four addresses each) and each
// lane's mask of testing steps.
constexpr uint32_t kMaxM = 24;  // longest lane program (the host's cost model and autotuner stay within it)
template <int ROW, int NK, bool CONC>
__host__ __device__ constexpr size_t bs_smem_bytes(unsigned W, uint32_t m) {
  return 2 * ((size_t)W * TableRows<CONC>::kRows * ROW * sizeof(uint2) + W * 64 * 4) +
         2 * Stage<NK>::kSlots * (32 * W) * 4 + (size_t)W * kCoopWords * 4 +
         (W == 1 ? (size_t)(m / 2) * 32 * sizeof(uint4) + 32 * 4 : 0);
}

template <int S, int ROW, int NK, bool CONC, bool ONE, bool NARROW>
__global__ void __launch_bounds__(32 * kMaxWarps) __maxnreg__((MaxRegs<S, NK>::value)) comparer_bs_kernel(
    const uint32_t* __restrict__ hi, const uint32_t* __restrict__ lo, const uint32_t* __restrict__ ot,
    const uint32_t* __restrict__ queue, const uint32_t* __restrict__ qcount, uint64_t seg_pos0,
    const uint32_t* __restrict__ prog, const uint32_t* __restrict__ pgid, uint32_t chunks, uint32_t m, uint32_t L,
    uint32_t* __restrict__ tile_ctr, uint64_t* __restrict__ hits, unsigned long long* __restrict__ hit_count,
    uint64_t hit_cap) {
  constexpr int NB = bit_width(S);
  constexpr int kPairWords = TableRows<CONC>::kRows * ROW;  // uint2 per pair
  const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned W = blockDim.x >> 5;  // pairs per tile = warps
  const uint32_t seg_w0 = (uint32_t)(seg_pos0 >> 5);  // the segment starts on a plane word
  const unsigned tile_n = W * 64;
  const uint32_t kBufWords = W * kPairWords;
  const uint32_t kBufBytes = kBufWords * (uint32_t)sizeof(uint2);
  extern __shared__ __align__(16) uint2 smem2[];
  uint2* tables = smem2;                                    // [2 buffers][W pairs][rows][ROW]
  uint32_t* ents_all = (uint32_t*)(smem2 + 2 * kBufWords);  // [2 buffers][W pairs][64]
  const uint32_t table_base = (uint32_t)__cvta_generic_to_shared(tables);
  // Window words of the next tile are staged here by cp.async while the
  // current tile is counted (per thread: candidate a's slots, then b's).
  const uint32_t kS = blockDim.x;  // staging slot stride, words
  const uint32_t* stage = ents_all + 2 * W * 64 + threadIdx.x;
  const uint32_t stage_a = (uint32_t)__cvta_generic_to_shared(stage);
  const uint32_t stage_b = stage_a + Stage<NK>::kSlots * kS * 4;
  // This warp's window copies: the three planes, then the meta word.
  auto coop_words = [&]() { return ents_all + 2 * W * 64 + 2 * Stage<NK>::kSlots * kS + warp * kCoopWords; };
  const uint32_t words = 1 + S / 2 + 2 * (m / 2);  // per lane program

  // Row 0 (pattern bytes that never mismatch: padding slots) stays zero.
  for (unsigned i = threadIdx.x; i < 2 * W * ROW; i += blockDim.x)
    tables[(i / ROW) * kPairWords + i % ROW] = make_uint2(0, 0);

  const uint32_t n = *qcount;
  const uint32_t ntiles = (n + tile_n - 1) / tile_n;
  // Tiles: blockIdx.x and blockIdx.x + gridDim.x first, then tiles claimed
  // from *tile_ctr (zeroed by the caller), so CTAs whose warps are issued
  // less often take fewer tiles instead of finishing last.  A claim is made
  // two tiles ahead and published to the CTA through claimed[] (one slot
  // per parity of the step, written before the step's barrier, read after
  // it); a CTA's tiles increase, so it stops at the first one past the end.
  __shared__ uint32_t claimed[2];
  uint32_t t = blockIdx.x, tn = blockIdx.x + gridDim.x;
  uint32_t claim = 0;
  if (threadIdx.x == 0) claim = 2 * gridDim.x + atomicAdd(tile_ctr, 1u);
  const uint32_t ca = warp * 64 + lane, cb = ca + 32;  // this lane's candidates within a tile
  // With one chunk per warp the lane's program stays in registers for the
  // whole kernel; its addresses follow the current buffer.
  const bool resident = chunks <= W;
  uint32_t addr[S], kmask[NB], kadd = 0, first_on = 0;
  if (resident && warp < chunks)
    load_program<S, NARROW>(prog + (size_t)warp * words * 32 + lane, table_base, addr, kmask, kadd, first_on);
  // One-warp CTAs: the program's steps as shared addresses in table buffer 0
  // (added word, removed word, for both steps of a pair), lane-minor, then
  // each lane's mask of the steps that end a variant.  Each lane reads back
  // only its own words.
  uint4* steps_sh = (uint4*)(ents_all + 2 * W * 64 + 2 * Stage<NK>::kSlots * kS + W * kCoopWords);
  uint32_t* emask_sh = (uint32_t*)(steps_sh + (m / 2) * 32);
  if (ONE && chunks == 1) {
    const uint2* src = (const uint2*)(prog + (1 + S / 2) * 32) + lane;
    uint32_t em = 0;
    for (uint32_t j = 0; j < m / 2; ++j) {
      const uint2 w = __ldg(src + j * 32);
      steps_sh[j * 32 + lane] = make_uint4(table_base + (w.x & 0x7FFFu), table_base + (w.x >> 16),
                                           table_base + (w.y & 0x7FFFu), table_base + (w.y >> 16));
      em |= ((w.x >> 15) & 1u) << (2 * j) | ((w.y >> 15) & 1u) << (2 * j + 1);
    }
    emask_sh[lane] = em;
  }
  const uint32_t steps_addr = (uint32_t)__cvta_generic_to_shared(steps_sh + lane);
  // Entries: e* of the tile being staged, n* of the tile after it.
  {
    uint32_t* cw = coop_words();
    stage_pair<NK>((uint32_t)__cvta_generic_to_shared(cw), cw + 3 * kWindowWords, stage_a, stage_b, kS * 4, hi, lo,
                   ot, load_entry(queue, t * tile_n + ca, n), load_entry(queue, t * tile_n + cb, n), seg_w0, lane,
                   ents_all + warp * 64);
  }
  uint32_t na = load_entry(queue, tn * tile_n + ca, n);
  uint32_t nb = load_entry(queue, tn * tile_n + cb, n);
  cp_async_wait_all();
  if (t < ntiles) {
    RawWindow<NK> ra, rb;
    const uint32_t* cw = coop_words();
    unstage_pair<NK>(ra, rb, cw, cw + 3 * kWindowWords, stage, kS, ents_all + warp * 64, lane, seg_w0);
    build_pair<NK, ROW, CONC>(ra, rb, L, lane, tables + warp * kPairWords);
  }
  if (threadIdx.x == 0) claimed[0] = claim;
  __syncthreads();
  // One tile per step: count the tile in buffer `cur` while the next tile's
  // words are in flight, then build the next tile into buffer cur ^ 1.
  unsigned cur = 0, par = 0;
  while (t < ntiles) {
    const uint32_t tnn = claimed[par];  // the tile after tn
    if (threadIdx.x == 0) claim = 2 * gridDim.x + atomicAdd(tile_ctr, 1u);
    {
      uint32_t* cw = coop_words();
      stage_pair<NK>((uint32_t)__cvta_generic_to_shared(cw), cw + 3 * kWindowWords, stage_a, stage_b, kS * 4, hi,
                     lo, ot, na, nb, seg_w0, lane, ents_all + (cur ^ 1) * (W * 64) + warp * 64);
    }
    na = load_entry(queue, tnn * tile_n + ca, n);
    nb = load_entry(queue, tnn * tile_n + cb, n);
    const uint32_t* ents = ents_all + cur * (W * 64);
    const uint32_t tbase = table_base + cur * kBufBytes;
    if constexpr (ONE) {
      // chunks == 1 (launch_bs): the program is resident; the buffer picks
      // the instance.
      if (cur)
        run_one<1, S, ROW, NK, CONC, NARROW>(addr, kmask, kadd, first_on, steps_addr, emask_sh + lane, pgid + lane, m,
                                     ents, seg_pos0, hits, hit_count, hit_cap);
      else
        run_one<0, S, ROW, NK, CONC, NARROW>(addr, kmask, kadd, first_on, steps_addr, emask_sh + lane, pgid + lane, m,
                                     ents, seg_pos0, hits, hit_count, hit_cap);
    } else {
      for (uint32_t c = warp; c < chunks; c += W) {
        const uint32_t* pr = prog + (size_t)c * words * 32 + lane;
        if (!resident) load_program<S, NARROW>(pr, tbase, addr, kmask, kadd, first_on);
        run_program<S, ROW, NK, CONC, NARROW>(addr, kmask, kadd, first_on, (const uint2*)(pr - lane + (1 + S / 2) * 32) + lane,
                                      pgid + (size_t)c * m * 32 + lane, m, tbase, W, ents, seg_pos0, hits, hit_count,
                                      hit_cap);
      }
    }
    cp_async_wait_all();
    if (tn < ntiles) {
      RawWindow<NK> ra, rb;
      const uint32_t* cw = coop_words();
      unstage_pair<NK>(ra, rb, cw, cw + 3 * kWindowWords, stage, kS, ents_all + (cur ^ 1) * (W * 64) + warp * 64,
                       lane, seg_w0);
      build_pair<NK, ROW, CONC>(ra, rb, L, lane, tables + (cur ^ 1) * kBufWords + warp * kPairWords);
    }
    if (threadIdx.x == 0) claimed[par ^ 1] = claim;
    __syncthreads();
    if (!ONE && resident) {  // one-warp CTAs address buffer 1 by immediates
      const uint32_t d = cur ? 0u - kBufBytes : kBufBytes;
#pragma unroll
      for (int s = 0; s < S; ++s) addr[s] += d;
    }
    cur ^= 1;
    par ^= 1;
    t = tn;
    tn = tnn;
  }
}

// Warps per CTA (= pairs of candidate groups per tile): one per chunk up to
// eight; above that the count in [4, 8] that splits the chunks most evenly.
inline unsigned bs_warps(uint32_t chunks) {
  if (chunks <= (uint32_t)kMaxWarps) return chunks ? chunks : 1;
  unsigned best = kMaxWarps, waste = ~0u;
  for (unsigned w = kMaxWarps; w >= 4; --w) {
    const unsigned x = (unsigned)(((chunks + w - 1) / w) * w - chunks);
    if (x < waste) {
      waste = x;
      best = w;
    }
  }
  return best;
}

template <int S, int ROW, int NK, bool CONC>
bool launch_bs(const GenomeView& g, const uint32_t* queue, const uint32_t* qcount, uint64_t seg_pos0,
               const uint32_t* prog, const uint32_t* pgid, uint32_t chunks, uint32_t m, bool narrow, uint32_t L,
               uint32_t* tile_ctr, uint64_t* hits, unsigned long long* hit_count, uint64_t hit_cap, int sm_count,
               cudaStream_t stream) {
  if (m > kMaxM) return false;  // the shared step words are sized for kMaxM
  const unsigned warps = bs_warps(chunks);
  // A one-warp CTA keeps one program's step words in shared memory: it must
  // have exactly one chunk (bs_warps gives one warp for one chunk only).
  if (warps == 1 && chunks != 1) return false;
  const int threads = 32 * (int)warps;
  const size_t smem = bs_smem_bytes<ROW, NK, CONC>(warps, m);
  // One-warp CTAs (one chunk) get the instance with the pair index constant;
  // programs of one variant (m = 1) test the carry of NB planes and never
  // take the narrow counters.
  const bool nar = narrow && m > 1;
  auto kernel = warps == 1 ? (nar ? comparer_bs_kernel<S, ROW, NK, CONC, true, true>
                                  : comparer_bs_kernel<S, ROW, NK, CONC, true, false>)
                           : (nar ? comparer_bs_kernel<S, ROW, NK, CONC, false, true>
                                  : comparer_bs_kernel<S, ROW, NK, CONC, false, false>);
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)std::max(bs_smem_bytes<ROW, NK, CONC>(kMaxWarps, 0), bs_smem_bytes<ROW, NK, CONC>(1, kMaxM)));
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  kernel<<<sm_count * per_sm, threads, smem, stream>>>(g.hi, g.lo, g.ot, queue, qcount, seg_pos0, prog, pgid, chunks,
                                                        m, L, tile_ctr, hits, hit_count, hit_cap);
  return true;
}

}  // namespace

template <int ROW, int NK, bool CONC>
bool dispatch_s(int slots, const GenomeView& g, const uint32_t* queue, const uint32_t* qcount, uint64_t seg_pos0,
                const uint32_t* prog, const uint32_t* pgid, uint32_t chunks, uint32_t m, bool narrow, uint32_t L,
                uint32_t* tile_ctr, uint64_t* hits, unsigned long long* hit_count, uint64_t hit_cap, int sm_count,
                cudaStream_t stream) {
#define COF_BS_CASE(SV)                                                                                  \
  case SV:                                                                                               \
    return launch_bs<SV, ROW, NK, CONC>(g, queue, qcount, seg_pos0, prog, pgid, chunks, m, narrow, L, tile_ctr, hits, \
                                        hit_count, hit_cap, sm_count, stream);
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

}  // namespace bs
}  // namespace cof
