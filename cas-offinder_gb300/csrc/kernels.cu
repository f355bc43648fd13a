// GB300 kernels of the Cas-OFFinder search path.
//
//   finder_kernel      replaces finder/finder_cpu (cas-offinder.cl:6-72,
//                      :157-213): PAM scan of 32 start positions per thread,
//                      bit-parallel over the planes, warp-aggregated append of
//                      strand-oriented candidates.
//   comparer_kernel    replaces comparer/comparer_cpu (cas-offinder.cl:73-155,
//                      :214-286): a tile of oriented candidate windows in
//                      shared memory against all compare variants of the
//                      pattern at once (one variant per thread, held in
//                      registers), mismatches counted by popcount.
//   row_len_kernel /   replace compareAll's host-side row formatting
//   write_rows_kernel  (cas-offinder.cpp:394-455): rows are written on the GPU
//                      from per-(variant, bulge, strand) row shapes.
//
// Mismatch rule (cas-offinder.cl:30-43) in plane form: for window bits
// (h, l, o) and a pattern byte with class masks (T, C, A, G, O),
//   mismatch = o ? O : (h ? (l ? G : A) : (l ? C : T)),
// evaluated for 32 positions per 32-bit word.  A '-' strand candidate is the
// reverse complement of the window (bit-reverse, flip hi) tested against the
// forward compare string; the IUPAC rule is complement-symmetric, so this
// counts the same mismatches as the reference's test of the reverse-complement
// compare string against the forward genome.
#include "kernels.cuh"

#include <algorithm>

namespace cof {

namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;

__device__ __forceinline__ uint32_t mux(uint32_t s, uint32_t a, uint32_t b) { return (s & a) | (~s & b); }

__device__ __forceinline__ uint32_t mismatch_word(uint32_t h, uint32_t l, uint32_t o, uint32_t mt, uint32_t mc,
                                                  uint32_t ma, uint32_t mg, uint32_t mo) {
  return mux(o, mo, mux(h, mux(l, mg, ma), mux(l, mc, mt)));
}

// 32 consecutive bits starting at bit k (0 <= k < 64) of the 96-bit value w0|w1|w2.
__device__ __forceinline__ uint32_t bits_at(uint32_t w0, uint32_t w1, uint32_t w2, unsigned k) {
  const unsigned r = k & 31;
  return (k & 32) ? __funnelshift_r(w1, w2, r) : __funnelshift_r(w0, w1, r);
}

}  // namespace

// ---------------------------------------------------------------- finder
// One warp = 32 x kFinderWords consecutive plane words (32 start positions
// each); lane `l` takes words l, l + 32, ... so every load is coalesced, and
// all of a lane's words are loaded before any is tested, to keep many loads
// in flight.  A warp's candidates (up to kFinderStage) are staged in shared
// memory in scan order, then written to the queue with one atomic
// reservation and coalesced 16-byte stores (the staged entries start at the
// queue position's offset within a 16-byte line, so source and destination
// line up); a warp with more candidates (dense patterns) stores them
// directly.
constexpr int kFinderThreads = 128;
constexpr int kFinderWords = 4;     // plane words per lane per pass
constexpr int kFinderStage = 1024;  // staged entries per warp; denser warps store directly

// Device form of a FinderPattern: per pattern position that can mismatch its
// window offset and its class bits, which pick the LOP3 truth table of the
// mismatch rule (one instruction per position and word).
struct FinderMasks {
  uint32_t L, nf, nr;
  uint8_t fk[kMaxL], rk[kMaxL];
  uint8_t fc[kMaxL], rc[kMaxL];  // class bits of each position (class_bits_of)
};

// One LOP3 with truth table LUT over (a, b, c) = (0xF0, 0xCC, 0xAA).
template <uint32_t LUT>
__device__ __forceinline__ uint32_t lop3(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t d;
  asm("lop3.b32 %0, %1, %2, %3, %4;" : "=r"(d) : "r"(a), "r"(b), "r"(c), "n"(LUT));
  return d;
}

// The mismatch rule of one pattern byte as one LOP3 of (hi, lo, other) bits:
// class bits T, C, A, G, other (bits 0-4) select the truth-table entries of
// (h, l, o) = (0,0,0), (0,1,0), (1,0,0), (1,1,0) and every o = 1.
__host__ __device__ constexpr uint32_t class_lut(uint32_t v) {
  return ((v & 1) ? 0x01u : 0u) | ((v & 2) ? 0x04u : 0u) | ((v & 4) ? 0x10u : 0u) | ((v & 8) ? 0x40u : 0u) |
         ((v & 16) ? 0xAAu : 0u);
}

// bad[k] |= mismatches of pattern class `cls` at window offset q, for the K
// words of a lane.  The class is the same for every lane (one pattern), so
// the switch is warp-uniform.
template <int NK, int K>
__device__ __forceinline__ void accumulate_position(uint32_t cls, unsigned q, const uint32_t (&h)[K][NK + 1],
                                                    const uint32_t (&l)[K][NK + 1], const uint32_t (&o)[K][NK + 1],
                                                    uint32_t (&bad)[K]);

// 32 consecutive bits starting at bit k of the window words x0|x1|x2 (NK = 1:
// k < 32 and x2 unused).
template <int NK>
__device__ __forceinline__ uint32_t window_bits(uint32_t x0, uint32_t x1, uint32_t x2, unsigned k) {
  if (NK == 1) return __funnelshift_r(x0, x1, k);
  return bits_at(x0, x1, x2, k);
}

template <int NK, int K>
__device__ __forceinline__ void accumulate_position(uint32_t cls, unsigned q, const uint32_t (&h)[K][NK + 1],
                                                    const uint32_t (&l)[K][NK + 1], const uint32_t (&o)[K][NK + 1],
                                                    uint32_t (&bad)[K]) {
  switch (cls) {
#define COF_CLASS_CASE(V)                                                                    \
  case V:                                                                                    \
    _Pragma("unroll") for (int k = 0; k < K; ++k) bad[k] |= lop3<class_lut(V)>(             \
        window_bits<NK>(h[k][0], h[k][1], h[k][NK], q), window_bits<NK>(l[k][0], l[k][1], l[k][NK], q), \
        window_bits<NK>(o[k][0], o[k][1], o[k][NK], q));                                     \
    break;
    COF_CLASS_CASE(1) COF_CLASS_CASE(2) COF_CLASS_CASE(3) COF_CLASS_CASE(4) COF_CLASS_CASE(5) COF_CLASS_CASE(6)
    COF_CLASS_CASE(7) COF_CLASS_CASE(8) COF_CLASS_CASE(9) COF_CLASS_CASE(10) COF_CLASS_CASE(11) COF_CLASS_CASE(12)
    COF_CLASS_CASE(13) COF_CLASS_CASE(14) COF_CLASS_CASE(15) COF_CLASS_CASE(16) COF_CLASS_CASE(17)
    COF_CLASS_CASE(18) COF_CLASS_CASE(19) COF_CLASS_CASE(20) COF_CLASS_CASE(21) COF_CLASS_CASE(22)
    COF_CLASS_CASE(23) COF_CLASS_CASE(24) COF_CLASS_CASE(25) COF_CLASS_CASE(26) COF_CLASS_CASE(27)
    COF_CLASS_CASE(28) COF_CLASS_CASE(29) COF_CLASS_CASE(30) COF_CLASS_CASE(31)
#undef COF_CLASS_CASE
    default:
      break;
  }
}

template <int NK>
__global__ void __launch_bounds__(kFinderThreads) finder_kernel(
    const uint32_t* __restrict__ hi, const uint32_t* __restrict__ lo, const uint32_t* __restrict__ ot,
    uint64_t w_begin, uint64_t w_end, uint64_t pos_end, const __grid_constant__ FinderMasks pat,
    uint32_t* __restrict__ queue, uint32_t* __restrict__ qcount) {
  constexpr int K = kFinderWords;
  // Four words of room for the queue's phase; rows stay 16-byte aligned.
  __shared__ __align__(16) uint32_t stage[kFinderThreads / 32][kFinderStage + 4];
  const unsigned lane = threadIdx.x & 31;
  uint32_t* my = stage[threadIdx.x >> 5];
  const bool vec_queue = ((uintptr_t)queue & 15u) == 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x * K;
  for (uint64_t wb = w_begin + ((uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u)) * K; wb < w_end;
       wb += stride) {
    // A window of L <= 32 starting in word w ends in word w + 1 (L <= 64: w + 2).
    uint32_t h[K][NK + 1], l[K][NK + 1], o[K][NK + 1];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const uint64_t w = wb + 32 * k + lane;
      const bool in = w < w_end;
#pragma unroll
      for (int i = 0; i <= NK; ++i) {
        h[k][i] = in ? hi[w + i] : 0u;
        l[k][i] = in ? lo[w + i] : 0u;
        o[k][i] = in ? ot[w + i] : 0u;
      }
    }
    static_assert(K % 2 == 0, "counts are scanned two per word");
    // Pattern position outer, word inner: each position's offset and class
    // masks are read once per pass.
    uint32_t badf[K], badr[K];
#pragma unroll
    for (int k = 0; k < K; ++k) badf[k] = badr[k] = 0;
    for (uint32_t j = 0; j < pat.nf; ++j) accumulate_position<NK, K>(pat.fc[j], pat.fk[j], h, l, o, badf);
    for (uint32_t j = 0; j < pat.nr; ++j) accumulate_position<NK, K>(pat.rc[j], pat.rk[j], h, l, o, badr);
    uint32_t fwd[K], rev[K], cnt[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const uint32_t h0 = h[k][0], h1 = h[k][1], h2 = NK == 1 ? 0u : h[k][NK];
      const uint32_t l0 = l[k][0], l1 = l[k][1], l2 = NK == 1 ? 0u : l[k][NK];
      const uint32_t o0 = o[k][0], o1 = o[k][1], o2 = NK == 1 ? 0u : o[k][NK];
      uint32_t f = ~badf[k], r = ~badr[k];
      // Words past w_end (loaded as zeros) test nothing; and only windows
      // that end inside the genome count: start < n - L + 1, whatever the
      // plane bits past the end hold.
      if (wb + 32 * k + lane >= w_end) f = r = 0;
      const uint64_t p0 = (wb + 32 * k + lane) << 5;
      if (p0 + 32 > pos_end) {
        const uint32_t keep = p0 >= pos_end ? 0u : (0xFFFFFFFFu >> (32 - (unsigned)(pos_end - p0)));
        f &= keep;
        r &= keep;
      }
      if (f | r) {
        // Drop windows holding a record separator (cas-offinder.cl:64-67).
        const uint32_t s0 = o0 & l0 & ~h0, s1 = o1 & l1 & ~h1, s2 = o2 & l2 & ~h2;
        if (s0 | s1 | s2) {
          uint32_t near = 0;
          for (unsigned q = 0; q < pat.L; ++q) near |= window_bits<NK>(s0, s1, s2, q);
          f &= ~near;
          r &= ~near;
        }
      }
      fwd[k] = f;
      rev[k] = r;
      cnt[k] = __popc(f) + __popc(r);
    }
    // Queue order = word order (pass k's 32 words, then pass k + 1's): the
    // comparer gathers the windows of consecutive entries together, so
    // nearby entries should be nearby in the genome.  Per-pass offsets come
    // from one scan of two 16-bit counts per word (a warp pass has at most
    // 32 x 64 candidates).
    uint32_t incl[K / 2], tot[K];
#pragma unroll
    for (int k = 0; k < K; k += 2) {
      uint32_t x = cnt[k] | (cnt[k + 1] << 16);
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const uint32_t t = __shfl_up_sync(kFull, x, d);
        if (lane >= (unsigned)d) x += t;
      }
      incl[k / 2] = x;
      const uint32_t all = __shfl_sync(kFull, x, 31);
      tot[k] = all & 0xFFFFu;
      tot[k + 1] = all >> 16;
    }
    uint32_t total = 0;
#pragma unroll
    for (int k = 0; k < K; ++k) total += tot[k];
    if (total == 0) continue;  // warp-uniform
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(qcount, total);
    base = __shfl_sync(kFull, base, 0);
    // Within a word: the '+' entries, then the '-' entries, each strand two
    // bits per iteration (its highest and lowest remaining candidates), so a
    // loop runs about half as often as the lane with the most candidates
    // has set bits.  The order inside a word does not matter (the comparer
    // reads a word's windows together; hits are sorted afterwards).
    auto emit = [&](uint32_t* dst) {
      uint32_t pass0 = 0;  // entries of the earlier passes
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const uint32_t mine = (k & 1) ? incl[k / 2] >> 16 : incl[k / 2] & 0xFFFFu;
        uint32_t at = pass0 + mine - cnt[k];
        pass0 += tot[k];
        const uint32_t e0 = (uint32_t)((wb + 32 * k + lane - w_begin) << 6);  // entry of bit 0, '+'
        uint32_t f = fwd[k], r = rev[k];
        while (f) {
          const unsigned hb = 31 - __clz(f), lb = __ffs(f) - 1;
          dst[at] = e0 + 2 * hb;
          if (lb != hb) dst[at + 1] = e0 + 2 * lb;
          at += lb != hb ? 2 : 1;
          f &= ~((1u << hb) | (1u << lb));
        }
        while (r) {
          const unsigned hb = 31 - __clz(r), lb = __ffs(r) - 1;
          dst[at] = e0 + 2 * hb + 1;
          if (lb != hb) dst[at + 1] = e0 + 2 * lb + 1;
          at += lb != hb ? 2 : 1;
          r &= ~((1u << hb) | (1u << lb));
        }
      }
    };
    if (total <= (uint32_t)kFinderStage && vec_queue) {  // warp-uniform
      // Entry i is staged at my[ph + i], so staged word w and queue word
      // base - ph + w share their offset within a 16-byte line.  Whole lines
      // are stored as uint4; the first and last lines, which the warp may
      // share with others, word by word.
      const uint32_t ph = base & 3u;
      emit(my + ph);
      __syncwarp();
      const uint32_t nv = (ph + total + 3) / 4;
      const uint4* src = reinterpret_cast<const uint4*>(my);
      uint32_t* q0 = queue + (base - ph);
      for (uint32_t v = lane; v < nv; v += 32) {
        const uint4 x = src[v];
        if (v > 0 && v + 1 < nv) {
          reinterpret_cast<uint4*>(q0)[v] = x;
        } else {
          const uint32_t w0 = 4 * v, xs[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
          for (uint32_t c = 0; c < 4; ++c)
            if (w0 + c >= ph && w0 + c < ph + total) q0[w0 + c] = xs[c];
        }
      }
      __syncwarp();
    } else if (total <= (uint32_t)kFinderStage) {
      emit(my);
      __syncwarp();
      for (uint32_t i = lane; i < total; i += 32) queue[base + i] = my[i];
      __syncwarp();
    } else {
      emit(queue + base);
    }
  }
}

void launch_finder(const GenomeView& g, uint64_t w_begin, uint64_t w_end, const FinderPattern& pat, uint32_t* queue,
                   uint32_t* qcount, cudaStream_t stream) {
  const uint64_t words = w_end - w_begin;
  uint64_t blocks = (words + kFinderThreads * kFinderWords - 1) / (kFinderThreads * kFinderWords);
  if (blocks > 65535ull * 8) blocks = 65535ull * 8;
  if (blocks == 0) return;
  const uint64_t pos_end = g.n >= pat.L ? g.n - pat.L + 1 : 0;
  FinderMasks fm{};
  fm.L = pat.L;
  fm.nf = pat.nf;
  fm.nr = pat.nr;
  for (uint32_t j = 0; j < pat.nf; ++j) {
    fm.fk[j] = pat.fk[j];
    fm.fc[j] = (uint8_t)(pat.fm[j] & 31u);
  }
  for (uint32_t j = 0; j < pat.nr; ++j) {
    fm.rk[j] = pat.rk[j];
    fm.rc[j] = (uint8_t)(pat.rm[j] & 31u);
  }
  if (pat.L <= 32)
    finder_kernel<1><<<(unsigned)blocks, kFinderThreads, 0, stream>>>(g.hi, g.lo, g.ot, w_begin, w_end, pos_end, fm,
                                                                     queue, qcount);
  else
    finder_kernel<2><<<(unsigned)blocks, kFinderThreads, 0, stream>>>(g.hi, g.lo, g.ot, w_begin, w_end, pos_end, fm,
                                                                     queue, qcount);
}

// ---------------------------------------------------------------- comparer
template <int NW>
struct CandWindow {
  uint32_t h[NW], l[NW], o[NW];
  uint32_t entry;
};

template <int NW>
__global__ void __launch_bounds__(256) comparer_kernel(const uint32_t* __restrict__ hi, const uint32_t* __restrict__ lo,
                                                       const uint32_t* __restrict__ ot,
                                                       const uint32_t* __restrict__ queue,
                                                       const uint32_t* __restrict__ qcount, uint64_t seg_pos0,
                                                       const VariantMask<NW>* __restrict__ vars, uint32_t nvar,
                                                       uint32_t L, uint64_t* __restrict__ hits,
                                                       unsigned long long* __restrict__ hit_count, uint64_t hit_cap) {
  __shared__ CandWindow<NW> tile[256];
  const uint32_t n = *qcount;
  const uint32_t ntiles = (n + 255) / 256;
  for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    // Stage one oriented window per thread.
    const uint32_t idx = t * 256 + threadIdx.x;
    if (idx < n) {
      const uint32_t e = queue[idx];
      const uint64_t pos = seg_pos0 + (e >> 1);
      const uint64_t w = pos >> 5;
      const unsigned r = (unsigned)(pos & 31);
      CandWindow<NW> cw;
      cw.entry = e;
      uint32_t hw[NW], lw[NW], ow[NW];
#pragma unroll
      for (int i = 0; i < NW; ++i) {
        hw[i] = __funnelshift_r(hi[w + i], hi[w + i + 1], r);
        lw[i] = __funnelshift_r(lo[w + i], lo[w + i + 1], r);
        ow[i] = __funnelshift_r(ot[w + i], ot[w + i + 1], r);
      }
      if (e & 1) {
        // Reverse complement of the L-position window: reverse the bit order,
        // then complement the bases (flip hi; non-base bytes keep o = 1).
        if (NW == 1) {
          const unsigned sh = 32 - L;
          cw.h[0] = ~(__brev(hw[0]) >> sh) & (0xFFFFFFFFu >> sh);
          cw.l[0] = __brev(lw[0]) >> sh;
          cw.o[0] = __brev(ow[0]) >> sh;
        } else {
          const unsigned sh = 64 - L;
          const uint64_t mask = ~0ull >> sh;
          const uint64_t H = ~(__brevll(((uint64_t)hw[NW - 1] << 32) | hw[0]) >> sh) & mask;
          const uint64_t Lw = __brevll(((uint64_t)lw[NW - 1] << 32) | lw[0]) >> sh;
          const uint64_t O = __brevll(((uint64_t)ow[NW - 1] << 32) | ow[0]) >> sh;
          cw.h[0] = (uint32_t)H;
          cw.h[NW - 1] = (uint32_t)(H >> 32);
          cw.l[0] = (uint32_t)Lw;
          cw.l[NW - 1] = (uint32_t)(Lw >> 32);
          cw.o[0] = (uint32_t)O;
          cw.o[NW - 1] = (uint32_t)(O >> 32);
        }
      } else {
#pragma unroll
        for (int i = 0; i < NW; ++i) {
          cw.h[i] = hw[i];
          cw.l[i] = lw[i];
          cw.o[i] = ow[i];
        }
      }
      tile[threadIdx.x] = cw;
    }
    __syncthreads();
    const uint32_t m = min(256u, n - t * 256);
    for (uint32_t v = threadIdx.x; v < nvar; v += blockDim.x) {
      const VariantMask<NW> vm = vars[v];
      for (uint32_t c = 0; c < m; ++c) {
        const CandWindow<NW>& cw = tile[c];
        uint32_t mm = 0;
#pragma unroll
        for (int i = 0; i < NW; ++i)
          mm += __popc(mismatch_word(cw.h[i], cw.l[i], cw.o[i], vm.t[i], vm.c[i], vm.a[i], vm.g[i], vm.o[i]));
        if (mm <= vm.thr) {
          const unsigned long long at = atomicAdd(hit_count, 1ull);
          if (at < hit_cap) hits[at] = make_hit(vm.gid, seg_pos0 + (cw.entry >> 1), cw.entry & 1, mm);
        }
      }
    }
    __syncthreads();
  }
}

void launch_comparer(const GenomeView& g, const uint32_t* queue, const uint32_t* qcount, uint64_t seg_pos0,
                     const void* vars, uint32_t nvar, int nw, uint32_t L, uint64_t* hits,
                     unsigned long long* hit_count, uint64_t hit_cap, int sm_count, cudaStream_t stream) {
  if (nvar == 0) return;
  const unsigned blocks = (unsigned)sm_count * 8;
  if (nw == 1)
    comparer_kernel<1><<<blocks, 256, 0, stream>>>(g.hi, g.lo, g.ot, queue, qcount, seg_pos0,
                                                   (const VariantMask<1>*)vars, nvar, L, hits, hit_count, hit_cap);
  else
    comparer_kernel<2><<<blocks, 256, 0, stream>>>(g.hi, g.lo, g.ot, queue, qcount, seg_pos0,
                                                   (const VariantMask<2>*)vars, nvar, L, hits, hit_count, hit_cap);
}

// ---------------------------------------------------------------- formatting
namespace {

__device__ bool dev_mismatch(unsigned char p, unsigned char g) {
  unsigned gb;
  switch (g) {
    case 'T': gb = 0; break;
    case 'C': gb = 1; break;
    case 'A': gb = 2; break;
    case 'G': gb = 3; break;
    default: gb = 4; break;
  }
  return (class_bits_of(p) >> gb) & 1u;
}

__device__ unsigned char dev_complement(unsigned char c) {
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

__device__ unsigned char genome_byte(const GenomeView& g, uint64_t p) {
  const uint64_t w = p >> 5;
  const unsigned b = (unsigned)(p & 31);
  const unsigned h = (g.hi[w] >> b) & 1, l = (g.lo[w] >> b) & 1, o = (g.ot[w] >> b) & 1;
  if (!o) return (unsigned char)"TCAG"[h * 2 + l];
  if (!h) return l ? ';' : 'N';
  uint64_t a = 0, z = g.n_exc;  // first exception position >= p
  while (a < z) {
    const uint64_t mid = (a + z) >> 1;
    if (g.exc_pos[mid] < p) a = mid + 1;
    else z = mid;
  }
  return (a < g.n_exc && g.exc_pos[a] == p) ? g.exc_byte[a] : (unsigned char)'N';
}

__device__ uint32_t record_of(const GenomeView& g, uint64_t p) {
  uint32_t a = 0, z = g.n_rec;  // first start > p
  while (a < z) {
    const uint32_t mid = (a + z) >> 1;
    if (g.rec_start[mid] <= p) a = mid + 1;
    else z = mid;
  }
  return a ? a - 1 : 0;
}

// Decimal text of row numbers.  Values below 2^32 (every location inside a
// record shorter than 4 Gbp, every mismatch count) take 32-bit arithmetic,
// where division by 10 is a multiply-high and a shift; a 64-bit division
// is a long software sequence.
__device__ __forceinline__ uint32_t decimal_len(uint64_t v) {
  if (v <= 0xFFFFFFFFull) {
    const uint32_t x = (uint32_t)v;
    uint32_t d = 1;
    for (uint32_t p = 10; d < 10 && x >= p; p *= 10) ++d;  // 10^9 is the last power below 2^32
    return d;
  }
  uint32_t d = 1;
  while (v >= 10) {
    v /= 10;
    ++d;
  }
  return d;
}

// Writes the digits last to first at their final places (no digit buffer:
// a per-thread array would live in local memory).
__device__ __forceinline__ char* put_decimal(char* o, uint64_t v) {
  const uint32_t len = decimal_len(v);
  char* e = o + len;
  while (v > 0xFFFFFFFFull) {
    *--e = (char)('0' + v % 10);
    v /= 10;
  }
  uint32_t x = (uint32_t)v;
  do {
    *--e = (char)('0' + x % 10);
    x /= 10;
  } while (x);
  return o + len;
}

struct HitView {
  uint32_t gid, strand, mm;
  uint64_t pos;
};
__device__ __forceinline__ HitView decode(uint64_t key) {
  HitView h;
  h.gid = (uint32_t)(key >> 44);
  h.pos = (key >> kHitPosShift) & kHitPosMask;
  h.strand = (uint32_t)((key >> 7) & 1);
  h.mm = (uint32_t)(key & 0x7F);
  return h;
}

}  // namespace

__global__ void row_len_kernel(GenomeView g, FormatTables ft, const uint64_t* __restrict__ hits, uint64_t n_hits,
                               uint64_t* __restrict__ row_bytes, uint32_t* __restrict__ row_count) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_hits) return;
  const HitView h = decode(hits[i]);
  const VariantFmt vf = ft.var[h.gid];
  const uint32_t rec = record_of(g, h.pos);
  const uint64_t rel = h.pos - g.rec_start[rec];
  const uint32_t fixed_sep = 5;  // tabs around chromosome, location, direction, mismatches
  uint64_t bytes = 0;
  for (uint32_t s = vf.shape_begin[h.strand]; s < vf.shape_end[h.strand]; ++s) {
    const ShapeFmt sh = ft.shape[s];
    bytes += sh.head_len + sh.dna_len + g.rec_name_len[rec] + decimal_len(rel + (uint64_t)sh.offset) + 1 +
             decimal_len(h.mm) + sh.tail_len + fixed_sep;
  }
  row_bytes[i] = bytes;
  row_count[i] = vf.shape_end[h.strand] - vf.shape_begin[h.strand];
}

// Rows of one hit at `o` (the bytes row_len_kernel counted).
__device__ __forceinline__ void write_row(const GenomeView& g, const FormatTables& ft, uint64_t key, char* o) {
  const HitView h = decode(key);
  // Fields read in place: a local copy of the struct, indexed by strand,
  // would live in local memory.
  const VariantFmt* vf = ft.var + h.gid;
  const uint32_t L = vf->L;
  const char* comp = ft.pool + vf->comp_off;
  const uint32_t s_begin = vf->shape_begin[h.strand], s_end = vf->shape_end[h.strand];
  // Oriented window with mismatches lower-cased (indicate_mismatches,
  // cas-offinder.cpp:299-317: byte += 32).
  // The window's plane bits, 64 positions from h.pos (three words per plane
  // cover any L <= 64 at any bit offset).
  const uint64_t w0 = h.pos >> 5;
  const unsigned b0 = (unsigned)(h.pos & 31);
  auto bits64 = [&](const uint32_t* plane) {
    const uint64_t lo64 = ((uint64_t)plane[w0 + 1] << 32) | plane[w0];
    return b0 ? (lo64 >> b0) | ((uint64_t)plane[w0 + 2] << (64 - b0)) : lo64;
  };
  const uint64_t H = bits64(g.hi), Lo = bits64(g.lo), O = bits64(g.ot);
  // Oriented position k of the window, as printed; computed where the DNA
  // column asks for it (a per-thread window array would live in local
  // memory).
  auto win = [&](uint32_t k) {
    const uint32_t q = h.strand ? L - 1 - k : k;  // window position of oriented position k
    const unsigned hb = (unsigned)(H >> q) & 1u, lb = (unsigned)(Lo >> q) & 1u;
    unsigned char c;
    // Bytes T, C, A, G (and their complements A, G, T, C) packed low to high.
    if (!((O >> q) & 1u)) c = (unsigned char)((h.strand ? 0x43544741u : 0x47414354u) >> (8 * (hb * 2 + lb)));
    else if (!hb) c = lb ? ';' : 'N';  // complement_byte leaves both as they are
    else c = h.strand ? dev_complement(genome_byte(g, h.pos + q)) : genome_byte(g, h.pos + q);
    if (dev_mismatch((unsigned char)comp[k], c)) c = (unsigned char)(c + 32);
    return c;
  };
  const uint32_t rec = record_of(g, h.pos);
  const uint64_t rel = h.pos - g.rec_start[rec];
  const char* name = g.rec_names + g.rec_name_off[rec];
  const uint32_t name_len = g.rec_name_len[rec];
  for (uint32_t s = s_begin; s < s_end; ++s) {
    const ShapeFmt sh = ft.shape[s];
    for (uint32_t k = 0; k < sh.head_len; ++k) *o++ = ft.pool[sh.head_off + k];
    for (uint32_t k = 0; k < sh.dna_len; ++k) {
      const unsigned char c = (unsigned char)ft.pool[sh.dna_off + k];
      *o++ = (char)(c >= 0x80 ? win(c - 0x80u) : c);
    }
    *o++ = '\t';
    for (uint32_t k = 0; k < name_len; ++k) *o++ = name[k];
    *o++ = '\t';
    o = put_decimal(o, rel + (uint64_t)sh.offset);
    *o++ = '\t';
    *o++ = sh.dir;
    *o++ = '\t';
    o = put_decimal(o, h.mm);
    *o++ = '\t';
    for (uint32_t k = 0; k < sh.tail_len; ++k) *o++ = ft.pool[sh.tail_off + k];
  }
}

// One thread per hit.  A block's rows are one contiguous byte range of the
// output; when it fits in shared memory the threads write it there (placed
// at the same offset mod 16 as in the output) and the block stores it with
// 16-byte stores, otherwise the threads write straight to the output.
constexpr int kRowThreads = 128;
constexpr uint32_t kRowStage = 32768;

__global__ void __launch_bounds__(kRowThreads) write_rows_kernel(GenomeView g, FormatTables ft,
                                                                 const uint64_t* __restrict__ hits, uint64_t n_hits,
                                                                 const uint64_t* __restrict__ offsets,
                                                                 uint64_t out_base, uint64_t total,
                                                                 char* __restrict__ out) {
  __shared__ __align__(16) char stage[kRowStage];
  const uint64_t i0 = (uint64_t)blockIdx.x * kRowThreads, i = i0 + threadIdx.x;
  const uint64_t i1 = min(i0 + kRowThreads, n_hits);
  // Byte positions relative to `out` (offsets - out_base).
  const uint64_t base = offsets[i0] - out_base, end = (i1 < n_hits ? offsets[i1] : total) - out_base;
  const uint64_t a0 = base & ~15ull;  // stage[0] holds output byte a0
  const bool staged = end - a0 <= kRowStage;
  if (i < n_hits)
    write_row(g, ft, hits[i], staged ? stage + (offsets[i] - out_base - a0) : out + (offsets[i] - out_base));
  if (!staged) return;  // the same for the whole block
  __syncthreads();
  for (uint64_t c = a0 + 16 * threadIdx.x; c < end; c += 16 * kRowThreads) {
    const char* src = stage + (c - a0);
    if (c >= base && c + 16 <= end) {
      *(uint4*)(out + c) = *(const uint4*)src;
    } else {
      for (uint32_t k = 0; k < 16; ++k)
        if (c + k >= base && c + k < end) out[c + k] = src[k];
    }
  }
}

void launch_row_lengths(const GenomeView& g, const FormatTables& ft, const uint64_t* hits, uint64_t n_hits,
                        uint64_t* row_bytes, uint32_t* row_count, cudaStream_t stream) {
  if (!n_hits) return;
  row_len_kernel<<<(unsigned)((n_hits + 255) / 256), 256, 0, stream>>>(g, ft, hits, n_hits, row_bytes, row_count);
}

uint64_t write_rows_wave_hits(int sm_count) {
  static int per_sm = 0;
  if (!per_sm && (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, write_rows_kernel, kRowThreads, 0) !=
                      cudaSuccess ||
                  per_sm < 1))
    per_sm = 1;
  return (uint64_t)per_sm * (uint64_t)std::max(sm_count, 1) * kRowThreads;
}

void launch_write_rows(const GenomeView& g, const FormatTables& ft, const uint64_t* hits, uint64_t n_hits,
                       const uint64_t* offsets, uint64_t base, uint64_t end, char* out, cudaStream_t stream) {
  if (!n_hits) return;
  write_rows_kernel<<<(unsigned)((n_hits + kRowThreads - 1) / kRowThreads), kRowThreads, 0, stream>>>(
      g, ft, hits, n_hits, offsets, base, end, out);
}

// Byte offset of each job's first row: job j's hits start at the first sorted
// key whose variant id is >= job_gid0[j]; out[J] = total bytes.
__global__ void job_bounds_kernel(const uint64_t* __restrict__ sorted, uint64_t n, const uint32_t* __restrict__ job_gid0,
                                  uint32_t njobs, const uint64_t* __restrict__ offsets,
                                  const uint64_t* __restrict__ row_bytes, uint64_t* __restrict__ out) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j > njobs) return;
  const uint64_t total = n ? offsets[n - 1] + row_bytes[n - 1] : 0;
  if (j == njobs) {
    out[j] = total;
    return;
  }
  const uint64_t key = (uint64_t)job_gid0[j] << 44;
  uint64_t a = 0, z = n;
  while (a < z) {
    const uint64_t mid = (a + z) >> 1;
    if (sorted[mid] < key) a = mid + 1;
    else z = mid;
  }
  out[j] = a < n ? offsets[a] : total;
}

void launch_job_bounds(const uint64_t* sorted, uint64_t n, const uint32_t* job_gid0, uint32_t njobs,
                       const uint64_t* offsets, const uint64_t* row_bytes, uint64_t* out, cudaStream_t stream) {
  job_bounds_kernel<<<(njobs + 1 + 127) / 128, 128, 0, stream>>>(sorted, n, job_gid0, njobs, offsets, row_bytes, out);
}

__global__ void hit_histogram_kernel(const uint64_t* __restrict__ keys, uint64_t n, uint32_t levels,
                                     uint32_t* __restrict__ counts) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  // Whole warps walk the keys together so that every lane joins the match.
  const uint64_t span = (n + 31) & ~(uint64_t)31;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < span; i += stride) {
    uint32_t idx = 0xFFFFFFFFu;
    if (i < n) {
      const uint64_t k = keys[i];
      idx = ((uint32_t)(k >> 44) * 2 + (uint32_t)((k >> 7) & 1)) * levels + (uint32_t)(k & 0x7F);
    }
    const uint32_t same = __match_any_sync(0xFFFFFFFFu, idx);
    if (idx != 0xFFFFFFFFu && (threadIdx.x & 31) == (uint32_t)(__ffs(same) - 1))
      atomicAdd(&counts[idx], (uint32_t)__popc(same));
  }
}

void launch_hit_histogram(const uint64_t* keys, uint64_t n, uint32_t levels, uint32_t* counts, cudaStream_t stream) {
  if (!n) return;
  const uint64_t blocks = std::min<uint64_t>((n + 255) / 256, 152 * 8);
  hit_histogram_kernel<<<(unsigned)blocks, 256, 0, stream>>>(keys, n, levels, counts);
}

// For each request a (ids from gid0[a]), the index of its first hit in the
// sorted keys; gid0 has one sentinel entry past the last request.
__global__ void run_starts_kernel(const uint64_t* __restrict__ sorted, uint64_t n, const uint32_t* __restrict__ gid0,
                                  uint32_t m, uint64_t* __restrict__ out) {
  const uint32_t a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= m) return;
  const uint64_t key = (uint64_t)gid0[a] << 44;
  uint64_t lo = 0, hi = n;
  while (lo < hi) {
    const uint64_t mid = (lo + hi) >> 1;
    if (sorted[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  out[a] = lo;
}

__global__ void rebase_hits_kernel(const uint64_t* __restrict__ src, uint64_t n, uint32_t gid0,
                                   uint64_t* __restrict__ dst) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[i] - ((uint64_t)gid0 << 44);
}

void launch_run_starts(const uint64_t* sorted, uint64_t n, const uint32_t* gid0, uint32_t m, uint64_t* out,
                       cudaStream_t stream) {
  run_starts_kernel<<<(m + 127) / 128, 128, 0, stream>>>(sorted, n, gid0, m, out);
}

// Each sorted step hit goes to its request's buffer: request a owns ids
// from gid0[a] and the hits [start[a], start[a + 1]) of the step; dst[a] is
// where its run goes (null: the request takes no more hits).
__global__ void scatter_runs_kernel(const uint64_t* __restrict__ sorted, uint64_t n, const uint32_t* __restrict__ gid0,
                                    const uint64_t* __restrict__ start, uint64_t* const* __restrict__ dst, uint32_t m) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t key = sorted[i];
  const uint32_t gid = (uint32_t)(key >> 44);
  uint32_t lo = 0, hi = m;  // last request whose first id <= gid
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (gid0[mid] <= gid) lo = mid;
    else hi = mid;
  }
  uint64_t* d = dst[lo];
  if (d) d[i - start[lo]] = key - ((uint64_t)gid0[lo] << 44);
}

void launch_scatter_runs(const uint64_t* sorted, uint64_t n, const uint32_t* gid0, const uint64_t* start,
                         uint64_t* const* dst, uint32_t m, cudaStream_t stream) {
  if (!n || !m) return;
  scatter_runs_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(sorted, n, gid0, start, dst, m);
}

__global__ void offset_ids_kernel(const uint64_t* __restrict__ src, uint64_t n, uint32_t add,
                                  uint64_t* __restrict__ dst) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[i] + ((uint64_t)add << 44);
}

void launch_offset_ids(const uint64_t* src, uint64_t n, uint32_t add, uint64_t* dst, cudaStream_t stream) {
  if (!n) return;
  offset_ids_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(src, n, add, dst);
}

void launch_rebase_hits(const uint64_t* src, uint64_t n, uint32_t gid0, uint64_t* dst, cudaStream_t stream) {
  if (!n) return;
  rebase_hits_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(src, n, gid0, dst);
}

}  // namespace cof
