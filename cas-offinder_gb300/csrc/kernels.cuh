// Device data layouts and kernel launchers of the GB300 search path.
//
// Genome: three bit planes (hi, lo, ot), one bit per position, 32 positions
// per uint32 word (layout and code in cof_internal.h).  The planes are read
// in place by every kernel; nothing else of the genome is resident.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace cof {

constexpr int kMaxL = 64;  // longest pattern: two 32-bit words per window

// Per-position mismatch classes of one pattern/compare byte: bit 0 mismatches
// a genome T, bit 1 C, bit 2 A, bit 3 G, bit 4 any non-base byte.
__host__ __device__ inline uint32_t class_bits_of(unsigned char p) {
  switch (p) {
    case 'A': return 0x1Bu;  // T C G other
    case 'C': return 0x1Du;  // T A G other
    case 'G': return 0x17u;  // T C A other
    case 'T': return 0x1Eu;  // C A G other
    case 'R': return 0x03u;  // A/G: T C
    case 'Y': return 0x0Cu;  // C/T: A G
    case 'K': return 0x06u;  // G/T: C A
    case 'M': return 0x09u;  // A/C: T G
    case 'W': return 0x0Au;  // A/T: C G
    case 'S': return 0x05u;  // C/G: T A
    case 'H': return 0x08u;  // A/C/T: G
    case 'B': return 0x04u;  // C/G/T: A
    case 'V': return 0x01u;  // A/C/G: T
    case 'D': return 0x02u;  // A/G/T: C
    default: return 0u;      // N and every other byte never mismatch
  }
}

// PAM scan pattern: the positions of the pattern (forward) and of its reverse
// complement that can mismatch, with their class bits.
struct FinderPattern {
  uint32_t L;
  uint32_t nf, nr;
  uint8_t fk[kMaxL], fm[kMaxL];
  uint8_t rk[kMaxL], rm[kMaxL];
};

// One compare variant as NW-word class masks (bit k = window position k).
template <int NW>
struct VariantMask {
  uint32_t t[NW], c[NW], a[NW], g[NW], o[NW];
  uint32_t thr;  // mismatch limit
  uint32_t gid;  // global variant index (row order rank)
};

// Hit key, sortable into output order:
//   [63:44] global variant index  [43:8] genome position
//   [7] strand (1 = '-')          [6:0] mismatches
constexpr int kHitPosShift = 8;
constexpr uint64_t kHitPosMask = (1ull << 36) - 1;
__host__ __device__ inline uint64_t make_hit(uint32_t gid, uint64_t pos, uint32_t strand, uint32_t mm) {
  return ((uint64_t)gid << 44) | (pos << kHitPosShift) | ((uint64_t)strand << 7) | (uint64_t)mm;
}

// Formatting tables (all offsets into one byte pool).
struct VariantFmt {
  uint32_t comp_off;            // compare string (L bytes)
  uint32_t L;
  uint32_t shape_begin[2], shape_end[2];  // rows per strand
};
struct ShapeFmt {
  uint32_t head_off, head_len, dna_off, dna_len, tail_off, tail_len;
  int64_t offset;
  char dir;
};

struct GenomeView {
  const uint32_t* hi;
  const uint32_t* lo;
  const uint32_t* ot;
  const uint64_t* exc_pos;
  const uint8_t* exc_byte;
  uint64_t n_exc;
  uint64_t n;
  const uint64_t* rec_start;
  const uint32_t* rec_name_off;
  const uint32_t* rec_name_len;
  const char* rec_names;
  uint32_t n_rec;
};

struct FormatTables {
  const VariantFmt* var;
  const ShapeFmt* shape;
  const char* pool;
};

// ---- launchers (kernels.cu).  All run on `stream`, none synchronizes.
// Scans start positions [32*w_begin, 32*w_end) below g.n - L + 1 (windows
// inside the genome) and appends oriented candidate entries
// (position - 32*w_begin) << 1 | strand to `queue`.
void launch_finder(const GenomeView& g, uint64_t w_begin, uint64_t w_end, const FinderPattern& pat, uint32_t* queue,
                   uint32_t* qcount, cudaStream_t stream);
// Tests every entry of `queue` (count read on the device) against `nvar`
// variants; appends hit keys to `hits` (count in *hit_count; entries past
// hit_cap are counted, not written).
void launch_comparer(const GenomeView& g, const uint32_t* queue, const uint32_t* qcount, uint64_t seg_pos0,
                     const void* vars, uint32_t nvar, int nw, uint32_t L, uint64_t* hits,
                     unsigned long long* hit_count, uint64_t hit_cap, int sm_count, cudaStream_t stream);
// Bit-sliced comparer (comparer_bs.cu) for variants with at most 32 positions
// that can mismatch.  The variants come as `chunks` chunks of 32 lane
// programs; a lane program tests up to `m` variants: its first variant is
// counted in full, each later one by updating the count with one added and one
// removed class word per step.  Words per lane program: words = 1 + slots/2 +
// 2 * (m / 2); chunk c occupies words * 32 words from c * words * 32:
//   word 0           bits 0-7: 2^NB - 1 - min(threshold, 2^NB - 1), NB =
//                    bit_width(slots); bit 8: the first variant is real
//   words 1..slots/2 the first variant's slots: u16 shared-memory byte
//                    offsets (class * row + (k + class) % row) * 8, two per
//                    word, 0 = padding
//   (these 1 + slots/2 words lane-minor: word w of lane l at w * 32 + l)
//   then the m - 1 steps (padded to an even count with zero words) as pairs,
//                    step s of lane l at (1 + slots/2) * 32 + ((s / 2) * 32
//                    + l) * 2 + s % 2: bits 0-14 offset of the word added,
//                    bit 15 a variant ends with this step (test it), bits
//                    16-30 offset of the word removed (offset 0 = nothing)
// `pgid[(c * m + e) * 32 + l]` is the global id of lane l's first variant
// (e = 0) and of the variant that its step e - 1 tests (e >= 1; none for a
// step without bit 15).  Returns false if no kernel instance fits (then use
// launch_comparer; also when seg_pos0 is not a multiple of 32: the kernels
// address windows from the segment's first plane word).  `concrete_only`: no
// variant uses a degenerate IUPAC code (only the four concrete-base class rows
// are built).  `narrow` (see bs_narrow_ok): every variant's count fits NB =
// bit_width(slots) planes under the lowered bias, so the update steps carry
// NB planes instead of NB + 1.  `tile_ctr`: a u32 the caller zeroes before
// each launch (CTAs claim tiles from it).
bool launch_comparer_bs(const GenomeView& g, const uint32_t* queue, const uint32_t* qcount, uint64_t seg_pos0,
                        const uint32_t* prog, const uint32_t* pgid, uint32_t chunks, uint32_t m, int slots,
                        bool narrow, uint32_t L, bool concrete_only, uint32_t* tile_ctr, uint64_t* hits,
                        unsigned long long* hit_count, uint64_t hit_cap, int sm_count, cudaStream_t stream);
// Whether lane programs with `slots` class words may count in NB =
// bit_width(slots) planes: with the bias 2^(NB-1) - 1 - t the top plane
// (2^(NB-1)) is set exactly where count > t, and the sum stays below 2^NB,
// when every variant's threshold t < 2^(NB-1) and its positions that can
// mismatch c satisfy c - t <= 2^(NB-1).  (Update steps are exact modulo
// 2^NB, so only the tested variants' counts must fit.)
bool bs_narrow_ok(int slots, const uint32_t* thresholds, const uint32_t* positions, size_t n);
// Op model of the count phase: LOP3-class logic instructions one lane issues
// per pair of 32-candidate groups for a lane program of m variants with
// `slots` class words (full count, bias, m - 1 update steps, hit votes; hit
// emission and the table build aside).  Every lane of a launch runs the same
// count, so a launch issues ceil(candidates / 64) * 32 * chunks times this.
double bs_lane_lop3(int slots, uint32_t m, bool narrow);
int bs_slots_for(int max_positions);  // 0 when more than 32 positions can mismatch
int bs_row_for(uint32_t L);           // words per class row of the shared table
uint32_t bs_class_of(unsigned char p);  // class row of a pattern byte (0: never mismatches)

// Row byte counts per sorted hit (and rows per hit).
void launch_row_lengths(const GenomeView& g, const FormatTables& ft, const uint64_t* hits, uint64_t n_hits,
                        uint64_t* row_bytes, uint32_t* row_count, cudaStream_t stream);
// Writes the rows of hits [0, n_hits) at out + (offsets[i] - base) (offsets:
// exclusive scan of row_bytes; `end` = the byte offset just past the last
// hit's rows).
// Hits one wave of write_rows blocks covers on the whole GPU (one thread per
// hit): launches sized to whole waves leave no SM idle at their tail.
uint64_t write_rows_wave_hits(int sm_count);
void launch_write_rows(const GenomeView& g, const FormatTables& ft, const uint64_t* hits, uint64_t n_hits,
                       const uint64_t* offsets, uint64_t base, uint64_t end, char* out, cudaStream_t stream);

// Per job (global variant ids job_gid0[j] .. job_gid0[j+1]), the byte offset
// of its first row in the formatted text; out[njobs] = total bytes.
void launch_job_bounds(const uint64_t* sorted, uint64_t n, const uint32_t* job_gid0, uint32_t njobs,
                       const uint64_t* offsets, const uint64_t* row_bytes, uint64_t* out, cudaStream_t stream);

// Summary table counts: counts[(gid * 2 + strand) * levels + mm] += 1 for
// each hit key (levels = largest mismatch limit + 1; counts zeroed by the
// caller).  Keys of one (gid, strand, mm) sit next to each other once sorted,
// so each warp adds one atomic per distinct counter it holds.
void launch_hit_histogram(const uint64_t* keys, uint64_t n, uint32_t levels, uint32_t* counts, cudaStream_t stream);

// Served mode: first index of each of m requests' id ranges (ids from
// gid0[a]) in sorted hit keys, and a copy of a run of keys with the request's
// first id subtracted.
void launch_run_starts(const uint64_t* sorted, uint64_t n, const uint32_t* gid0, uint32_t m, uint64_t* out,
                       cudaStream_t stream);
void launch_rebase_hits(const uint64_t* src, uint64_t n, uint32_t gid0, uint64_t* dst, cudaStream_t stream);
// All requests' runs of sorted step keys in one launch: request a (ids from
// gid0[a], keys [start[a], start[a + 1])) gets its run, ids rebased, at
// dst[a] (null: skipped).
void launch_scatter_runs(const uint64_t* sorted, uint64_t n, const uint32_t* gid0, const uint64_t* start,
                         uint64_t* const* dst, uint32_t m, cudaStream_t stream);
// The reverse of launch_rebase_hits: a copy of n keys with `add` added to their variant ids.
void launch_offset_ids(const uint64_t* src, uint64_t n, uint32_t add, uint64_t* dst, cudaStream_t stream);

}  // namespace cof
