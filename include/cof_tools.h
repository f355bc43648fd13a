/*
 * cof_tools.h - helpers of libcasoff.so that are not part of the reference's
 * interface: a deterministic synthetic genome generator used to make
 * benchmark and test genomes of a stated shape without any download.
 */
#ifndef COF_TOOLS_H
#define COF_TOOLS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Writes `len` bytes of one synthetic record (A, C, G, T, N) to `out`.
 * Bases are drawn i.i.d. with P(G) = P(C) = gc_w / 2 and P(A) = P(T) =
 * (1 - gc_w) / 2, where gc_w = gc + gc_drift * U(-1, 1), redrawn for every
 * window of `drift_window` bases (gc_drift = 0: one GC fraction throughout).
 * Then round(n_frac * len / mean_run) runs of N are placed at uniform starts
 * with lengths uniform in [n_run_min, n_run_max] (runs may overlap).  The
 * output depends only on (seed, record, the parameters): it is the same on
 * every platform and thread count.  Returns the number of N bytes written. */
uint64_t cofx_synth_record(uint64_t seed, uint32_t record, uint64_t len, double gc, double gc_drift,
                           uint32_t drift_window, double n_frac, uint32_t n_run_min, uint32_t n_run_max,
                           char* out);

/* Writes the engine's mismatch predicate as 65536 bytes: out[p * 256 + g] = 1
 * when pattern byte p mismatches genome byte g (the class table every kernel
 * uses: a genome byte is one of T, C, A, G or "any other byte"). */
void cofx_mismatch_table(uint8_t* out);

/* Test hook: loads a FASTA or 2BIT file with the engine's loaders (no GPU
 * needed) and writes the reference's genome string (records joined by ';')
 * to `out` when `cap` suffices; *n = its length.  Returns 0, or 1 when the
 * file is neither format. */
int cofx_genome_text(const char* path, char* out, uint64_t cap, uint64_t* n);

/* Test hook: parses one input file (the whole text) and builds the lane
 * programs of the bit-sliced comparer for its compare variants (layout in
 * cas-offinder_gb300/csrc/kernels.cuh, launch_comparer_bs).  info[0..6] =
 * {chunks, m, slots, class-row words, variants, bytes of keys, narrow}, where
 * narrow = 1 when the counts fit bit_width(slots) planes (bs_narrow_ok; the
 * kernels then use them for programs of more than one variant).  Each output
 * is filled when its capacity suffices: prog chunks * (1 + slots/2 + 2 *
 * (m / 2)) * 32 words, pgid chunks * m * 32 words, keys one "key\tthreshold\n" line per
 * variant in id order.  Returns 0; 1 on a parse error; 2 when the variants do
 * not fit the bit-sliced comparer. */
int cofx_bs_programs(const char* input, size_t len, uint32_t* info, uint32_t* prog, size_t prog_cap, uint32_t* pgid,
                     size_t pgid_cap, char* keys, size_t keys_cap);

#ifdef __cplusplus
}
#endif

#endif /* COF_TOOLS_H */
