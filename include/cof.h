/*
 * cof.h - C ABI of the GB300 Cas-OFFinder search engine (libcasoff.so).
 *
 * The reference (Cas-OFFinder 3.0.0) has no plugin API: its search path sits
 * behind the C++ class Cas_OFFinder (cas-offinder.h:24-107) and the OpenCL
 * kernels finder/comparer (cas-offinder.cl:6-155).  This header is the C ABI
 * that replaces that OpenCL device path.  Every entry point below names the
 * reference interface it stands in for.  All calls return a cof_status
 * (COF_OK = 0) instead of exit(1) (oclfunctions.cpp:5-296), take plain
 * pointers and sizes, and never call exit().  A handle is used by one host
 * thread at a time, like the reference's in-order queues
 * (cas-offinder.cpp:123).
 *
 * Typical use (what the cas-offinder CLI does, mirroring main.cpp:72-157):
 *   cof_open(0, &h);
 *   cof_read_input(h, text, len);                 // readInputFile
 *   cof_genome_load_file(h, path);                // read_fasta / read_twobit
 *   cof_search(h, &rows, &nrows_bytes);           // loadNextChunk..compareAll
 *   fwrite(rows, 1, nrows_bytes, out);
 *   cof_close(h);
 */
#ifndef COF_H
#define COF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int cof_status;
enum {
  COF_OK = 0,
  COF_ERR_CUDA = 1,        /* a CUDA runtime call failed (message in cof_last_error) */
  COF_ERR_ARG = 2,         /* a bad argument (null pointer, size out of range) */
  COF_ERR_NOMEM = 3,       /* device or host allocation failed */
  COF_ERR_INPUT = 4,       /* malformed input file; message = the reference's text */
  COF_ERR_IO = 5,          /* a file could not be read, or the caller's row writer failed */
  COF_ERR_STATE = 6,       /* call out of order (no input or no genome loaded) */
  COF_ERR_UNSUPPORTED = 7, /* pattern longer than COF_MAX_PATTERN; gzip output without zlib */
  COF_ERR_NOT_GENOME = 8,  /* file is neither FASTA nor 2BIT ("Skipping non-acceptable file") */
  COF_ERR_DEVICE = 9,      /* a kernel reported an internal inconsistency */
  COF_ERR_TOO_LARGE = 10,  /* input larger than a fixed limit of the entry point */
  COF_ERR_TIMEOUT = 11     /* a wait ended before the request finished */
};

/* Longest pattern (PAM + spacer + DNA-bulge padding) the kernels accept. */
#define COF_MAX_PATTERN 64

typedef struct cof_handle cof_handle;

/* ---- engine lifetime: Cas_OFFinder::Cas_OFFinder / ~Cas_OFFinder
 *      (cas-offinder.cpp:131-173).  `device` is the CUDA ordinal (the CLI's
 *      G0 selects device 0). */
cof_status cof_open(int device, cof_handle** out);
void cof_close(cof_handle* h);
/* Text of the last error on this handle ("" if none).  Valid until the next call. */
const char* cof_last_error(const cof_handle* h);
/* Same for errors of cof_open itself (no handle exists yet). */
const char* cof_open_error(void);

/* ---- input file: Cas_OFFinder::readInputFile / parseInput
 *      (cas-offinder.cpp:590-751).  `text` holds the whole input file.  On a
 *      malformed file the status is COF_ERR_INPUT and cof_last_error() holds
 *      the reference's message ("Malformed input file." ...). */
cof_status cof_read_input(cof_handle* h, const char* text, size_t len);
/* Line 1 of the input file: genome file or directory (Cas_OFFinder::m_chrdir). */
const char* cof_genome_path(const cof_handle* h);
/* Pattern length L (m_patternlen), number of compare variants (m_compares.size()). */
cof_status cof_input_info(const cof_handle* h, uint32_t* pattern_len, uint32_t* n_variants,
                          uint32_t* n_bulge_records);

/* ---- genome: read_fasta (read_fasta.cpp:11-58) / read_twobit
 *      (read_twobit.cpp:44-131) + Cas_OFFinder::setChrData
 *      (cas-offinder.cpp:175-208).  The genome is packed to 2-bit planes plus
 *      an exception bitmap and stays resident in HBM until replaced.
 *      FASTA is tried first, then 2BIT, as run_cas_offinder does
 *      (main.cpp:49-53); COF_ERR_NOT_GENOME if neither parses. */
cof_status cof_genome_load_file(cof_handle* h, const char* path);
/* The reference's in-memory genome: records joined by ';' (`seq`, n bytes),
 * record names and record start offsets (Cas_OFFinder::m_chrdata, m_chrnames,
 * m_chrpos; cas-offinder.h:86-89). */
cof_status cof_genome_load_text(cof_handle* h, const char* seq, uint64_t n, const char* const* names,
                                const uint64_t* starts, uint32_t n_records);
/* Pre-packed genome (what cof_pack_text produces, e.g. from pinned memory).
 * Plane word w bit b describes position 32*w+b; each plane has
 * cof_plane_words(n) words; bits past position n - 1 are ignored.  The byte
 * before each record start but the first must be the ';' separator, as in the
 * reference's genome string (COF_ERR_ARG otherwise).  `exc_pos`/`exc_byte`
 * list, in ascending position order, the bytes that are not A/C/G/T/N/';'
 * (n_exc entries). */
cof_status cof_genome_load_planes(cof_handle* h, const uint32_t* hi, const uint32_t* lo, const uint32_t* ot,
                                  uint64_t n, const uint64_t* exc_pos, const uint8_t* exc_byte, uint64_t n_exc,
                                  const char* const* names, const uint64_t* starts, uint32_t n_records);
/* Genome length in bytes (separators included) and record count. */
cof_status cof_genome_info(const cof_handle* h, uint64_t* n, uint32_t* n_records);

/* ---- search: loadNextChunk + findPattern + compareAll + releaseLociinfo
 *      (cas-offinder.cpp:210-469, 502-519).  Searches the resident genome
 *      with the current input and formats every output row (the TSV body, no
 *      header lines) on the GPU.  Row order: compare variants in the
 *      reference's std::map key order, hits of a variant by position with '+'
 *      before '-', bulge records of a hit in insertion order - the order the
 *      reference emits for a single chunk with work-items run in order.
 *      `*rows` points into a buffer owned by the handle, valid until the next
 *      search or cof_close. */
cof_status cof_search(cof_handle* h, const char** rows, size_t* rows_len);
/* Receives row text: returns 0 to go on, anything else to stop (the search
 * then returns COF_ERR_IO). */
typedef int (*cof_write_fn)(void* ctx, const char* data, size_t len);
/* cof_search with the rows streamed to `write` in order, in chunks of about
 * 10^6 hits, instead of one buffer (the reference writes rows as it formats
 * them, cas-offinder.cpp:450-455): chunk k+1 is formatted and copied to host
 * memory while the caller writes chunk k, and memory use stays bounded for
 * searches with billions of bytes of rows.  *bytes_written (may be null)
 * = total bytes handed to `write`.  Summary counts as after cof_search. */
cof_status cof_search_stream(cof_handle* h, cof_write_fn write, void* ctx, uint64_t* bytes_written);
/* Load + search in one call, for a genome that lives in host memory (the
 * reference's per-file loop: setChrData, then loadNextChunk / findPattern /
 * compareAll per chunk, cas-offinder.cpp:175-297, 330-469).  Arguments as
 * cof_genome_load_planes, results as cof_search.  From page-locked planes
 * every segment's copy is queued at once on a copy stream and each segment's
 * scan starts as soon as its planes (and the next segment's first words) have
 * arrived, so the copy hides under the search; pageable planes are copied a
 * segment ahead of the scans, each copy synchronous.  The host planes are read
 * only during the call; afterwards the genome stays resident as after
 * cof_genome_load_planes. */
cof_status cof_search_planes(cof_handle* h, const uint32_t* hi, const uint32_t* lo, const uint32_t* ot, uint64_t n,
                             const uint64_t* exc_pos, const uint8_t* exc_byte, uint64_t n_exc,
                             const char* const* names, const uint64_t* starts, uint32_t n_records,
                             const char** rows, size_t* rows_len);
/* ---- batched search: several input files ("jobs") over the resident genome
 * in one pass.  Jobs whose padded patterns are equal share one PAM scan and
 * one comparer launch per genome segment; each job keeps its own compare
 * variants (no key merging across jobs), ids, thresholds and rows, exactly as
 * if it were searched alone.  cof_read_input replaces the batch by a single
 * job; cof_batch_add_input appends one (its `genome path` line is ignored:
 * the batch searches the resident genome).  cof_search then searches every
 * job and returns the rows of all jobs concatenated in job order;
 * cof_job_rows gives one job's rows (valid until the next search). */
cof_status cof_batch_clear(cof_handle* h);
cof_status cof_batch_add_input(cof_handle* h, const char* text, size_t len, uint32_t* job_index);
cof_status cof_batch_size(const cof_handle* h, uint32_t* n_jobs);
cof_status cof_job_rows(const cof_handle* h, uint32_t job, const char** rows, size_t* rows_len);
/* ---- served mode: continuous batching of requests over the resident genome.
 * No counterpart in the reference (one input file per process, main.cpp).
 * A request is one input file (its genome line is ignored).  The server walks
 * the genome as a ring of segments; every ring step searches one segment for
 * all active requests, and waiting requests are admitted at any step boundary
 * while the active compare variants fit `max_active_variants` (0 = 2^17; a
 * request larger than that runs alone).  A request finishes after one full
 * ring, wherever it joined.  Active requests with the same padded pattern
 * share the PAM scan and the comparer launch of each step, but each request's
 * rows are exactly those of cof_search on that input file alone.
 * Memory: the candidate queues are sized by the ring segment and shared by
 * all requests, so admission adds no candidate memory; each running request
 * holds a device hit buffer (8 B per hit) until its rows are formatted.  A
 * request is charged the larger of its hit buffer and a reservation (32 KiB
 * per compare variant within [1, 64] MiB unless cof_server_set_hit_reserve
 * says otherwise), and a waiting request is
 * admitted only while the charges of the running and finishing requests plus
 * its own reservation fit `hit_buffer_bytes` (0 = 8 GiB); nothing running
 * always admits one.  One step's hits must fit `hit_buffer_bytes` as well.
 * While a server runs, use the handle only through server calls;
 * submit/wait/release are thread-safe. */
typedef struct cof_server cof_server;
/* `segment_positions` sets the ring's granularity (rounded down to a multiple
 * of 32, at most 2^26 = the default for 0): smaller segments let requests join
 * and leave sooner at the cost of more launches per ring. */
cof_status cof_server_start(cof_handle* h, uint64_t max_active_variants, uint64_t hit_buffer_bytes,
                            uint64_t segment_positions, cof_server** out);
/* Parses and queues a request; *ticket identifies it.  COF_ERR_INPUT (message
 * in cof_server_last_error) for a malformed input file. */
cof_status cof_server_submit(cof_server* s, const char* text, size_t len, uint64_t* ticket);
/* Waits up to timeout_ms (negative: no limit) for a request.  COF_OK: *rows
 * holds its TSV rows (valid until cof_server_release) and *latency_ms the time
 * from submit to completion; COF_ERR_TIMEOUT: not finished yet. */
cof_status cof_server_wait(cof_server* s, uint64_t ticket, int timeout_ms, const char** rows, size_t* rows_len,
                           double* latency_ms);
cof_status cof_server_release(cof_server* s, uint64_t ticket);
/* Where a finished request's latency went (after cof_server_wait, before
 * cof_server_release), in ms; the four add up to its latency:
 *   admission  submit -> admitted (waiting for the variant and hit budgets)
 *   build      admitted -> its comparer tables in use (host table build, then
 *              the next ring step boundary)
 *   ring       one full ring of steps with its tables
 *   format     ring done -> rows sorted, formatted and in host memory.
 * No counterpart in the reference, which has no request queue. */
cof_status cof_server_timing(cof_server* s, uint64_t ticket, double* admission_ms, double* build_ms, double* ring_ms,
                             double* format_ms);
cof_status cof_server_stats(cof_server* s, uint64_t* steps, uint64_t* admitted, uint64_t* completed,
                            uint64_t* pending, uint64_t* active, uint64_t* max_active);
/* Ring segments one step searches at most (default 4): while a segment takes
 * less than 2 ms to search, a step runs the PAM scans and comparers of that
 * many consecutive segments back to back (the next segment's scan
 * overlapping the current comparer) before the host sorts the step's hits
 * and admits requests, so fewer host round trips per ring; slower segments
 * (a loaded ring) are stepped one at a time.  A step never spans more
 * segments than a running request still needs.  Requests join only at step
 * boundaries.  Applies from the next step. */
cof_status cof_server_set_step_segments(cof_server* s, uint32_t segments);
/* Hit memory charged per running request at least; applies to admissions
 * after the call.  By default (or after a call with 0) a request reserves
 * 32 KiB per compare variant, at least 1 MiB and at most 64 MiB. */
cof_status cof_server_set_hit_reserve(cof_server* s, uint64_t bytes);
/* Device bytes of request hit buffers after the latest ring step, their
 * maximum so far, and the bytes of the two shared candidate queues. */
cof_status cof_server_memory(cof_server* s, uint64_t* held_hit_bytes, uint64_t* max_held_hit_bytes,
                             uint64_t* queue_bytes);
const char* cof_server_last_error(cof_server* s);
/* Stops the worker; requests not finished end with COF_ERR_STATE. */
void cof_server_stop(cof_server* s);

/* ---- served mode over several resident genomes.  No counterpart in the
 * reference, which searches the genome named on line 1 of its input file: one
 * file, or every file of a directory in readdir order with rows written file
 * by file (main.cpp:133-147).  A router keeps such genomes resident on one
 * device, one handle and one server (as cof_server_start) per genome file,
 * and routes each request to the genome its input file's line 1 names; the
 * request's rows are the rows of each file of that genome in its file order,
 * as the CLI writes them (without the header).  Genomes are keyed by their
 * resolved path. */
typedef struct cof_router cof_router;
/* Server settings as cof_server_start, for every genome file.  With auto_load
 * a request naming a genome that is not resident loads it first; without,
 * such a request is refused with COF_ERR_STATE. */
cof_status cof_router_open(int device, uint64_t max_active_variants, uint64_t hit_buffer_bytes,
                           uint64_t segment_positions, int auto_load, cof_router** out);
/* Loads a genome (file or directory) and starts its servers; *n_files (may be
 * NULL) = the genome files kept (files that are neither FASTA nor 2BIT are
 * skipped, as the CLI does).  A genome already resident is not reloaded. */
cof_status cof_router_add_genome(cof_router* r, const char* path, uint32_t* n_files);
/* Stops a genome's servers and frees its device memory; COF_ERR_STATE while
 * requests for it are not released. */
cof_status cof_router_drop_genome(cof_router* r, const char* path);
cof_status cof_router_genomes(cof_router* r, uint32_t* n_genomes, uint32_t* n_files);
/* As cof_server_submit / wait / release; thread-safe.  *latency_ms = submit
 * to completion of the genome's last file. */
cof_status cof_router_submit(cof_router* r, const char* text, size_t len, uint64_t* ticket);
cof_status cof_router_wait(cof_router* r, uint64_t ticket, int timeout_ms, const char** rows, size_t* rows_len,
                           double* latency_ms);
cof_status cof_router_release(cof_router* r, uint64_t ticket);
const char* cof_router_last_error(cof_router* r);
/* Stops every server; requests not finished end. */
void cof_router_close(cof_router* r);

/* ---- gzip row output.  The reference writes plain text (cas-offinder.cpp:450);
 * for searches with GBs of rows the output can be written gzip-compressed:
 * blocks of 8 MiB are deflated on `threads` host threads (0 = one per core),
 * each into one gzip member, and written in order (gunzip, zcat and zlib read
 * the members as one stream).  `level` 1 (fastest) .. 9.  Needs the system
 * zlib (libz.so.1, loaded at run time): COF_ERR_UNSUPPORTED without it.  The
 * CLI uses it when the output file name ends in ".gz".  `path` "-" = stdout. */
typedef struct cof_gzip cof_gzip;
cof_status cof_gzip_open(const char* path, int level, int threads, cof_gzip** out);
cof_status cof_gzip_write(cof_gzip* z, const char* data, size_t len);
/* cof_gzip_write as a cof_write_fn (ctx = the cof_gzip*), for cof_search_stream. */
int cof_gzip_write_fn(void* ctx, const char* data, size_t len);
/* Compresses and writes what is left, closes the file and frees `z`; returns
 * the first error of any write. */
cof_status cof_gzip_close(cof_gzip* z);

/* Hit count of the last search (hits = (variant, position, strand) triples
 * with mismatches <= threshold, before expansion into bulge rows). */
cof_status cof_last_hit_count(const cof_handle* h, uint64_t* n_hits, uint64_t* n_rows);
/* Count rows into the summary table during searches (off by default; the CLI
 * turns it on for --summary, main.cpp:90-97). */
cof_status cof_set_summary(cof_handle* h, int enable);
/* Summary table of all searches since cof_read_input, as the reference writes
 * it with --summary (Cas_OFFinder::writeSummaryTable, cas-offinder.cpp:471-500). */
cof_status cof_summary_text(cof_handle* h, const char** text, size_t* len);
/* The same for one job of a batch (cof_summary_text = job 0). */
cof_status cof_job_summary_text(cof_handle* h, uint32_t job, const char** text, size_t* len);

/* ---- header lines: Cas_OFFinder::writeHeaders (cas-offinder.cpp:319-328). */
const char* cof_header_text(void);

/* ---- kernel-level entry points with the OpenCL kernels' argument contracts.
 * cof_finder_chunk replaces finder/finder_cpu (cas-offinder.cl:6-72,
 * :157-213): `chr` is the chunk (worksize + L - 1 bytes), `pat` the pattern
 * and its reverse complement (2L bytes, as readInputFile builds it,
 * cas-offinder.cpp:708-714).  Outputs candidate start offsets and flags
 * (0 both strands, 1 forward only, 2 reverse only) in ascending offset order;
 * *entrycount receives the count (capacity: worksize entries). */
cof_status cof_finder_chunk(cof_handle* h, const char* chr, uint64_t worksize, const char* pat,
                            uint32_t patternlen, uint32_t* loci, uint8_t* flag, uint32_t* entrycount);
/* cof_comparer_chunk replaces comparer/comparer_cpu (cas-offinder.cl:73-155,
 * :214-286): one compare string `comp` (L bytes; its reverse complement is
 * formed internally) with `threshold`, over `locicnt` candidates.  Hits are
 * written ordered by candidate then '+' before '-' (capacity 2*locicnt). */
cof_status cof_comparer_chunk(cof_handle* h, const char* chr, uint64_t chrlen, const uint32_t* loci,
                              const uint8_t* flag, uint32_t locicnt, const char* comp, uint32_t patternlen,
                              uint16_t threshold, uint32_t* mm_loci, uint16_t* mm_count, char* direction,
                              uint32_t* entrycount);

/* ---- allocation-free chunk search.  No counterpart in the reference: it is
 * for callers that may not allocate device memory when they search (a host
 * application that reserved all its GPU memory in its own pool, or a caller
 * that cannot afford the device-wide synchronization of cudaMalloc/cudaFree).
 * The caller passes device memory for everything it owns: the chunk's genome
 * planes (`d_hi`/`d_lo`/`d_ot`, cof_plane_words(n) words each, packed as
 * cof_pack_text packs, so positions past n read as separators), the hit keys
 * `d_hits` (hit_cap u64: bits 43..8 start position, bit 7 strand ('-' = 1),
 * bits 6..0 mismatches) and the hit counter `d_hit_count` (set to the number
 * of hits; hits past hit_cap are counted, not written).  `pattern` and `comp`
 * are host strings of patternlen bytes (the padded pattern and one compare
 * string; reverse complements are formed internally), `stream` a
 * cudaStream_t (0 = default stream).  Work is queued on `stream`; the results
 * are valid once it completes.  The candidate queue is a fixed 16 MiB device
 * array inside the library (held by every GPU that loads it), so n is limited
 * to 2^21 positions: larger chunks return COF_ERR_TOO_LARGE.  The first call
 * on a device looks up that array's device address; make it before any stream
 * capture.  All calls share the array: calls that overlap on the GPU race, so
 * order them (e.g. one stream).  Nothing is allocated or freed.  `pattern` and
 * `comp` are upper-cased first (as the reference upper-cases its input file);
 * the compare string's masks travel as a kernel argument, so nothing on the
 * host is read after the call returns.  If the calling thread already holds an
 * unread CUDA error, the call returns COF_ERR_CUDA without queuing work and
 * leaves that error for the caller. */
cof_status cof_search_chunk_static(const uint32_t* d_hi, const uint32_t* d_lo, const uint32_t* d_ot, uint64_t n,
                                   const char* pattern, const char* comp, uint32_t patternlen, uint16_t threshold,
                                   uint64_t* d_hits, uint64_t hit_cap, unsigned long long* d_hit_count,
                                   void* stream);

/* ---- packing helpers (host side). */
/* Words per plane for a genome of n bytes (includes the tail padding). */
uint64_t cof_plane_words(uint64_t n);
/* Pack the reference's genome string into planes; returns the number of
 * exception bytes, written to exc_pos/exc_byte when those are non-null
 * (call once with nulls to size them). */
uint64_t cof_pack_text(const char* seq, uint64_t n, uint32_t* hi, uint32_t* lo, uint32_t* ot, uint64_t* exc_pos,
                       uint8_t* exc_byte);

/* ---- comparer selection.  0 (default): the bit-sliced comparer when every
 * compare variant has at most 32 positions that can mismatch, else the
 * popcount comparer; 1: always the popcount comparer; 2: bit-sliced where
 * possible (same as 0).  Both give identical hits. */
cof_status cof_set_comparer(cof_handle* h, int kind);
/* Autotuner of the bit-sliced comparer's lane-program length (variants per
 * lane program): on by default; on the first search of a job set it times the
 * comparer on one genome segment for the cost model's best lengths and keeps
 * the fastest.  Off: the cost model alone chooses. */
cof_status cof_set_autotune(cof_handle* h, int enable);
/* One line per pattern group of the last search: pattern, variants, slots,
 * chosen program length m and chunk count, and the autotuner's timings.
 * Valid until the next call that returns text. */
cof_status cof_schedule_text(cof_handle* h, const char** text, size_t* len);
/* Comparer used by the last search: *kind 1 popcount, 2 bit-sliced; *slots =
 * the bit-sliced slot count (mismatchable positions per variant, padded). */
cof_status cof_comparer_info(const cof_handle* h, int* kind, int* slots);

/* ---- instrumentation: per-kernel CUDA-event timing on the engine's stream. */
cof_status cof_set_profiling(cof_handle* h, int enable);
/* Totals since profiling was enabled for kernel `name` ("finder", "comparer",
 * "format"; "comparer.tests" counts variant tests in `units`,
 * "comparer.lop3" the lane LOP3 instructions the bit-sliced comparer's count
 * issues by its op model, "finder.candidates" the queue entries written,
 * "sort" the hit-key sort, "rows_to_host" the row copies to host memory from
 * the first chunk's copy to the last's end, `units` = bytes): launches,
 * summed device milliseconds and algorithmic units
 * (finder: genome positions scanned; comparer: base comparisons, i.e. the
 * non-N positions of each compare variant times the strand-oriented
 * candidates it was tested against, counted without early exit). */
cof_status cof_kernel_stats(const cof_handle* h, const char* name, uint64_t* launches, double* total_ms,
                            double* units);
cof_status cof_reset_stats(cof_handle* h);
/* Device-side step timer: records a CUDA event on the handle's stream at
 * start and stop; stop waits for the stream and returns the elapsed ms. */
cof_status cof_timer_start(cof_handle* h);
cof_status cof_timer_stop(cof_handle* h, double* ms);
/* Wait for all work of the handle's stream. */
cof_status cof_synchronize(cof_handle* h);

#ifdef __cplusplus
}
#endif

#endif /* COF_H */
