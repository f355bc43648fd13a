// Internal types of libcasoff.so shared by engine.cu and server.cu: device
// buffers, the resident genome, pattern groups and the handle.  Not part of
// the public ABI.
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/cof.h"
#include "cof_internal.h"
#include "kernels.cuh"

namespace cof {
namespace eng {

constexpr uint64_t kSegPositions = 1ull << 26;  // start positions per finder/comparer pass
constexpr uint64_t kSegWords = kSegPositions / 32;

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  // With a stream set, allocation and release are stream-ordered
  // (cudaMallocAsync / cudaFreeAsync on it): no device-wide synchronisation.
  cudaStream_t st = nullptr;
  DevBuf() = default;
  explicit DevBuf(cudaStream_t s) : st(s) {}
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), cap(o.cap), st(o.st) { o.p = nullptr, o.cap = 0; }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p, cap = o.cap, st = o.st;
      o.p = nullptr, o.cap = 0;
    }
    return *this;
  }
  ~DevBuf() { release(); }
  void release() {
    if (p) st ? cudaFreeAsync(p, st) : cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    release();
    cudaError_t e = st ? cudaMallocAsync(&p, bytes ? bytes : 1, st) : cudaMalloc(&p, bytes ? bytes : 1);
    if (e == cudaSuccess) cap = bytes;
    else p = nullptr;
    return e;
  }
  template <typename T>
  T* as() const {
    return (T*)p;
  }
};

struct HostPinned {
  void* p = nullptr;
  size_t cap = 0;
  ~HostPinned() {
    if (p) cudaFreeHost(p);
  }
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    cudaError_t e = cudaMallocHost(&p, bytes ? bytes : 1);
    if (e == cudaSuccess) cap = bytes;
    return e;
  }
};

// A genome resident on the device.
struct DevGenome {
  uint64_t n = 0;
  uint32_t n_rec = 0;
  uint64_t n_exc = 0;
  DevBuf hi, lo, ot, exc_pos, exc_byte, rec_start, rec_name_off, rec_name_len, rec_names;
  bool loaded = false;
  GenomeView view() const {
    GenomeView g;
    g.hi = hi.as<uint32_t>();
    g.lo = lo.as<uint32_t>();
    g.ot = ot.as<uint32_t>();
    g.exc_pos = exc_pos.as<uint64_t>();
    g.exc_byte = exc_byte.as<uint8_t>();
    g.n_exc = n_exc;
    g.n = n;
    g.rec_start = rec_start.as<uint64_t>();
    g.rec_name_off = rec_name_off.as<uint32_t>();
    g.rec_name_len = rec_name_len.as<uint32_t>();
    g.rec_names = rec_names.as<char>();
    g.n_rec = n_rec;
    return g;
  }
};

struct KernelStat {
  uint64_t launches = 0;
  double ms = 0;
  double units = 0;
};

// Compare variants (of one or more jobs) that share one padded pattern.
struct PatternGroup {
  std::string pattern;
  uint32_t L = 0;
  FinderPattern fpat{};
  int nw = 1;                  // 32-bit words per window (popcount comparer)
  int bs_slots = 0;            // bit-sliced slot count, 0 = popcount comparer
  bool concrete_only = true;   // no variant uses a degenerate IUPAC code
  bool bs_narrow = false;      // bit-sliced counts fit bit_width(bs_slots) planes (bs_narrow_ok)
  std::vector<uint32_t> gids;  // global variant ids, ascending
  double nonN_sum = 0;         // sum of non-N positions over the group's variants
  // Bit-sliced comparer programs (layout in kernels.cuh): bs_chunks chunks of
  // 32 lane programs, each a first variant and bs_m - 1 update steps.
  uint32_t bs_chunks = 0, bs_m = 1;
  std::vector<uint32_t> bs_candidates;             // lengths m worth timing (cost model's best first)
  std::vector<std::pair<uint32_t, float>> bs_tuned;  // (m, comparer µs per segment) measured by the autotuner
  DevBuf vmask, bs_prog, bs_pgid;
};

}  // namespace eng
}  // namespace cof

using namespace cof;
using namespace cof::eng;

struct cof_handle {
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;   // comparer, formatting, copies
  cudaStream_t stream2 = nullptr;  // finder passes, one segment ahead of the comparer
  cudaEvent_t ev_start = nullptr, ev_found[2] = {nullptr, nullptr}, ev_used[2] = {nullptr, nullptr};
  // Streamed upload (cof_search_planes): plane copies per segment.  From
  // page-locked planes every copy is queued at once on stream3, which runs
  // ahead at the link's rate; upload_ev[c] marks chunk c and the first words
  // of chunk c + 1 (what segment c's windows read) as copied.  From pageable
  // planes the copies go on stream2, one segment ahead of the finders.
  cudaStream_t stream3 = nullptr;
  std::vector<cudaEvent_t> upload_ev;
  size_t upload_pending = 0;  // chunks of the current streamed upload (0: none)
  size_t upload_issued = 0;   // chunks whose copies are queued so far
  bool upload_pinned = false;  // the host planes are page-locked (copies can be graph nodes)
  const uint32_t* upload_src[3] = {nullptr, nullptr, nullptr};  // host planes (valid during the call)
  uint64_t upload_words = 0;
  std::string err;

  // The batch: one or more parsed input files ("jobs").  Variant ids are
  // global and job-major (job j owns [job_gid0[j], job_gid0[j+1])), so one
  // sort of the hit keys yields every job's rows contiguously, in job order.
  std::vector<Job> jobs;
  std::vector<uint32_t> job_gid0;
  bool jobs_on_device = false;
  bool force_popc = false;
  std::vector<PatternGroup> groups;  // jobs sharing a padded pattern share finder + comparer passes
  DevBuf vfmt, sfmt, pool;           // row formatting tables over all variants
  DevGenome genome, scratch;

  DevBuf queue[2], qcounts, hits, hits_sorted, summary_counts, hit_count, sort_tmp, row_bytes, row_offsets, row_count, text, small,
      job_start, job_bytes;
  HostPinned host_text;
  DevBuf stream_dev[2];  // cof_search_stream: row chunks on the device / in pinned memory
  HostPinned stream_host[2];
  cudaEvent_t stream_ev[2] = {nullptr, nullptr};
  std::string summary_text;
  std::vector<std::map<std::string, unsigned long long>> summaries;  // per job
  bool summary_on = false;
  uint64_t last_hits = 0, last_rows = 0;
  std::vector<uint64_t> job_byte0;  // row text of job j: [job_byte0[j], job_byte0[j+1]) of host_text

  bool profiling = false;
  // Pinned host buffers for served results, reused across requests.
  std::mutex pinned_mu;
  std::multimap<size_t, void*> pinned_free;
  size_t pinned_pooled = 0;
  // CUDA graph of the finder / comparer passes of a search, replayed while
  // everything its launches depend on (pass_key) is unchanged.
  cudaGraphExec_t pass_graph = nullptr;
  std::string pass_key;
  uint64_t pass_nseg = 0;
  bool use_graphs = true;
  bool autotune = true;  // time the lane-program lengths on the first search of a job set
  std::map<std::string, KernelStat> stats;
  std::vector<cudaEvent_t> event_pool;  // reused timing events (profiling)
  cudaEvent_t timer_a = nullptr, timer_b = nullptr;
};


namespace cof {
namespace eng {

cof_status fail(cof_handle* h, cof_status st, const std::string& msg);

#define COF_CUDA(h, call)                                                                           \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess)                                                                          \
      return ::cof::eng::fail(h, e_ == cudaErrorMemoryAllocation ? COF_ERR_NOMEM : COF_ERR_CUDA,    \
                              std::string(#call) + ": " + cudaGetErrorString(e_));                  \
  } while (0)

// PAM-scan pattern from the forward pattern and its reverse complement.
bool make_finder_pattern(const std::string& fwd, const std::string& rev, FinderPattern& fp);
std::string revcomp(const std::string& s);
// Initialises g (pattern, L, word count, finder pattern) for a padded pattern.
void init_group(PatternGroup& g, const std::string& pattern);
// Builds and uploads g's comparer tables for its variants `vars` (g.gids
// already set, one id per variant).  Synchronizes h->stream.
// Pool of pinned host buffers kept by the handle: acquire returns a buffer of
// at least `bytes` (its size in *cap), or nullptr; release gives it back.
// Thread-safe.
void* pinned_acquire(cof_handle* h, size_t bytes, size_t* cap);
void pinned_release(cof_handle* h, void* p, size_t cap);

// Host side of a pattern group's comparer tables (built without the GPU).
struct GroupHost {
  std::vector<unsigned char> masks;  // popcount comparer (only when the bit-sliced one cannot run)
  std::vector<uint32_t> prog, pgid;  // bit-sliced lane programs
};
// Fills g's host-side fields (slots, chunks, m, ...) and `gh` for `vars`
// (ids g.gids).  Thread-safe: touches only its arguments.
void build_group_host(bool force_popc, PatternGroup& g, const std::vector<const Variant*>& vars, GroupHost& gh);
// Copies `gh` into g's device buffers on `st`; gh must stay alive until the
// copies are done.
cof_status upload_group(cof_handle* h, PatternGroup& g, const GroupHost& gh, cudaStream_t st);
cof_status build_group_tables(cof_handle* h, PatternGroup& g, const std::vector<const Variant*>& vars);
// Lane programs of the bit-sliced comparer for `vars` (ids `gids`), `S` slots,
// class rows of `row` words; layout in kernels.cuh.
// force_m (1-24) replaces the cost model's choice of m; `ranked` (may be
// null) receives the model's best m and up to two runners-up.
void build_bs_programs(const std::vector<const Variant*>& vars, const std::vector<uint32_t>& gids, int S,
                       uint32_t row, std::vector<uint32_t>& prog, std::vector<uint32_t>& pgid, uint32_t& chunks,
                       uint32_t& m, uint32_t force_m, std::vector<uint32_t>* ranked);
// Row shapes of `vars` (variant i gets id first_gid + i) appended to the
// formatting tables vf (indexed by id), sf and pool.
void append_format_tables(const Job& job, std::vector<VariantFmt>& vf, std::vector<ShapeFmt>& sf, std::string& pool);

}  // namespace eng
}  // namespace cof
