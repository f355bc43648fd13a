// Served mode: continuous batching of search requests over the resident genome.
//
// The reference runs one input file per process (main.cpp:72-157).  A server
// keeps the packed genome resident and searches many requests (each one input
// file) at once.  The genome is walked as a ring of segments; one step
// processes one segment for every request in the current comparer tables.
// Requests are admitted at any step boundary -- while others are already
// running -- as long as the admitted compare variants fit the variant budget
// and their hit memory fits the hit budget (below), and each request is
// complete once it has seen every segment of the ring, wherever it joined.  Requests with the same padded pattern share one PAM
// scan and one comparer launch per step, but keep their own variants, ids and
// thresholds, so every request's rows are exactly those of a search of that
// input file alone.
//
// Threads.  cof_server_submit / wait / release may be called from any host
// thread (submit parses the input file on the caller's thread).  Three server
// threads keep host work off the ring:
//   worker    runs the ring steps on the handle's streams;
//   builder   compiles the comparer tables of the admitted set (lane
//             programs, masks) while the worker keeps stepping with the
//             previous tables; the worker adopts a finished set at a step
//             boundary, and a request counts steps only from then on;
//   finisher  sorts and formats a completed request's hits on its own stream
//             and copies the rows into a pinned host buffer taken from the
//             handle's pool (returned on cof_server_release), so delivering
//             GBs of rows touches no fresh pages once the pool is warm.
// Memory.  The candidate queues (two, 2 x segment positions x 4 B each) and
// the step's hit buffer are sized by the ring segment and shared by every
// request, so admitting a request adds no candidate memory.  What grows with
// the admitted set is each request's own device hit buffer (8 B per hit,
// kept until its rows are formatted).  A running request is charged the
// larger of that buffer and a per-request reservation (reserve_of),
// and a waiting request is admitted only while the charges of the running
// and finishing requests plus its own reservation fit hit_buffer_bytes;
// nothing running always admits one.
// Device buffers that change with the request mix are stream-ordered
// (cudaMallocAsync / cudaFreeAsync), so no step waits for a device-wide
// synchronisation.  While a server runs, the handle must not be used for
// anything else.
#include <cub/cub.cuh>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>

#include "engine_internal.h"

namespace {

using namespace cof;
using namespace cof::eng;

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Request {
  uint64_t ticket = 0;
  Job job;
  uint32_t nvar = 0;
  // submit, admitted, first step with its tables, ring complete, rows in host memory
  double t_submit = 0, t_admit = 0, t_adopt = 0, t_ran = 0, t_done = 0;
  // worker-owned until handed to the finisher
  uint64_t steps_seen = 0;
  bool ran = false;  // has completed the ring (or failed): no more hits
  DevBuf hits;       // device hit keys with request-local variant ids
  uint64_t n_hits = 0;
  uint64_t charged = 0;  // hits.cap when handed to the finisher (server's finishing_bytes)
  cudaEvent_t last_append = nullptr;
  // result, published under the server mutex with `done`
  bool done = false;
  cof_status status = COF_OK;
  std::string err;
  char* rows = nullptr;  // pinned buffer from the handle's pool (rows_cap bytes)
  size_t rows_cap = 0;
  uint64_t rows_len = 0;
  cof_handle* pool = nullptr;  // returns `rows` to the pool on destruction
  Request() = default;
  Request(const Request&) = delete;
  Request& operator=(const Request&) = delete;
  ~Request() {
    if (rows) pinned_release(pool, rows, rows_cap);
  }
};

using ReqPtr = std::shared_ptr<Request>;

// Comparer tables of one set of requests: ids request by request in set
// order, groups keyed by padded pattern.
struct TableSet {
  std::vector<ReqPtr> reqs;
  std::vector<uint32_t> gid0;
  std::vector<PatternGroup> groups;
  std::vector<GroupHost> host;  // upload source, kept with the set
};

}  // namespace

struct cof_server {
  cof_handle* h = nullptr;
  uint64_t max_active_variants = 0;
  uint64_t hit_buffer_bytes = 0;
  uint64_t hit_reserve_bytes = 0;  // charged per running request at least; 0: by its variants (reserve_of)
  uint64_t finishing_bytes = 0;              // hit buffers handed to the finisher, not yet freed (under mu)
  uint64_t held_hit_bytes = 0, max_held_hit_bytes = 0;  // after the latest step (under mu)

  std::thread worker, builder, finisher;
  std::mutex mu;
  std::condition_variable cv_work, cv_done, cv_build, cv_finish;
  bool stop = false;
  std::deque<ReqPtr> pending;
  std::vector<ReqPtr> active;  // admitted, not yet through the ring
  std::unordered_map<uint64_t, ReqPtr> tickets;
  uint64_t next_ticket = 1;
  std::string last_error;
  std::atomic<uint64_t> steps{0};
  uint64_t admitted = 0, completed = 0, max_active_seen = 0;

  // builder hand-off (under mu)
  bool build_wanted = false;
  std::vector<ReqPtr> build_input;
  std::unique_ptr<TableSet> built;
  // finisher hand-off (under mu); the finisher drains until the worker is gone
  std::deque<ReqPtr> to_finish;
  bool worker_gone = false;

  // worker-only state
  std::unique_ptr<TableSet> tables;
  uint64_t seg_words = kSegWords;  // plane words (32 start positions each) per ring segment
  std::atomic<uint32_t> step_segments{4};  // ring segments per step at most (cof_server_set_step_segments)
  uint64_t ring = 0, cur = 0;      // ring length in segments, current segment
  DevBuf step_hits, step_sorted, step_count, step_bounds, step_gid0, step_dst, sort_tmp;
  // finisher-only state
  cudaStream_t fin_stream = nullptr;
  DevBuf fmt_in, fmt_hits, fmt_bytes, fmt_off, fmt_cnt, fmt_tmp, fmt_text, fmt_vf, fmt_sf, fmt_pool, fmt_small,
      fmt_gid0, fmt_bounds;
};

namespace {

// Builder thread: compiles the tables of the latest admitted set.
void builder_main(cof_server* s) {
  for (;;) {
    std::vector<ReqPtr> reqs;
    {
      std::unique_lock<std::mutex> lock(s->mu);
      s->cv_build.wait(lock, [&] { return s->stop || s->build_wanted; });
      if (s->stop) return;
      reqs = s->build_input;
      s->build_wanted = false;
    }
    auto ts = std::make_unique<TableSet>();
    ts->reqs = reqs;
    std::map<std::string, size_t> group_of;
    std::vector<std::vector<const Variant*>> vars;
    uint32_t next = 0;
    for (const ReqPtr& r : reqs) {
      ts->gid0.push_back(next);
      auto it = group_of.find(r->job.pattern);
      if (it == group_of.end()) {
        it = group_of.emplace(r->job.pattern, ts->groups.size()).first;
        ts->groups.emplace_back();
        init_group(ts->groups.back(), r->job.pattern);
        vars.emplace_back();
      }
      for (size_t v = 0; v < r->job.variants.size(); ++v) {
        ts->groups[it->second].gids.push_back(next + (uint32_t)v);
        vars[it->second].push_back(&r->job.variants[v]);
      }
      next += r->nvar;
    }
    ts->host.resize(ts->groups.size());
    for (size_t g = 0; g < ts->groups.size(); ++g)
      build_group_host(s->h->force_popc, ts->groups[g], vars[g], ts->host[g]);
    {
      std::lock_guard<std::mutex> lock(s->mu);
      s->built = std::move(ts);
    }
    s->cv_work.notify_all();
  }
}

// Asks the builder for tables of the current admitted set (under mu).
void want_build(cof_server* s) {
  s->build_input = s->active;
  s->build_wanted = true;
  s->cv_build.notify_one();
}

// Device bytes a running request is charged against the hit budget.  Runs
// on the worker thread, the only thread that grows a running request's hits.
// A request's reservation: the set value, or by default 32 KiB per compare
// variant (about the hits a variant finds over a human-sized genome at the
// mismatch limits of the served mix) between 1 and 64 MiB, so a burst of
// small requests is admitted together while a large one still reserves 64 MiB.
uint64_t reserve_of(const cof_server* s, const Request& r) {
  if (s->hit_reserve_bytes) return s->hit_reserve_bytes;
  return std::min<uint64_t>(64ull << 20, std::max<uint64_t>(1ull << 20, (uint64_t)r.nvar << 15));
}
uint64_t hit_charge(const cof_server* s, const Request& r) { return std::max<uint64_t>(r.hits.cap, reserve_of(s, r)); }

// True when the front pending request fits the variant budget and the hit
// memory budget (under mu, on the worker thread).
bool admissible(const cof_server* s) {
  if (s->pending.empty()) return false;
  if (s->active.empty()) return true;
  uint64_t used = 0, bytes = s->finishing_bytes;
  for (const ReqPtr& r : s->active) {
    used += r->nvar;
    bytes += hit_charge(s, *r);
  }
  return used + s->pending.front()->nvar <= s->max_active_variants &&
         bytes + reserve_of(s, *s->pending.front()) <= s->hit_buffer_bytes;
}

// True when the current tables hold a request still walking the ring.
bool tables_live(const cof_server* s) {
  if (!s->tables) return false;
  for (const ReqPtr& r : s->tables->reqs)
    if (!r->ran) return true;
  return false;
}

// One ring step: segments s->cur .. s->cur + k - 1 (mod the ring) for every
// group of the current tables, the finder of each pass on the second stream
// running ahead of the comparers on the first as in a plain search.  Appends
// each hit to its request (request-local variant id) unless the request has
// already completed the ring.  The caller picks k no larger than the
// segments any request of the tables still needs, so no request sees a
// segment twice.
cof_status run_step(cof_server* s, uint64_t k) {
  cof_handle* h = s->h;
  TableSet& T = *s->tables;
  const GenomeView gv = h->genome.view();
  const uint64_t n = h->genome.n;
  uint64_t cap = std::max<uint64_t>(s->step_hits.cap / 8, 1u << 16);
  COF_CUDA(h, s->step_hits.ensure(cap * 8));
  COF_CUDA(h, s->step_count.ensure(8));
  // candidate counts per (segment, group), then the comparer's tile counters
  const size_t nq = std::max<size_t>(T.groups.size(), 1) * (size_t)k;
  COF_CUDA(h, h->qcounts.ensure(2 * nq * 4));
  // at most two oriented candidates per start position of a segment
  COF_CUDA(h, h->queue[0].ensure(2 * s->seg_words * 32 * 4));
  COF_CUDA(h, h->queue[1].ensure(2 * s->seg_words * 32 * 4));
  uint64_t count = 0;
  for (;;) {
    COF_CUDA(h, cudaMemsetAsync(h->qcounts.p, 0, 2 * nq * 4, h->stream));
    COF_CUDA(h, cudaMemsetAsync(s->step_count.p, 0, 8, h->stream));
    COF_CUDA(h, cudaEventRecord(h->ev_start, h->stream));
    COF_CUDA(h, cudaStreamWaitEvent(h->stream2, h->ev_start, 0));
    uint64_t pass = 0;
    for (uint64_t si = 0; si < k; ++si)
    for (size_t gi = 0; gi < T.groups.size(); ++gi) {
      const PatternGroup& g = T.groups[gi];
      const uint64_t npos = n >= g.L ? n - g.L + 1 : 0;
      const uint64_t words = (npos + 31) / 32;
      const uint64_t seg = (s->cur + si) % s->ring;
      const uint64_t w0 = seg * s->seg_words, w1 = std::min(words, w0 + s->seg_words);
      if (w0 >= w1 || g.gids.empty()) continue;
      const int b = (int)(pass & 1);
      uint32_t* qc = h->qcounts.as<uint32_t>() + si * T.groups.size() + gi;
      uint32_t* q = h->queue[b].as<uint32_t>();
      if (pass >= 2) COF_CUDA(h, cudaStreamWaitEvent(h->stream2, h->ev_used[b], 0));
      launch_finder(gv, w0, w1, g.fpat, q, qc, h->stream2);
      COF_CUDA(h, cudaEventRecord(h->ev_found[b], h->stream2));
      COF_CUDA(h, cudaStreamWaitEvent(h->stream, h->ev_found[b], 0));
      const uint32_t V = (uint32_t)g.gids.size();
      if (!g.bs_slots ||
          !launch_comparer_bs(gv, q, qc, w0 * 32, g.bs_prog.as<uint32_t>(), g.bs_pgid.as<uint32_t>(),
                              g.bs_chunks, g.bs_m, g.bs_slots, g.bs_narrow, g.L, g.concrete_only, qc + nq,
                              s->step_hits.as<uint64_t>(), s->step_count.as<unsigned long long>(), cap, h->sm_count,
                              h->stream))
        launch_comparer(gv, q, qc, w0 * 32, g.vmask.p, V, g.nw, g.L, s->step_hits.as<uint64_t>(),
                        s->step_count.as<unsigned long long>(), cap, h->sm_count, h->stream);
      COF_CUDA(h, cudaEventRecord(h->ev_used[b], h->stream));
      ++pass;
    }
    COF_CUDA(h, cudaEventRecord(h->ev_start, h->stream2));
    COF_CUDA(h, cudaStreamWaitEvent(h->stream, h->ev_start, 0));
    COF_CUDA(h, cudaGetLastError());
    COF_CUDA(h, cudaMemcpyAsync(&count, s->step_count.p, 8, cudaMemcpyDeviceToHost, h->stream));
    COF_CUDA(h, cudaStreamSynchronize(h->stream));
    if (count <= cap) break;
    if (count * 8 > s->hit_buffer_bytes)
      return fail(h, COF_ERR_NOMEM, "one ring step found " + std::to_string(count) +
                                        " hits, more than the hit buffer budget allows");
    cap = count + count / 8;
    COF_CUDA(h, s->step_hits.ensure(cap * 8));
  }
  if (count) {
    // Sort the step's hits: each request's ids are one consecutive range, so
    // its hits become one run, appended to the request's own device buffer.
    const size_t A = T.reqs.size();
    COF_CUDA(h, s->step_sorted.ensure(count * 8));
    COF_CUDA(h, s->step_bounds.ensure((A + 1) * 8));
    COF_CUDA(h, s->step_gid0.ensure((A + 1) * 4));
    size_t tmp = 0;
    COF_CUDA(h, cub::DeviceRadixSort::SortKeys(nullptr, tmp, s->step_hits.as<uint64_t>(),
                                               s->step_sorted.as<uint64_t>(), (int64_t)count, 0, 64, h->stream));
    COF_CUDA(h, s->sort_tmp.ensure(tmp));
    tmp = s->sort_tmp.cap;
    COF_CUDA(h, cub::DeviceRadixSort::SortKeys(s->sort_tmp.p, tmp, s->step_hits.as<uint64_t>(),
                                               s->step_sorted.as<uint64_t>(), (int64_t)count, 0, 64, h->stream));
    COF_CUDA(h, cudaMemcpyAsync(s->step_gid0.p, T.gid0.data(), A * 4, cudaMemcpyHostToDevice, h->stream));
    launch_run_starts(s->step_sorted.as<uint64_t>(), count, s->step_gid0.as<uint32_t>(), (uint32_t)A,
                      s->step_bounds.as<uint64_t>(), h->stream);
    std::vector<uint64_t> start(A + 1);
    COF_CUDA(h, cudaMemcpyAsync(start.data(), s->step_bounds.p, A * 8, cudaMemcpyDeviceToHost, h->stream));
    COF_CUDA(h, cudaStreamSynchronize(h->stream));
    start[A] = count;
    // Destinations of each request's run (buffers grown first), then one
    // launch moves every run.
    std::vector<uint64_t*> dst(A, nullptr);
    for (size_t a = 0; a < A; ++a) {
      Request& r = *T.reqs[a];
      const uint64_t k = start[a + 1] - start[a];
      if (!k || r.ran) continue;
      if ((r.n_hits + k) * 8 > r.hits.cap) {  // grow by doubling, keeping the hits so far
        DevBuf bigger(h->stream);
        COF_CUDA(h, bigger.ensure(std::max<uint64_t>((r.n_hits + k) * 8, 2 * r.hits.cap)));
        if (r.n_hits)
          COF_CUDA(h, cudaMemcpyAsync(bigger.p, r.hits.p, r.n_hits * 8, cudaMemcpyDeviceToDevice, h->stream));
        r.hits = std::move(bigger);  // the old buffer is freed in stream order
      }
      dst[a] = r.hits.as<uint64_t>() + r.n_hits;
      r.n_hits += k;
    }
    COF_CUDA(h, s->step_dst.ensure(A * sizeof(uint64_t*)));
    COF_CUDA(h, cudaMemcpyAsync(s->step_bounds.p, start.data(), (A + 1) * 8, cudaMemcpyHostToDevice, h->stream));
    COF_CUDA(h, cudaMemcpyAsync(s->step_dst.p, dst.data(), A * sizeof(uint64_t*), cudaMemcpyHostToDevice, h->stream));
    launch_scatter_runs(s->step_sorted.as<uint64_t>(), count, s->step_gid0.as<uint32_t>(),
                        s->step_bounds.as<uint64_t>(), s->step_dst.as<uint64_t*>(), (uint32_t)A, h->stream);
    COF_CUDA(h, cudaGetLastError());
  }
  s->steps += k;
  return COF_OK;
}

// CUDA check for the finisher: reports through `err`, not the handle.
#define COF_FIN(call)                                                                   \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) {                                                            \
      err = std::string(#call) + ": " + cudaGetErrorString(e_);                         \
      return e_ == cudaErrorMemoryAllocation ? COF_ERR_NOMEM : COF_ERR_CUDA;            \
    }                                                                                   \
  } while (0)

// Formats a batch of finished requests together on the finisher's stream:
// their hits are copied into one buffer with the variant ids of request j
// offset by the variants of the requests before it (the layout of a batched
// search, each request keeping its own ids, thresholds and rows), sorted
// once, their rows written in one pass, and each request's byte range copied
// into a pinned host buffer of its own from the handle's pool.  Requests that
// complete together (a burst that shared a ring pass) thus cost one sort and
// one row pass instead of one each.
cof_status format_batch(cof_server* s, const std::vector<ReqPtr>& rs, std::string& err,
                        const std::function<void(size_t)>& delivered) {
  cof_handle* h = s->h;
  cudaStream_t st = s->fin_stream;
  const size_t k = rs.size();
  std::vector<uint32_t> gid0(k);
  uint64_t nh = 0;
  uint32_t ids = 0;
  for (size_t j = 0; j < k; ++j) {
    if (rs[j]->last_append) COF_FIN(cudaStreamWaitEvent(st, rs[j]->last_append, 0));
    gid0[j] = ids;
    ids += rs[j]->nvar;
    nh += rs[j]->n_hits;
  }
  if (!nh) {
    for (size_t j = 0; j < k; ++j) delivered(j);
    return COF_OK;
  }
  std::vector<VariantFmt> vf;
  std::vector<ShapeFmt> sf;
  std::string pool;
  for (const ReqPtr& r : rs) append_format_tables(r->job, vf, sf, pool);
  COF_FIN(s->fmt_vf.ensure(vf.size() * sizeof(VariantFmt)));
  COF_FIN(s->fmt_sf.ensure(std::max<size_t>(sf.size(), 1) * sizeof(ShapeFmt)));
  COF_FIN(s->fmt_pool.ensure(std::max<size_t>(pool.size(), 1)));
  COF_FIN(s->fmt_in.ensure(nh * 8));
  COF_FIN(s->fmt_hits.ensure(nh * 8));
  COF_FIN(s->fmt_bytes.ensure(nh * 8));
  COF_FIN(s->fmt_off.ensure(nh * 8));
  COF_FIN(s->fmt_cnt.ensure(nh * 4));
  COF_FIN(s->fmt_gid0.ensure(k * 4));
  COF_FIN(s->fmt_bounds.ensure((k + 1) * 8));
  COF_FIN(cudaMemcpyAsync(s->fmt_vf.p, vf.data(), vf.size() * sizeof(VariantFmt), cudaMemcpyHostToDevice, st));
  if (!sf.empty())
    COF_FIN(cudaMemcpyAsync(s->fmt_sf.p, sf.data(), sf.size() * sizeof(ShapeFmt), cudaMemcpyHostToDevice, st));
  if (!pool.empty()) COF_FIN(cudaMemcpyAsync(s->fmt_pool.p, pool.data(), pool.size(), cudaMemcpyHostToDevice, st));
  COF_FIN(cudaMemcpyAsync(s->fmt_gid0.p, gid0.data(), k * 4, cudaMemcpyHostToDevice, st));
  uint64_t at = 0;
  for (size_t j = 0; j < k; ++j) {
    Request& r = *rs[j];
    launch_offset_ids(r.hits.as<uint64_t>(), r.n_hits, gid0[j], s->fmt_in.as<uint64_t>() + at, st);
    at += r.n_hits;
    r.hits.st = st;  // freed in order after its copy on this stream
    r.hits.release();
  }
  // Row order depends on the strand bit, the position and the variant id.
  int end_bit = 44;
  for (uint32_t v = std::max<uint32_t>(ids, 2) - 1; v; v >>= 1) ++end_bit;
  end_bit = std::min(end_bit, 64);
  size_t t0 = 0, t1 = 0;
  COF_FIN(cub::DeviceRadixSort::SortKeys(nullptr, t0, s->fmt_in.as<uint64_t>(), s->fmt_hits.as<uint64_t>(),
                                         (int64_t)nh, 7, end_bit, st));
  COF_FIN(cub::DeviceScan::ExclusiveSum(nullptr, t1, s->fmt_bytes.as<uint64_t>(), s->fmt_off.as<uint64_t>(),
                                        (int64_t)nh, st));
  COF_FIN(s->fmt_tmp.ensure(std::max(t0, t1)));
  t0 = s->fmt_tmp.cap;
  COF_FIN(cub::DeviceRadixSort::SortKeys(s->fmt_tmp.p, t0, s->fmt_in.as<uint64_t>(), s->fmt_hits.as<uint64_t>(),
                                         (int64_t)nh, 7, end_bit, st));
  const GenomeView gv = h->genome.view();
  FormatTables ft{s->fmt_vf.as<VariantFmt>(), s->fmt_sf.as<ShapeFmt>(), s->fmt_pool.as<char>()};
  launch_row_lengths(gv, ft, s->fmt_hits.as<uint64_t>(), nh, s->fmt_bytes.as<uint64_t>(), s->fmt_cnt.as<uint32_t>(),
                     st);
  t1 = s->fmt_tmp.cap;
  COF_FIN(cub::DeviceScan::ExclusiveSum(s->fmt_tmp.p, t1, s->fmt_bytes.as<uint64_t>(), s->fmt_off.as<uint64_t>(),
                                        (int64_t)nh, st));
  launch_job_bounds(s->fmt_hits.as<uint64_t>(), nh, s->fmt_gid0.as<uint32_t>(), (uint32_t)k, s->fmt_off.as<uint64_t>(),
                    s->fmt_bytes.as<uint64_t>(), s->fmt_bounds.as<uint64_t>(), st);
  std::vector<uint64_t> bounds(k + 1);
  COF_FIN(cudaMemcpyAsync(bounds.data(), s->fmt_bounds.p, (k + 1) * 8, cudaMemcpyDeviceToHost, st));
  COF_FIN(cudaStreamSynchronize(st));
  const uint64_t bytes = bounds[k];
  COF_FIN(s->fmt_text.ensure(bytes + 1));
  launch_write_rows(gv, ft, s->fmt_hits.as<uint64_t>(), nh, s->fmt_off.as<uint64_t>(), 0, bytes,
                    s->fmt_text.as<char>(), st);
  COF_FIN(cudaGetLastError());
  COF_FIN(cudaStreamSynchronize(st));
  // Each request's rows go straight to a pinned host buffer from the pool,
  // one request after the other, and each request is delivered as soon as
  // its rows have landed: callers that release their rows promptly hand
  // their buffers back for the next requests of the batch, so a batch does
  // not need all of its rows pinned at once.
  for (size_t j = 0; j < k; ++j) {
    const uint64_t len = bounds[j + 1] - bounds[j];
    rs[j]->rows_len = len;
    if (len) {
      size_t cap = 0;
      char* dst = (char*)pinned_acquire(h, len + 1, &cap);
      if (!dst) {
        err = "no pinned host memory for " + std::to_string(len) + " bytes of rows";
        return COF_ERR_NOMEM;
      }
      rs[j]->pool = h;
      rs[j]->rows = dst;
      rs[j]->rows_cap = cap;
      COF_FIN(cudaMemcpyAsync(dst, s->fmt_text.as<char>() + bounds[j], len, cudaMemcpyDeviceToHost, st));
      COF_FIN(cudaStreamSynchronize(st));
      dst[len] = 0;
    }
    delivered(j);
  }
  return COF_OK;
}

#undef COF_FIN

void finish(cof_server* s, const ReqPtr& r, cof_status st, const std::string& err) {
  std::lock_guard<std::mutex> lock(s->mu);
  r->status = st;
  r->err = err;
  r->done = true;
  r->t_done = now_s();
  ++s->completed;
  s->cv_done.notify_all();
}

// Finisher thread: formats completed requests in completion order, the
// requests waiting when it looks in batches of up to kFinishBatch requests,
// kFinishBatchHits hits (so the batch buffers stay modest and are reused
// from batch to batch) and 2^20 compare variants.
constexpr size_t kFinishBatch = 1024;
constexpr uint64_t kFinishBatchHits = 1ull << 22;

void finisher_main(cof_server* s) {
  cudaSetDevice(s->h->device);
  for (;;) {
    std::vector<ReqPtr> batch;
    {
      std::unique_lock<std::mutex> lock(s->mu);
      s->cv_finish.wait(lock, [&] { return s->worker_gone || !s->to_finish.empty(); });
      if (s->to_finish.empty()) return;  // the worker has stopped and everything is drained
      uint64_t ids = 0, hits = 0;
      while (!s->to_finish.empty() && batch.size() < kFinishBatch &&
             (batch.empty() || (ids + s->to_finish.front()->nvar < (1u << 20) &&
                                hits + s->to_finish.front()->n_hits <= kFinishBatchHits))) {
        ids += s->to_finish.front()->nvar;
        hits += s->to_finish.front()->n_hits;
        batch.push_back(s->to_finish.front());
        s->to_finish.pop_front();
      }
    }
    // Requests that failed on the ring finish with their error; the rest are
    // formatted together and delivered one by one as their rows land.
    auto close = [&](const ReqPtr& r, cof_status st, const std::string& e) {
      r->hits.st = s->fin_stream;
      r->hits.release();
      {
        std::lock_guard<std::mutex> lock(s->mu);
        s->finishing_bytes -= r->charged;
      }
      if (r->last_append) {
        cudaEventDestroy(r->last_append);
        r->last_append = nullptr;
      }
      finish(s, r, st, e);
    };
    std::vector<ReqPtr> ok;
    for (const ReqPtr& r : batch) {
      if (r->status) close(r, r->status, r->err);
      else ok.push_back(r);
    }
    std::vector<bool> closed(ok.size(), false);
    std::string err;
    const cof_status st = ok.empty() ? COF_OK : format_batch(s, ok, err, [&](size_t j) {
      closed[j] = true;
      close(ok[j], COF_OK, std::string());
    });
    for (size_t j = 0; j < ok.size(); ++j)
      if (!closed[j]) close(ok[j], st ? st : COF_ERR_STATE, st ? err : std::string("not formatted"));
  }
}

// Ring steps merge segments while one segment takes less than this (ms).
constexpr double kMergeSegmentsBelowMs = 2.0;

void worker_main(cof_server* s) {
  cof_handle* h = s->h;
  cudaSetDevice(h->device);
  double last_seg_ms = 0;  // host time per segment of the latest step
  const uint64_t words = (h->genome.n + 31) / 32;
  s->ring = std::max<uint64_t>(1, (words + s->seg_words - 1) / s->seg_words);
  for (;;) {
    std::unique_ptr<TableSet> fresh;
    {
      std::unique_lock<std::mutex> lock(s->mu);
      s->cv_work.wait(lock, [&] { return s->stop || admissible(s) || s->built || tables_live(s); });
      if (s->stop) break;
      // Admit waiting requests while the variant budget allows (always at
      // least one, so a request larger than the budget still runs alone).
      bool changed = false;
      while (admissible(s)) {
        const ReqPtr r = s->pending.front();
        s->pending.pop_front();
        r->t_admit = now_s();
        s->active.push_back(r);
        ++s->admitted;
        changed = true;
      }
      s->max_active_seen = std::max<uint64_t>(s->max_active_seen, s->active.size());
      if (changed) want_build(s);
      fresh = std::move(s->built);
    }
    if (fresh) {
      // Adopt the new tables at this step boundary: uploads on the worker's
      // stream, ahead of the step's kernels; the old set's device buffers are
      // freed in stream order.
      cof_status st = COF_OK;
      for (size_t g = 0; g < fresh->groups.size() && !st; ++g) {
        PatternGroup& pg = fresh->groups[g];
        pg.vmask.st = pg.bs_prog.st = pg.bs_pgid.st = h->stream;
        st = upload_group(h, pg, fresh->host[g], h->stream);
      }
      s->tables = std::move(fresh);
      const double t = now_s();
      for (const ReqPtr& r : s->tables->reqs)
        if (r->t_adopt == 0) r->t_adopt = t;
      if (st) {
        std::lock_guard<std::mutex> lock(s->mu);
        for (const ReqPtr& r : s->tables->reqs)
          if (!r->ran) {
            r->ran = true;
            r->status = st;
            r->err = h->err;
            s->to_finish.push_back(r);
          }
        s->active.erase(std::remove_if(s->active.begin(), s->active.end(), [](const ReqPtr& r) { return r->ran; }),
                        s->active.end());
        s->cv_finish.notify_one();
        continue;
      }
    }
    if (!tables_live(s)) continue;
    // Segments this step: up to the step limit while segments are quick to
    // search (the host round trips of a step are then a large share of it);
    // one at a time once the ring is loaded, so that the finisher's short
    // launches find the GPU between steps.  Never more than any request of
    // the tables still needs to complete its ring.
    uint64_t k = last_seg_ms < kMergeSegmentsBelowMs ? std::max<uint64_t>(1, s->step_segments.load()) : 1;
    for (const ReqPtr& r : s->tables->reqs)
      if (!r->ran) k = std::min<uint64_t>(k, s->ring - std::min<uint64_t>(r->steps_seen, s->ring - 1));
    const double t_step = now_s();
    const cof_status st = run_step(s, k);
    last_seg_ms = (now_s() - t_step) * 1e3 / (double)k;
    {
      std::lock_guard<std::mutex> lock(s->mu);
      uint64_t held = s->finishing_bytes;
      for (const ReqPtr& r : s->active) held += r->hits.cap;
      s->held_hit_bytes = held;
      s->max_held_hit_bytes = std::max(s->max_held_hit_bytes, held);
    }
    std::vector<ReqPtr> finished;
    for (const ReqPtr& r : s->tables->reqs)
      if (!r->ran && (st || (r->steps_seen += k) >= s->ring)) finished.push_back(r);
    if (!finished.empty()) {
      const double t = now_s();
      for (const ReqPtr& r : finished) r->t_ran = t;
    }
    if (!finished.empty()) {
      std::lock_guard<std::mutex> lock(s->mu);
      for (const ReqPtr& r : finished) {
        r->ran = true;
        r->charged = r->hits.cap;  // freed by the finisher
        s->finishing_bytes += r->charged;
        if (st) {
          r->status = st;
          r->err = h->err;
        } else if (cudaEventCreateWithFlags(&r->last_append, cudaEventDisableTiming) == cudaSuccess) {
          cudaEventRecord(r->last_append, h->stream);
        }
        s->to_finish.push_back(r);
      }
      s->active.erase(std::remove_if(s->active.begin(), s->active.end(), [](const ReqPtr& r) { return r->ran; }),
                      s->active.end());
      want_build(s);
      s->cv_finish.notify_one();
    }
    s->cur = (s->cur + k) % s->ring;
  }
  // Stopped: requests still queued or running end with COF_ERR_STATE.
  std::vector<ReqPtr> left;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    for (const ReqPtr& r : s->active)
      if (!r->ran) left.push_back(r);
    left.insert(left.end(), s->pending.begin(), s->pending.end());
    s->active.clear();
    s->pending.clear();
  }
  for (const ReqPtr& r : left) {
    r->ran = true;
    r->hits.release();
    finish(s, r, COF_ERR_STATE, "server stopped");
  }
  s->tables.reset();
  cudaStreamSynchronize(h->stream);
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->worker_gone = true;
  }
  s->cv_finish.notify_all();
}

}  // namespace

extern "C" {

cof_status cof_server_start(cof_handle* h, uint64_t max_active_variants, uint64_t hit_buffer_bytes,
                            uint64_t segment_positions, cof_server** out) {
  if (!h || !out) return COF_ERR_ARG;
  *out = nullptr;
  if (!h->genome.loaded) return fail(h, COF_ERR_STATE, "no genome is loaded");
  cudaSetDevice(h->device);
  cof_server* s = new cof_server();
  s->h = h;
  s->max_active_variants = max_active_variants ? max_active_variants : (1u << 17);
  if (s->max_active_variants >= (1u << 20)) s->max_active_variants = (1u << 20) - 1;
  s->hit_buffer_bytes = hit_buffer_bytes ? hit_buffer_bytes : (8ull << 30);
  if (segment_positions) s->seg_words = std::min<uint64_t>(kSegWords, std::max<uint64_t>(1, segment_positions / 32));
  // The finisher's stream has the greatest priority: a completed request's
  // sort and row formatting are small next to the ring's comparer launches,
  // and its CTAs go first whenever an SM frees up, so finished requests are
  // not held behind the steps queued after them.
  int lo_prio = 0, hi_prio = 0;
  cudaError_t e = cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio);
  if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&s->fin_stream, cudaStreamNonBlocking, hi_prio);
  if (e != cudaSuccess) {
    delete s;
    return fail(h, COF_ERR_CUDA, std::string("server stream: ") + cudaGetErrorString(e));
  }
  // Buffers that grow with the request mix are stream-ordered on the stream
  // that uses them (a plain cudaFree would wait for the whole device).
  for (DevBuf* b : {&s->step_hits, &s->step_sorted, &s->step_count, &s->step_bounds, &s->step_gid0, &s->step_dst,
                    &s->sort_tmp})
    b->st = h->stream;
  for (DevBuf* b : {&s->fmt_hits, &s->fmt_bytes, &s->fmt_off, &s->fmt_cnt, &s->fmt_tmp, &s->fmt_text, &s->fmt_vf,
                    &s->fmt_sf, &s->fmt_pool, &s->fmt_small, &s->fmt_in, &s->fmt_gid0, &s->fmt_bounds})
    b->st = s->fin_stream;
  s->worker = std::thread(worker_main, s);
  s->builder = std::thread(builder_main, s);
  s->finisher = std::thread(finisher_main, s);
  *out = s;
  return COF_OK;
}

cof_status cof_server_submit(cof_server* s, const char* text, size_t len, uint64_t* ticket) {
  if (!s || (!text && len) || !ticket) return COF_ERR_ARG;
  auto r = std::make_shared<Request>();
  r->hits.st = s->h->stream;
  std::string err;
  if (!parse_job(text ? text : "", len, r->job, err) || !build_shapes(r->job, err)) {
    std::lock_guard<std::mutex> lock(s->mu);
    s->last_error = err;
    return COF_ERR_INPUT;
  }
  if (r->job.pattern.size() > (size_t)kMaxL) {
    std::lock_guard<std::mutex> lock(s->mu);
    s->last_error = "pattern longer than " + std::to_string(kMaxL);
    return COF_ERR_UNSUPPORTED;
  }
  r->nvar = (uint32_t)r->job.variants.size();
  r->t_submit = now_s();
  {
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->stop) return COF_ERR_STATE;
    if (r->nvar >= (1u << 20)) {
      s->last_error = "request has more than 2^20 compare variants";
      return COF_ERR_UNSUPPORTED;
    }
    r->ticket = s->next_ticket++;
    *ticket = r->ticket;
    s->tickets[r->ticket] = r;
    if (r->nvar == 0) {  // nothing to search: done at once
      r->done = r->ran = true;
      r->t_admit = r->t_adopt = r->t_ran = r->t_done = r->t_submit;
      ++s->completed;
      s->cv_done.notify_all();
      return COF_OK;
    }
    s->pending.push_back(r);
  }
  s->cv_work.notify_one();
  return COF_OK;
}

cof_status cof_server_wait(cof_server* s, uint64_t ticket, int timeout_ms, const char** rows, size_t* rows_len,
                           double* latency_ms) {
  if (!s) return COF_ERR_ARG;
  std::unique_lock<std::mutex> lock(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return COF_ERR_ARG;
  ReqPtr r = it->second;
  auto ready = [&] { return r->done; };
  if (timeout_ms < 0) s->cv_done.wait(lock, ready);
  else if (!s->cv_done.wait_for(lock, std::chrono::milliseconds(timeout_ms), ready)) return COF_ERR_TIMEOUT;
  if (rows) *rows = r->rows ? r->rows : "";
  if (rows_len) *rows_len = r->rows_len;
  if (latency_ms) *latency_ms = (r->t_done - r->t_submit) * 1e3;
  if (r->status) s->last_error = r->err;
  return r->status;
}

cof_status cof_server_timing(cof_server* s, uint64_t ticket, double* admission_ms, double* build_ms, double* ring_ms,
                             double* format_ms) {
  if (!s) return COF_ERR_ARG;
  std::lock_guard<std::mutex> lock(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end() || !it->second->done) return COF_ERR_ARG;
  const Request& r = *it->second;
  // A request that failed before its tables were adopted has no later stages.
  const double adopt = r.t_adopt ? r.t_adopt : r.t_admit, ran = r.t_ran ? r.t_ran : adopt;
  if (admission_ms) *admission_ms = (r.t_admit - r.t_submit) * 1e3;
  if (build_ms) *build_ms = (adopt - r.t_admit) * 1e3;
  if (ring_ms) *ring_ms = (ran - adopt) * 1e3;
  if (format_ms) *format_ms = (r.t_done - ran) * 1e3;
  return COF_OK;
}

cof_status cof_server_release(cof_server* s, uint64_t ticket) {
  if (!s) return COF_ERR_ARG;
  std::lock_guard<std::mutex> lock(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end() || !it->second->done) return COF_ERR_ARG;
  s->tickets.erase(it);
  return COF_OK;
}

cof_status cof_server_set_step_segments(cof_server* s, uint32_t segments) {
  if (!s || segments == 0) return COF_ERR_ARG;
  s->step_segments = segments;
  return COF_OK;
}

cof_status cof_server_set_hit_reserve(cof_server* s, uint64_t bytes) {
  if (!s) return COF_ERR_ARG;
  std::lock_guard<std::mutex> lock(s->mu);
  s->hit_reserve_bytes = bytes;
  return COF_OK;
}

cof_status cof_server_memory(cof_server* s, uint64_t* held_hit_bytes, uint64_t* max_held_hit_bytes,
                             uint64_t* queue_bytes) {
  if (!s) return COF_ERR_ARG;
  std::lock_guard<std::mutex> lock(s->mu);
  if (held_hit_bytes) *held_hit_bytes = s->held_hit_bytes;
  if (max_held_hit_bytes) *max_held_hit_bytes = s->max_held_hit_bytes;
  if (queue_bytes) *queue_bytes = 2 * (2 * s->seg_words * 32 * 4);
  return COF_OK;
}

cof_status cof_server_stats(cof_server* s, uint64_t* steps, uint64_t* admitted, uint64_t* completed,
                            uint64_t* pending, uint64_t* active, uint64_t* max_active) {
  if (!s) return COF_ERR_ARG;
  std::lock_guard<std::mutex> lock(s->mu);
  if (steps) *steps = s->steps.load();
  if (max_active) *max_active = s->max_active_seen;
  if (admitted) *admitted = s->admitted;
  if (completed) *completed = s->completed;
  if (pending) *pending = s->pending.size();
  if (active) *active = s->active.size();
  return COF_OK;
}

const char* cof_server_last_error(cof_server* s) {
  if (!s) return "null server";
  std::lock_guard<std::mutex> lock(s->mu);
  return s->last_error.c_str();
}

void cof_server_stop(cof_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  s->cv_build.notify_all();
  if (s->worker.joinable()) s->worker.join();
  if (s->builder.joinable()) s->builder.join();
  // The finisher drains what the worker handed over, then exits.
  if (s->finisher.joinable()) s->finisher.join();
  cudaSetDevice(s->h->device);
  s->built.reset();
  cudaStreamSynchronize(s->fin_stream);
  cudaStreamSynchronize(s->h->stream);
  cudaStream_t fs = s->fin_stream;
  delete s;
  cudaStreamSynchronize(fs);
  cudaStreamDestroy(fs);
}

}  // extern "C"
