// libcasoff.so: the C ABI of include/cof.h on top of the GB300 kernels.
//
// One handle = one CUDA device, one stream, one resident genome and one
// parsed input file (a "job").  A search walks the genome in segments of
// kSegPositions start positions: the finder appends that segment's oriented
// candidates to a queue, the comparer tests them against every compare
// variant and appends hit keys.  Hits are then sorted on the device into the
// reference's row order and formatted into TSV rows on the device.  The host
// only waits twice per search: for the hit count and for the text size.
#include <cub/cub.cuh>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <iterator>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/cof.h"
#include "../../include/cof_tools.h"
#include "engine_internal.h"

namespace cof {
namespace eng {

cof_status fail(cof_handle* h, cof_status st, const std::string& msg) {
  h->err = msg;
  return st;
}

}  // namespace eng
}  // namespace cof

namespace {

using namespace cof;
using namespace cof::eng;

std::mutex g_open_mu;
std::string g_open_err;

// Uploads a packed genome into `dg` (copies are stream-ordered on h->stream).
// Queues the copies of streamed-upload chunks [issued, upto) on h->stream2,
// the finders' stream: each finder follows the copies queued before it.
cof_status issue_upload(cof_handle* h, size_t upto) {
  upto = std::min(upto, h->upload_pending);
  DevGenome& dg = h->genome;
  const uint64_t W = h->upload_words;
  for (; h->upload_issued < upto; ++h->upload_issued) {
    const size_t c = h->upload_issued;
    const uint64_t w0 = c * kSegWords, nw = std::min<uint64_t>(W - w0, kSegWords);
    uint32_t* dst[3] = {dg.hi.as<uint32_t>(), dg.lo.as<uint32_t>(), dg.ot.as<uint32_t>()};
    for (int p = 0; p < 3; ++p)
      COF_CUDA(h, cudaMemcpyAsync(dst[p] + w0, h->upload_src[p] + w0, nw * 4, cudaMemcpyHostToDevice, h->stream2));
  }
  return COF_OK;
}

// Words of chunk c + 1 that segment c's windows read (a window of up to 64
// positions starting in the chunk's last word ends two words later).
constexpr uint64_t kUploadHeadWords = 2;

// Events upload_ev[0 .. n), created outside any stream capture.
cof_status ensure_upload_events(cof_handle* h, size_t n) {
  while (h->upload_ev.size() < n) {
    cudaEvent_t e = nullptr;
    COF_CUDA(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    h->upload_ev.push_back(e);
  }
  return COF_OK;
}

// Page-locked planes: queues the whole upload on stream3 after the work
// already on h->stream -- chunk 0, then for each c the first words of chunk
// c + 1 and the rest of it -- with upload_ev[c] recorded once chunk c and the
// first words of chunk c + 1 are copied.  The copies then run back to back at
// the link's rate, ahead of the scans that wait for them.
cof_status queue_upload_ahead(cof_handle* h) {
  DevGenome& dg = h->genome;
  const uint64_t W = h->upload_words;
  const size_t chunks = h->upload_pending;
  uint32_t* dst[3] = {dg.hi.as<uint32_t>(), dg.lo.as<uint32_t>(), dg.ot.as<uint32_t>()};
  auto copy = [&](uint64_t w0, uint64_t w1) -> cof_status {
    if (w0 >= w1) return COF_OK;
    for (int p = 0; p < 3; ++p)
      COF_CUDA(h, cudaMemcpyAsync(dst[p] + w0, h->upload_src[p] + w0, (w1 - w0) * 4, cudaMemcpyHostToDevice,
                                  h->stream3));
    return COF_OK;
  };
  COF_CUDA(h, cudaStreamWaitEvent(h->stream3, h->ev_start, 0));
  cof_status st = copy(0, std::min<uint64_t>(W, kSegWords));
  for (size_t c = 0; c < chunks && st == COF_OK; ++c) {
    const uint64_t n0 = (c + 1) * kSegWords;                 // chunk c + 1
    const uint64_t h1 = std::min<uint64_t>(W, n0 + kUploadHeadWords);
    if ((st = copy(n0, h1))) break;
    COF_CUDA(h, cudaEventRecord(h->upload_ev[c], h->stream3));
    st = copy(h1, std::min<uint64_t>(W, n0 + kSegWords));
  }
  h->upload_issued = chunks;
  return st;
}

// With `streamed` the plane copies are left to the search (run_passes queues
// them: see queue_upload_ahead and issue_upload): the host planes must stay
// valid until that search is done.
cof_status upload_genome(cof_handle* h, DevGenome& dg, const uint32_t* hi, const uint32_t* lo, const uint32_t* ot,
                         uint64_t n, const uint64_t* exc_pos, const uint8_t* exc_byte, uint64_t n_exc,
                         const std::vector<std::string>& names, const std::vector<uint64_t>& starts,
                         bool streamed = false) {
  const uint64_t W = plane_words(n);
  dg.loaded = false;
  // The record table must describe the genome like the reference's m_chrpos:
  // first start 0, non-decreasing, inside the genome.
  if (n >= (1ull << 36)) return fail(h, COF_ERR_UNSUPPORTED, "genome longer than 2^36 positions");
  if (names.size() != starts.size()) return fail(h, COF_ERR_ARG, "record names and starts differ in count");
  if (n > 0 && (starts.empty() || starts[0] != 0)) return fail(h, COF_ERR_ARG, "first record must start at 0");
  for (size_t i = 1; i < starts.size(); ++i)
    if (starts[i] < starts[i - 1] || starts[i] > n) return fail(h, COF_ERR_ARG, "record starts must be sorted");
  // Each later record follows a ';' (read_fasta.cpp:41): windows holding it
  // are dropped, so the planes must mark it (other byte, lo set, hi clear).
  for (size_t i = 1; i < starts.size(); ++i) {
    const uint64_t p = starts[i] - 1, w = p >> 5;
    const uint32_t b = 1u << (p & 31);
    if (starts[i] == 0 || !(ot[w] & b) || !(lo[w] & b) || (hi[w] & b))
      return fail(h, COF_ERR_ARG, "no ';' separator before record " + std::to_string(i) + " in the planes");
  }
  COF_CUDA(h, dg.hi.ensure(W * 4));
  COF_CUDA(h, dg.lo.ensure(W * 4));
  COF_CUDA(h, dg.ot.ensure(W * 4));
  h->upload_pending = 0;
  if (!streamed) {
    COF_CUDA(h, cudaMemcpyAsync(dg.hi.p, hi, W * 4, cudaMemcpyHostToDevice, h->stream));
    COF_CUDA(h, cudaMemcpyAsync(dg.lo.p, lo, W * 4, cudaMemcpyHostToDevice, h->stream));
    COF_CUDA(h, cudaMemcpyAsync(dg.ot.p, ot, W * 4, cudaMemcpyHostToDevice, h->stream));
  } else {
    const size_t chunks = (size_t)((W + kSegWords - 1) / kSegWords);
    h->upload_src[0] = hi;
    h->upload_src[1] = lo;
    h->upload_src[2] = ot;
    h->upload_words = W;
    h->upload_issued = 0;
    h->upload_pending = chunks;
  }
  COF_CUDA(h, dg.exc_pos.ensure(n_exc * 8));
  COF_CUDA(h, dg.exc_byte.ensure(n_exc));
  if (n_exc) {
    COF_CUDA(h, cudaMemcpyAsync(dg.exc_pos.p, exc_pos, n_exc * 8, cudaMemcpyHostToDevice, h->stream));
    COF_CUDA(h, cudaMemcpyAsync(dg.exc_byte.p, exc_byte, n_exc, cudaMemcpyHostToDevice, h->stream));
  }
  std::vector<uint32_t> off(names.size()), len(names.size());
  std::string pool;
  for (size_t i = 0; i < names.size(); ++i) {
    off[i] = (uint32_t)pool.size();
    len[i] = (uint32_t)names[i].size();
    pool += names[i];
  }
  const size_t R = std::min(names.size(), starts.size());
  COF_CUDA(h, dg.rec_start.ensure(std::max<size_t>(R, 1) * 8));
  COF_CUDA(h, dg.rec_name_off.ensure(std::max<size_t>(R, 1) * 4));
  COF_CUDA(h, dg.rec_name_len.ensure(std::max<size_t>(R, 1) * 4));
  COF_CUDA(h, dg.rec_names.ensure(std::max<size_t>(pool.size(), 1)));
  if (R) {
    COF_CUDA(h, cudaMemcpyAsync(dg.rec_start.p, starts.data(), R * 8, cudaMemcpyHostToDevice, h->stream));
    COF_CUDA(h, cudaMemcpyAsync(dg.rec_name_off.p, off.data(), R * 4, cudaMemcpyHostToDevice, h->stream));
    COF_CUDA(h, cudaMemcpyAsync(dg.rec_name_len.p, len.data(), R * 4, cudaMemcpyHostToDevice, h->stream));
  }
  if (!pool.empty())
    COF_CUDA(h, cudaMemcpyAsync(dg.rec_names.p, pool.data(), pool.size(), cudaMemcpyHostToDevice, h->stream));
  // Host vectors above are freed on return: wait for the copies.
  COF_CUDA(h, cudaStreamSynchronize(h->stream));
  dg.n = n;
  dg.n_exc = n_exc;
  dg.n_rec = (uint32_t)R;
  dg.loaded = true;
  return COF_OK;
}

cof_status upload_packed(cof_handle* h, DevGenome& dg, const PackedGenome& g) {
  return upload_genome(h, dg, g.hi.data(), g.lo.data(), g.ot.data(), g.n, g.exc_pos.data(), g.exc_byte.data(),
                       g.exc_pos.size(), g.names, g.starts);
}

}  // namespace

namespace cof {
namespace eng {

bool make_finder_pattern(const std::string& fwd, const std::string& rev, FinderPattern& fp) {
  const size_t L = fwd.size();
  if (L == 0 || L > (size_t)kMaxL || rev.size() != L) return false;
  std::memset(&fp, 0, sizeof fp);
  fp.L = (uint32_t)L;
  for (size_t k = 0; k < L; ++k) {
    const uint32_t mf = class_bits_of((unsigned char)fwd[k]);
    if (mf) {
      fp.fk[fp.nf] = (uint8_t)k;
      fp.fm[fp.nf++] = (uint8_t)mf;
    }
    const uint32_t mr = class_bits_of((unsigned char)rev[k]);
    if (mr) {
      fp.rk[fp.nr] = (uint8_t)k;
      fp.rm[fp.nr++] = (uint8_t)mr;
    }
  }
  return true;
}

std::string revcomp(const std::string& s) {
  std::string r(s.rbegin(), s.rend());
  for (char& c : r) c = (char)complement_byte((unsigned char)c);
  return r;
}

template <int NW>
void fill_mask(VariantMask<NW>& vm, const std::string& comp, uint32_t thr, uint32_t gid) {
  std::memset(&vm, 0, sizeof vm);
  for (size_t k = 0; k < comp.size(); ++k) {
    const uint32_t m = class_bits_of((unsigned char)comp[k]);
    const uint32_t bit = 1u << (k & 31);
    const int w = (int)(k >> 5);
    if (m & 1) vm.t[w] |= bit;
    if (m & 2) vm.c[w] |= bit;
    if (m & 4) vm.a[w] |= bit;
    if (m & 8) vm.g[w] |= bit;
    if (m & 16) vm.o[w] |= bit;
  }
  vm.thr = thr;
  vm.gid = gid;
}

void init_group(PatternGroup& g, const std::string& pattern) {
  g.pattern = pattern;
  g.L = (uint32_t)pattern.size();
  g.nw = g.L <= 32 ? 1 : 2;
  make_finder_pattern(pattern, revcomp(pattern), g.fpat);
}

// Lane programs of the bit-sliced comparer (layout in kernels.cuh).
//
// Variants are taken in generation order -- job by job, then by first
// insertion, the order in which the reference's parseInput produces them
// (cas-offinder.cpp:647-682) -- where consecutive DNA-bulge variants of one
// guide differ by one guide base moved across the gap and consecutive
// RNA-bulge variants by one base.  Each such difference is one class word
// added and one removed, so after a first variant counted in full the kernel
// updates the count instead of recounting.  A chain breaks where the next
// variant differs by more than two words each way or has another threshold;
// every step is the exact set difference of the two variants' slots, so the
// counts do not depend on how the chains are cut.  The steps per lane program
// (m - 1) are chosen to minimise the work of the resulting 32-lane chunks.
void build_bs_programs(const std::vector<const Variant*>& vars, const std::vector<uint32_t>& gids, int S,
                       uint32_t row, std::vector<uint32_t>& prog, std::vector<uint32_t>& pgid, uint32_t& chunks,
                       uint32_t& m_out, uint32_t force_m, std::vector<uint32_t>* ranked) {
  const size_t V = vars.size();
  const int NB = [&] { int b = 1; while ((1 << b) <= S) ++b; return b; }();  // bit_width(S)
  // Slots of each variant as sorted u16 offsets, S per variant (cnt used).
  std::vector<uint16_t> slot((size_t)std::max<size_t>(V, 1) * S);
  std::vector<uint8_t> cnt(V);
  std::vector<uint32_t> kadd(V);
  for (size_t i = 0; i < V; ++i) {
    const std::string& key = vars[i]->key;
    uint16_t* sl = &slot[i * S];
    int c = 0;
    for (size_t k = 0; k < key.size() && c < S; ++k) {
      const uint32_t cl = bs_class_of((unsigned char)key[k]);
      if (cl) sl[c++] = (uint16_t)((cl * row + ((uint32_t)k + cl) % row) * 8);
    }
    std::sort(sl, sl + c);
    cnt[i] = (uint8_t)c;
    kadd[i] = (1u << NB) - 1 - std::min<uint32_t>(vars[i]->threshold, (1u << NB) - 1);
  }
  // Generation order: jobs are contiguous runs of one variant array.
  std::vector<uint64_t> rank(V);
  uint64_t job = 0;
  for (size_t i = 0; i < V; ++i) {
    if (i && vars[i] != vars[i - 1] + 1) ++job;
    rank[i] = (job << 32) | vars[i]->order;
  }
  std::vector<uint32_t> ord(V);
  for (size_t i = 0; i < V; ++i) ord[i] = (uint32_t)i;
  std::sort(ord.begin(), ord.end(), [&](uint32_t a, uint32_t b) { return rank[a] < rank[b]; });
  // Steps from variant u to v: (added, removed) offset pairs, 0 = none; at
  // most 2S.  Returns the step count (at least one, so v is tested).
  auto diff = [&](uint32_t u, uint32_t v, uint16_t* add, uint16_t* rem) {
    const uint16_t *x = &slot[(size_t)u * S], *y = &slot[(size_t)v * S];
    int i = 0, j = 0, na = 0, nr = 0;
    while (i < cnt[u] || j < cnt[v]) {
      if (j >= cnt[v] || (i < cnt[u] && x[i] < y[j])) rem[nr++] = x[i++];
      else if (i >= cnt[u] || y[j] < x[i]) add[na++] = y[j++];
      else ++i, ++j;
    }
    const int k = std::max(1, std::max(na, nr));
    for (int t = na; t < k; ++t) add[t] = 0;
    for (int t = nr; t < k; ++t) rem[t] = 0;
    return k;
  };
  std::vector<uint16_t> add(2 * S + 1), rem(2 * S + 1);
  // Chains: cost of each link in steps (0 = chain break before this variant).
  std::vector<uint8_t> link(V, 0);
  for (size_t x = 1; x < V; ++x) {
    const uint32_t u = ord[x - 1], v = ord[x];
    if (kadd[u] != kadd[v]) continue;
    const int k = diff(u, v, add.data(), rem.data());
    if (k <= 2) link[x] = (uint8_t)k;
  }
  // Pieces for a step budget of m - 1: greedy along the chains.
  auto cut = [&](uint32_t m, std::vector<std::pair<size_t, size_t>>* pieces) {
    size_t n = 0, begin = 0;
    uint32_t used = 0;
    for (size_t x = 0; x <= V; ++x) {
      const bool extend = x < V && x > begin && link[x] && used + link[x] <= m - 1;
      if (x > 0 && !extend) {
        if (pieces) pieces->emplace_back(begin, x);
        ++n;
        begin = x;
        used = 0;
      } else if (extend) {
        used += link[x];
      }
    }
    return n;
  };
  // Work per chunk and pair of candidate groups, in issued instructions: a
  // full count ~(4.6 S + 26), a step ~37.
  uint32_t best_m = 1;
  double best = 1e300;
  std::vector<std::pair<double, uint32_t>> costs;
  for (uint32_t m = 1; m <= 24; ++m) {
    const size_t pieces = cut(m, nullptr);
    const double cost = (double)((pieces + 31) / 32) * (4.6 * S + 26 + 37.0 * (m - 1));
    costs.emplace_back(cost, m);
    if (cost < best * 0.999) {
      best = cost;
      best_m = m;
    }
  }
  if (ranked) {
    // Candidates for the autotuner: the model's best and the next cheapest
    // lengths within 1.5x of it (at most three).
    std::stable_sort(costs.begin(), costs.end());
    ranked->assign(1, best_m);
    for (const auto& c : costs)
      if (ranked->size() < 3 && c.second != best_m && c.first <= 1.5 * best) ranked->push_back(c.second);
  }
  if (force_m >= 1 && force_m <= 24) best_m = force_m;
  std::vector<std::pair<size_t, size_t>> pieces;
  cut(best_m, &pieces);
  const uint32_t m = best_m;
  chunks = (uint32_t)((pieces.size() + 31) / 32);
  m_out = m;
  const size_t words = 1 + S / 2 + 2 * (m / 2);
  prog.assign(std::max<size_t>(chunks, 1) * words * 32, 0);
  pgid.assign(std::max<size_t>(chunks, 1) * m * 32, 0xFFFFFFFFu);
  for (size_t pi = 0; pi < pieces.size(); ++pi) {
    const size_t c = pi / 32, l = pi % 32;
    uint32_t* base = &prog[c * words * 32];
    const uint32_t first = ord[pieces[pi].first];
    base[l] = kadd[first] | (1u << 8);
    for (int sl = 0; sl < cnt[first]; ++sl)
      base[(1 + sl / 2) * 32 + l] |= (uint32_t)slot[(size_t)first * S + sl] << (16 * (sl & 1));
    // Ids: entry 0 = the first variant, entry st + 1 = the variant that step
    // st emits (steps that only lead to the next variant have none).
    pgid[(c * m + 0) * 32 + l] = gids[first];
    size_t step = 0;
    for (size_t x = pieces[pi].first + 1; x < pieces[pi].second; ++x) {
      const int k = diff(ord[x - 1], ord[x], add.data(), rem.data());
      for (int j = 0; j < k; ++j, ++step)
        base[(1 + S / 2) * 32 + ((step / 2) * 32 + l) * 2 + step % 2] =
            add[j] | (j + 1 == k ? 0x8000u : 0u) | ((uint32_t)rem[j] << 16);
      pgid[(c * m + step) * 32 + l] = gids[ord[x]];  // emitted by step - 1
    }
  }
}

void* pinned_acquire(cof_handle* h, size_t bytes, size_t* cap) {
  constexpr size_t kUnit = 64ull << 20;
  const size_t want = std::max<size_t>(kUnit, (bytes + kUnit - 1) / kUnit * kUnit);
  {
    std::lock_guard<std::mutex> lock(h->pinned_mu);
    auto it = h->pinned_free.lower_bound(want);
    if (it != h->pinned_free.end() && it->first <= 2 * want) {
      void* p = it->second;
      *cap = it->first;
      h->pinned_pooled -= it->first;
      h->pinned_free.erase(it);
      return p;
    }
  }
  void* p = nullptr;
  if (cudaMallocHost(&p, want) != cudaSuccess) {
    // Give the pool back to the system and try once more.
    std::lock_guard<std::mutex> lock(h->pinned_mu);
    for (auto& kv : h->pinned_free) cudaFreeHost(kv.second);
    h->pinned_free.clear();
    h->pinned_pooled = 0;
    p = nullptr;
    if (cudaMallocHost(&p, want) != cudaSuccess) return nullptr;
  }
  *cap = want;
  return p;
}

void pinned_release(cof_handle* h, void* p, size_t cap) {
  if (!p) return;
  constexpr size_t kMaxPooled = 32ull << 30;
  std::lock_guard<std::mutex> lock(h->pinned_mu);
  h->pinned_free.emplace(cap, p);
  h->pinned_pooled += cap;
  while (h->pinned_pooled > kMaxPooled && !h->pinned_free.empty()) {
    auto big = std::prev(h->pinned_free.end());
    cudaFreeHost(big->second);
    h->pinned_pooled -= big->first;
    h->pinned_free.erase(big);
  }
}

void build_group_host(bool force_popc, PatternGroup& g, const std::vector<const Variant*>& vars, GroupHost& gh) {
  const size_t V = vars.size();
  const size_t msz = g.nw == 1 ? sizeof(VariantMask<1>) : sizeof(VariantMask<2>);
  gh.masks.assign(std::max<size_t>(V, 1) * msz, 0);
  int maxpos = 0;
  g.nonN_sum = 0;
  g.concrete_only = true;
  std::vector<uint32_t> thr(V), npos(V);
  for (size_t i = 0; i < V; ++i) {
    const Variant& var = *vars[i];
    if (g.nw == 1) fill_mask<1>(((VariantMask<1>*)gh.masks.data())[i], var.key, var.threshold, g.gids[i]);
    else fill_mask<2>(((VariantMask<2>*)gh.masks.data())[i], var.key, var.threshold, g.gids[i]);
    int c = 0;
    for (char ch : var.key) {
      const uint32_t cls = bs_class_of((unsigned char)ch);
      c += cls != 0;
      if (cls > 4) g.concrete_only = false;
      g.nonN_sum += ch != 'N';
    }
    maxpos = std::max(maxpos, c);
    thr[i] = var.threshold;
    npos[i] = (uint32_t)c;
  }
  g.bs_slots = force_popc ? 0 : bs_slots_for(maxpos);
  g.bs_narrow = g.bs_slots && bs_narrow_ok(g.bs_slots, thr.data(), npos.data(), V);
  gh.prog.clear();
  gh.pgid.clear();
  g.bs_chunks = 0;
  g.bs_m = 1;
  if (g.bs_slots)
    build_bs_programs(vars, g.gids, g.bs_slots, (uint32_t)bs_row_for(g.L), gh.prog, gh.pgid, g.bs_chunks, g.bs_m, 0,
                      &g.bs_candidates);
}

cof_status upload_group(cof_handle* h, PatternGroup& g, const GroupHost& gh, cudaStream_t st) {
  COF_CUDA(h, g.vmask.ensure(gh.masks.size()));
  COF_CUDA(h, cudaMemcpyAsync(g.vmask.p, gh.masks.data(), gh.masks.size(), cudaMemcpyHostToDevice, st));
  if (g.bs_slots) {
    COF_CUDA(h, g.bs_prog.ensure(gh.prog.size() * 4));
    COF_CUDA(h, g.bs_pgid.ensure(gh.pgid.size() * 4));
    COF_CUDA(h, cudaMemcpyAsync(g.bs_prog.p, gh.prog.data(), gh.prog.size() * 4, cudaMemcpyHostToDevice, st));
    COF_CUDA(h, cudaMemcpyAsync(g.bs_pgid.p, gh.pgid.data(), gh.pgid.size() * 4, cudaMemcpyHostToDevice, st));
  }
  return COF_OK;
}

cof_status build_group_tables(cof_handle* h, PatternGroup& g, const std::vector<const Variant*>& vars) {
  GroupHost gh;
  build_group_host(h->force_popc, g, vars, gh);
  cof_status st = upload_group(h, g, gh, h->stream);
  if (st) return st;
  // The host vectors die on return: wait for the copies.
  COF_CUDA(h, cudaStreamSynchronize(h->stream));
  return COF_OK;
}

void append_format_tables(const Job& job, std::vector<VariantFmt>& vf, std::vector<ShapeFmt>& sf, std::string& pool) {
  auto put = [&](const std::string& str) {
    const uint32_t o = (uint32_t)pool.size();
    pool += str;
    return o;
  };
  for (size_t v = 0; v < job.variants.size(); ++v) {
    VariantFmt f{};
    f.comp_off = put(job.variants[v].key);
    f.L = (uint32_t)job.pattern.size();
    for (int st = 0; st < 2; ++st) {
      f.shape_begin[st] = (uint32_t)sf.size();
      for (const RowShape& r : job.shapes[st][v]) {
        ShapeFmt x;
        x.head_off = put(r.head);
        x.head_len = (uint32_t)r.head.size();
        x.dna_off = put(r.dna);
        x.dna_len = (uint32_t)r.dna.size();
        x.tail_off = put(r.tail);
        x.tail_len = (uint32_t)r.tail.size();
        x.offset = r.offset;
        x.dir = st ? '-' : '+';
        sf.push_back(x);
      }
      f.shape_end[st] = (uint32_t)sf.size();
    }
    vf.push_back(f);
  }
}

}  // namespace eng
}  // namespace cof

namespace {

using namespace cof;
using namespace cof::eng;

// Builds the pattern groups and uploads every variant's comparer and
// formatting tables for the current batch.
// Autotuner of the lane-program length m: the comparer is timed on one full
// genome segment for each of the cost model's candidates (twice each, the
// faster run counts) and the fastest is kept.  Runs once per job set, on the
// first search; groups whose genome is shorter than two segments keep the
// model's choice.
cof_status autotune_group(cof_handle* h, PatternGroup& g, const std::vector<const Variant*>& vars) {
  g.bs_tuned.clear();
  if (!g.bs_slots || g.bs_candidates.size() < 2) return COF_OK;
  const DevGenome& dg = h->genome;
  const uint64_t npos = dg.n >= g.L ? dg.n - g.L + 1 : 0;
  const uint64_t words = (npos + 31) / 32;
  if (words < 2 * kSegWords) return COF_OK;
  const uint64_t w0 = (words / kSegWords / 2) * kSegWords, w1 = std::min(words, w0 + kSegWords);
  COF_CUDA(h, h->queue[0].ensure(2 * kSegPositions * 4));
  COF_CUDA(h, h->qcounts.ensure(std::max<size_t>(h->qcounts.cap, 8)));  // count, tile counter
  COF_CUDA(h, h->hit_count.ensure(8));
  const uint64_t cap = std::max<uint64_t>(h->hits.cap / 8, 1u << 20);
  COF_CUDA(h, h->hits.ensure(cap * 8));
  const GenomeView gv = dg.view();
  uint32_t* q = h->queue[0].as<uint32_t>();
  uint32_t* qc = h->qcounts.as<uint32_t>();
  COF_CUDA(h, cudaMemsetAsync(qc, 0, 4, h->stream));
  launch_finder(gv, w0, w1, g.fpat, q, qc, h->stream);
  cudaEvent_t ev[2] = {nullptr, nullptr};
  for (cudaEvent_t& e : ev) COF_CUDA(h, cudaEventCreate(&e));
  const uint32_t row = (uint32_t)bs_row_for(g.L);
  float best_us = 1e30f;
  uint32_t best_m = g.bs_m, best_chunks = g.bs_chunks;
  std::vector<uint32_t> best_prog, best_pgid;
  cof_status st = COF_OK;
  for (uint32_t m : g.bs_candidates) {
    std::vector<uint32_t> prog, pgid;
    uint32_t chunks = 0, mm = 0;
    build_bs_programs(vars, g.gids, g.bs_slots, row, prog, pgid, chunks, mm, m, nullptr);
    DevBuf dprog, dpgid;
    float us = 1e30f;
    bool declined = false;  // the launcher refused this geometry: m is not a candidate
    auto run = [&]() -> cof_status {
      COF_CUDA(h, dprog.ensure(prog.size() * 4));
      COF_CUDA(h, dpgid.ensure(pgid.size() * 4));
      COF_CUDA(h, cudaMemcpyAsync(dprog.p, prog.data(), prog.size() * 4, cudaMemcpyHostToDevice, h->stream));
      COF_CUDA(h, cudaMemcpyAsync(dpgid.p, pgid.data(), pgid.size() * 4, cudaMemcpyHostToDevice, h->stream));
      for (int rep = 0; rep < 2; ++rep) {
        COF_CUDA(h, cudaMemsetAsync(h->hit_count.p, 0, 8, h->stream));
        COF_CUDA(h, cudaMemsetAsync(qc + 1, 0, 4, h->stream));
        COF_CUDA(h, cudaEventRecord(ev[0], h->stream));
        if (!launch_comparer_bs(gv, q, qc, w0 * 32, dprog.as<uint32_t>(), dpgid.as<uint32_t>(), chunks, mm,
                                g.bs_slots, g.bs_narrow, g.L, g.concrete_only, qc + 1, h->hits.as<uint64_t>(),
                                h->hit_count.as<unsigned long long>(), cap, h->sm_count, h->stream)) {
          declined = true;
          return COF_OK;
        }
        COF_CUDA(h, cudaEventRecord(ev[1], h->stream));
        COF_CUDA(h, cudaEventSynchronize(ev[1]));
        float ms = 0;
        COF_CUDA(h, cudaEventElapsedTime(&ms, ev[0], ev[1]));
        us = std::min(us, ms * 1e3f);
      }
      COF_CUDA(h, cudaGetLastError());
      return COF_OK;
    };
    if ((st = run())) break;
    if (declined) continue;
    g.bs_tuned.emplace_back(mm, us);
    if (us < best_us) {
      best_us = us;
      best_m = mm;
      best_chunks = chunks;
      best_prog.swap(prog);
      best_pgid.swap(pgid);
    }
  }
  for (cudaEvent_t e : ev)
    if (e) cudaEventDestroy(e);
  if (st) return st;
  if (best_m != g.bs_m) {
    COF_CUDA(h, g.bs_prog.ensure(best_prog.size() * 4));
    COF_CUDA(h, g.bs_pgid.ensure(best_pgid.size() * 4));
    COF_CUDA(h, cudaMemcpyAsync(g.bs_prog.p, best_prog.data(), best_prog.size() * 4, cudaMemcpyHostToDevice,
                                h->stream));
    COF_CUDA(h, cudaMemcpyAsync(g.bs_pgid.p, best_pgid.data(), best_pgid.size() * 4, cudaMemcpyHostToDevice,
                                h->stream));
    COF_CUDA(h, cudaStreamSynchronize(h->stream));
    g.bs_m = best_m;
    g.bs_chunks = best_chunks;
  }
  return COF_OK;
}

cof_status upload_jobs(cof_handle* h) {
  if (h->jobs_on_device) return COF_OK;
  h->groups.clear();
  h->job_gid0.assign(1, 0);
  for (const Job& job : h->jobs) {
    if (job.pattern.size() > (size_t)kMaxL)
      return fail(h, COF_ERR_UNSUPPORTED,
                  "pattern length " + std::to_string(job.pattern.size()) + " exceeds " + std::to_string(kMaxL));
    h->job_gid0.push_back(h->job_gid0.back() + (uint32_t)job.variants.size());
  }
  const uint64_t total = h->job_gid0.back();
  if (total >= (1u << 20)) return fail(h, COF_ERR_UNSUPPORTED, "more than 2^20 compare variants in one batch");
  std::map<std::string, size_t> group_of;
  std::vector<std::vector<const Variant*>> group_vars;
  for (size_t j = 0; j < h->jobs.size(); ++j) {
    const Job& job = h->jobs[j];
    auto it = group_of.find(job.pattern);
    if (it == group_of.end()) {
      it = group_of.emplace(job.pattern, h->groups.size()).first;
      h->groups.emplace_back();
      init_group(h->groups.back(), job.pattern);
      group_vars.emplace_back();
    }
    for (size_t v = 0; v < job.variants.size(); ++v) {
      h->groups[it->second].gids.push_back(h->job_gid0[j] + (uint32_t)v);
      group_vars[it->second].push_back(&job.variants[v]);
    }
  }
  // Formatting tables over all variants (ids are job-major, so appending job
  // by job gives id order).
  std::string pool;
  std::vector<VariantFmt> vf;
  std::vector<ShapeFmt> sf;
  for (const Job& job : h->jobs) append_format_tables(job, vf, sf, pool);
  if (pool.size() >= (1ull << 32)) return fail(h, COF_ERR_UNSUPPORTED, "row tables exceed 4 GB");
  for (size_t gi = 0; gi < h->groups.size(); ++gi) {
    cof_status st = build_group_tables(h, h->groups[gi], group_vars[gi]);
    if (st) return st;
  }
  // The planes of a streamed upload are not resident yet: such a search
  // keeps the cost model's choice.
  if (h->autotune && !h->upload_pending)
    for (size_t gi = 0; gi < h->groups.size(); ++gi) {
      cof_status st = autotune_group(h, h->groups[gi], group_vars[gi]);
      if (st) return st;
    }
  COF_CUDA(h, h->vfmt.ensure(std::max<size_t>(total, 1) * sizeof(VariantFmt)));
  COF_CUDA(h, h->sfmt.ensure(std::max<size_t>(sf.size(), 1) * sizeof(ShapeFmt)));
  COF_CUDA(h, h->pool.ensure(std::max<size_t>(pool.size(), 1)));
  if (total)
    COF_CUDA(h, cudaMemcpyAsync(h->vfmt.p, vf.data(), total * sizeof(VariantFmt), cudaMemcpyHostToDevice, h->stream));
  if (!sf.empty())
    COF_CUDA(h, cudaMemcpyAsync(h->sfmt.p, sf.data(), sf.size() * sizeof(ShapeFmt), cudaMemcpyHostToDevice, h->stream));
  if (!pool.empty()) COF_CUDA(h, cudaMemcpyAsync(h->pool.p, pool.data(), pool.size(), cudaMemcpyHostToDevice, h->stream));
  COF_CUDA(h, cudaStreamSynchronize(h->stream));
  h->jobs_on_device = true;
  return COF_OK;
}

struct EventPair {
  cudaEvent_t a = nullptr, b = nullptr;
  std::string name;
  double units = 0;
};

cof_status record_start(cof_handle* h, std::vector<EventPair>& evs, const char* name, double units,
                        cudaStream_t st) {
  if (!h->profiling) return COF_OK;
  EventPair p;
  p.name = name;
  p.units = units;
  for (cudaEvent_t* e : {&p.a, &p.b}) {
    if (!h->event_pool.empty()) {
      *e = h->event_pool.back();
      h->event_pool.pop_back();
    } else {
      COF_CUDA(h, cudaEventCreate(e));
    }
  }
  COF_CUDA(h, cudaEventRecord(p.a, st));
  evs.push_back(p);
  return COF_OK;
}
cof_status record_stop(cof_handle* h, std::vector<EventPair>& evs, cudaStream_t st) {
  if (!h->profiling) return COF_OK;
  COF_CUDA(h, cudaEventRecord(evs.back().b, st));
  return COF_OK;
}
void collect(cof_handle* h, std::vector<EventPair>& evs) {
  for (EventPair& p : evs) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      KernelStat& s = h->stats[p.name];
      s.launches += 1;
      s.ms += ms;
      s.units += p.units;
    }
    h->event_pool.push_back(p.a);
    h->event_pool.push_back(p.b);
  }
  evs.clear();
}

// Finder + comparer over the whole genome for every pattern group; leaves the
// hit count in h->hit_count.  Pass i = (segment s, group g) scans on stream2
// into queue[i % 2] while the comparer works on pass i - 1 on the main
// stream; events order the two.  qcounts[s * groups + g] keeps each pass's
// candidate count.
cof_status run_passes(cof_handle* h, uint64_t hit_cap, std::vector<EventPair>& evs, uint64_t* seg_count) {
  const DevGenome& dg = h->genome;
  const GenomeView gv = dg.view();
  const size_t G = h->groups.size();
  uint64_t max_words = 0;
  for (const PatternGroup& g : h->groups) {
    const uint64_t npos = dg.n >= g.L ? dg.n - g.L + 1 : 0;
    max_words = std::max(max_words, (npos + 31) / 32);
  }
  const uint64_t nseg = (max_words + kSegWords - 1) / kSegWords;
  *seg_count = nseg;
  // qcounts: candidate counts per pass, then the comparer's tile counters.
  const uint64_t nq = std::max<uint64_t>(nseg * G, 1);
  COF_CUDA(h, h->qcounts.ensure(2 * nq * 4));
  COF_CUDA(h, cudaMemsetAsync(h->qcounts.p, 0, 2 * nq * 4, h->stream));
  COF_CUDA(h, cudaMemsetAsync(h->hit_count.p, 0, 8, h->stream));
  COF_CUDA(h, cudaEventRecord(h->ev_start, h->stream));
  COF_CUDA(h, cudaStreamWaitEvent(h->stream2, h->ev_start, 0));
  // A streamed upload from page-locked planes is queued whole on stream3;
  // from pageable planes it follows the scans (issue_upload below).
  const bool ahead = h->upload_pending && h->upload_pinned;
  if (ahead) {
    if (h->upload_ev.size() < h->upload_pending)
      return fail(h, COF_ERR_STATE, "upload events not created before the passes");
    cof_status st = queue_upload_ahead(h);
    if (st) return st;
  }
  uint64_t pass = 0;
  for (uint64_t s = 0; s < nseg; ++s) {
    for (size_t gi = 0; gi < G; ++gi) {
      const PatternGroup& g = h->groups[gi];
      const uint64_t npos = dg.n >= g.L ? dg.n - g.L + 1 : 0;
      const uint64_t words = (npos + 31) / 32;
      const uint64_t w0 = s * kSegWords, w1 = std::min(words, w0 + kSegWords);
      if (w0 >= w1 || g.gids.empty()) continue;
      const int b = (int)(pass & 1);
      uint32_t* qc = h->qcounts.as<uint32_t>() + s * G + gi;
      uint32_t* q = h->queue[b].as<uint32_t>();
      if (pass >= 2) COF_CUDA(h, cudaStreamWaitEvent(h->stream2, h->ev_used[b], 0));
      // A profiled search times every launch alone: the finder also waits
      // for the previous pass's comparer, or its events would count the time
      // it spends queued behind that comparer's CTAs.
      if (h->profiling && pass >= 1) COF_CUDA(h, cudaStreamWaitEvent(h->stream2, h->ev_used[1 - b], 0));
      if (ahead) {
        // Segment s reads chunk s and the first words of chunk s + 1.
        COF_CUDA(h, cudaStreamWaitEvent(h->stream2, h->upload_ev[std::min<size_t>(s, h->upload_pending - 1)], 0));
      } else if (h->upload_pending) {
        // Segment s reads plane words up to w1 + 2 (chunks s and s + 1); its
        // finder follows the copies up to chunk s + 1 on the same stream, and
        // the copy of chunk s + 2 runs under the comparer of segment s.
        cof_status st = issue_upload(h, (size_t)s + 2);
        if (st) return st;
      }
      cof_status st = record_start(h, evs, "finder", (double)(w1 - w0) * 32, h->stream2);
      if (st) return st;
      launch_finder(gv, w0, w1, g.fpat, q, qc, h->stream2);
      if ((st = record_stop(h, evs, h->stream2))) return st;
      COF_CUDA(h, cudaEventRecord(h->ev_found[b], h->stream2));
      COF_CUDA(h, cudaStreamWaitEvent(h->stream, h->ev_found[b], 0));
      // Comparer units are filled in from qcounts after the search.
      if ((st = record_start(h, evs, "comparer", (double)(s * G + gi), h->stream))) return st;
      const uint32_t V = (uint32_t)g.gids.size();
      if (!g.bs_slots ||
          !launch_comparer_bs(gv, q, qc, w0 * 32, g.bs_prog.as<uint32_t>(), g.bs_pgid.as<uint32_t>(),
                              g.bs_chunks, g.bs_m, g.bs_slots, g.bs_narrow, g.L, g.concrete_only, qc + nq,
                              h->hits.as<uint64_t>(), h->hit_count.as<unsigned long long>(), hit_cap, h->sm_count,
                              h->stream))
        launch_comparer(gv, q, qc, w0 * 32, g.vmask.p, V, g.nw, g.L, h->hits.as<uint64_t>(),
                        h->hit_count.as<unsigned long long>(), hit_cap, h->sm_count, h->stream);
      if ((st = record_stop(h, evs, h->stream))) return st;
      COF_CUDA(h, cudaEventRecord(h->ev_used[b], h->stream));
      ++pass;
    }
  }
  // Row formatting reads the planes: the rest of a streamed upload goes
  // before the join.
  if (ahead) {
    COF_CUDA(h, cudaStreamWaitEvent(h->stream2, h->upload_ev[h->upload_pending - 1], 0));
  } else if (h->upload_pending) {
    cof_status st = issue_upload(h, h->upload_pending);
    if (st) return st;
  }
  // Join stream2 into the main stream (it may end with a finder whose
  // comparer was skipped, or with copies; normally the last comparer already
  // waited on it).
  COF_CUDA(h, cudaEventRecord(h->ev_start, h->stream2));
  COF_CUDA(h, cudaStreamWaitEvent(h->stream, h->ev_start, 0));
  COF_CUDA(h, cudaGetLastError());
  return COF_OK;
}

// Everything the captured passes depend on: buffers, sizes and each group's
// launch parameters.
std::string pass_graph_key(const cof_handle* h, uint64_t cap) {
  std::string k;
  auto put = [&](const void* p, size_t n) { k.append((const char*)p, n); };
  auto put64 = [&](uint64_t v) { put(&v, 8); };
  for (const void* p : {h->genome.hi.p, h->genome.lo.p, h->genome.ot.p, h->queue[0].p, h->queue[1].p, h->qcounts.p,
                        h->hits.p, h->hit_count.p})
    put64((uint64_t)p);
  put64(h->genome.n);
  put64(h->qcounts.cap);
  // A streamed upload's copies are part of the graph.
  put64(h->upload_pending);
  for (const uint32_t* p : h->upload_src) put64(h->upload_pending ? (uint64_t)p : 0);
  put64(h->upload_pending ? h->upload_words : 0);
  put64(cap);
  put64((uint64_t)h->sm_count);
  for (const PatternGroup& g : h->groups) {
    for (uint64_t v : {(uint64_t)g.L, (uint64_t)g.nw, (uint64_t)g.bs_slots, (uint64_t)g.bs_narrow, (uint64_t)g.bs_chunks, (uint64_t)g.bs_m,
                       (uint64_t)g.concrete_only, (uint64_t)g.gids.size()})
      put64(v);
    for (const void* p : {g.bs_prog.p, g.bs_pgid.p, g.vmask.p}) put64((uint64_t)p);
    put(&g.fpat, sizeof(g.fpat));
  }
  return k;
}

// run_passes through a CUDA graph: captured on first use (or when the key
// changes), then one cudaGraphLaunch per search.
cof_status run_passes_graph(cof_handle* h, uint64_t cap, uint64_t* nseg) {
  // Buffers run_passes would allocate must exist before capture.
  uint64_t max_words = 0;
  for (const PatternGroup& g : h->groups) {
    const uint64_t npos = h->genome.n >= g.L ? h->genome.n - g.L + 1 : 0;
    max_words = std::max(max_words, (npos + 31) / 32);
  }
  const uint64_t ns = (max_words + kSegWords - 1) / kSegWords;
  COF_CUDA(h, h->qcounts.ensure(2 * std::max<uint64_t>(ns * h->groups.size(), 1) * 4));
  const std::string key = pass_graph_key(h, cap);
  if (!h->pass_graph || key != h->pass_key) {
    if (h->pass_graph) cudaGraphExecDestroy(h->pass_graph);
    h->pass_graph = nullptr;
    std::vector<EventPair> none;
    h->upload_issued = 0;  // a streamed upload is captured whole
    if (h->upload_pending) {
      cof_status se = ensure_upload_events(h, h->upload_pending);
      if (se) return se;
    }
    COF_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    const cof_status st = run_passes(h, cap, none, nseg);
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
    if (st || e != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      return st ? st : fail(h, COF_ERR_CUDA, std::string("pass capture: ") + cudaGetErrorString(e));
    }
    const cudaError_t ei = cudaGraphInstantiate(&h->pass_graph, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) {
      h->pass_graph = nullptr;
      return fail(h, COF_ERR_CUDA, std::string("pass graph: ") + cudaGetErrorString(ei));
    }
    h->pass_key = key;
    h->pass_nseg = *nseg;
  }
  *nseg = h->pass_nseg;
  COF_CUDA(h, cudaGraphLaunch(h->pass_graph, h->stream));
  h->upload_issued = h->upload_pending;  // the graph copies every chunk
  return COF_OK;
}

// Where cof_search_stream sends the rows.
struct StreamSink {
  cof_write_fn fn;
  void* ctx;
  uint64_t written;
};

// Summary table (cas-offinder.cpp:451-454): each row of a hit counts once
// under (id, bulge type, bulge size, mismatches).  The device counts hits per
// (variant, strand, mismatches); the host spreads each count over the row
// shapes of that variant and strand.
cof_status summarise(cof_handle* h, uint64_t nhits) {
  const uint32_t G = h->job_gid0.back();
  uint32_t levels = 1;
  for (const Job& job : h->jobs)
    for (const Variant& v : job.variants) levels = std::max<uint32_t>(levels, (uint32_t)v.threshold + 1);
  levels = std::min<uint32_t>(levels, 128);
  const size_t ncount = (size_t)G * 2 * levels;
  COF_CUDA(h, h->summary_counts.ensure(ncount * 4));
  COF_CUDA(h, cudaMemsetAsync(h->summary_counts.p, 0, ncount * 4, h->stream));
  launch_hit_histogram(h->hits_sorted.as<uint64_t>(), nhits, levels, h->summary_counts.as<uint32_t>(), h->stream);
  COF_CUDA(h, cudaGetLastError());
  std::vector<uint32_t> counts(ncount);
  COF_CUDA(h, cudaMemcpyAsync(counts.data(), h->summary_counts.p, ncount * 4, cudaMemcpyDeviceToHost, h->stream));
  COF_CUDA(h, cudaStreamSynchronize(h->stream));
  size_t j = 0;
  for (uint32_t gid = 0; gid < G; ++gid) {
    while (gid >= h->job_gid0[j + 1]) ++j;
    const Variant& var = h->jobs[j].variants[gid - h->job_gid0[j]];
    for (uint32_t strand = 0; strand < 2; ++strand)
      for (uint32_t mm = 0; mm < levels; ++mm) {
        const uint32_t c = counts[((size_t)gid * 2 + strand) * levels + mm];
        if (!c) continue;
        for (const RowShape& r : h->jobs[j].shapes[strand][gid - h->job_gid0[j]]) {
          char key[10000];
          snprintf(key, sizeof key, "%s,%s,%d,%d", var.id.c_str(), r.type.c_str(), (int)r.bulge_size, (int)mm);
          h->summaries[j][key] += c;
        }
      }
  }
  return COF_OK;
}

cof_status do_search(cof_handle* h, const char** rows, size_t* rows_len, StreamSink* sink = nullptr) {
  if (h->jobs.empty()) return fail(h, COF_ERR_STATE, "no input file has been read");
  if (!h->genome.loaded) return fail(h, COF_ERR_STATE, "no genome is loaded");
  cof_status st = upload_jobs(h);
  if (st) return st;
  const size_t J = h->jobs.size();
  *rows = "";
  *rows_len = 0;
  h->last_hits = h->last_rows = 0;
  h->job_byte0.assign(J + 1, 0);
  if (h->summaries.size() != J) h->summaries.assign(J, {});
  if (h->job_gid0.back() == 0) return COF_OK;
  COF_CUDA(h, h->queue[0].ensure(2 * kSegPositions * 4));
  COF_CUDA(h, h->queue[1].ensure(2 * kSegPositions * 4));
  COF_CUDA(h, h->hit_count.ensure(8));
  uint64_t cap = std::max<uint64_t>(h->hits.cap / 8, 1u << 20);
  COF_CUDA(h, h->hits.ensure(cap * 8));
  std::vector<EventPair> evs;
  uint64_t nseg = 0, nhits = 0;
  // Profiled searches time each launch with events, and copies from pageable
  // host memory cannot be graph nodes: both run the passes directly.
  const bool graph = h->use_graphs && !h->profiling && (!h->upload_pending || h->upload_pinned);
  if (h->upload_pending && (st = ensure_upload_events(h, h->upload_pending))) return st;
  for (;;) {
    st = graph ? run_passes_graph(h, cap, &nseg) : run_passes(h, cap, evs, &nseg);
    if (st) return st;
    COF_CUDA(h, cudaMemcpyAsync(&nhits, h->hit_count.p, 8, cudaMemcpyDeviceToHost, h->stream));
    COF_CUDA(h, cudaStreamSynchronize(h->stream));
    if (nhits <= cap) break;
    for (EventPair& p : evs) {  // discard the overflowing pass's timings
      h->event_pool.push_back(p.a);
      h->event_pool.push_back(p.b);
    }
    evs.clear();
    cap = nhits + nhits / 8;
    COF_CUDA(h, h->hits.ensure(cap * 8));
  }
  if (h->profiling) {
    // Comparer units: base comparisons = oriented candidates x non-N positions
    // of each variant; variant tests go to "comparer.tests".
    const size_t G = h->groups.size();
    std::vector<uint32_t> qc(std::max<uint64_t>(nseg * G, 1), 0);
    COF_CUDA(h, cudaMemcpy(qc.data(), h->qcounts.p, nseg * G * 4, cudaMemcpyDeviceToHost));
    for (EventPair& p : evs)
      if (p.name == "comparer") {
        const size_t idx = (size_t)p.units;
        const PatternGroup& g = h->groups[idx % G];
        p.units = (double)qc[idx] * g.nonN_sum;
        h->stats["comparer.tests"].units += (double)qc[idx] * (double)g.gids.size();
        if (g.bs_slots && g.bs_chunks)  // lane LOP3 ops the bit-sliced count issues (op model)
          h->stats["comparer.lop3"].units +=
              (double)((qc[idx] + 63) / 64) * 32.0 * g.bs_chunks * bs_lane_lop3(g.bs_slots, g.bs_m, g.bs_narrow);
        h->stats["finder.candidates"].units += (double)qc[idx];  // queue entries the finder wrote
      }
    collect(h, evs);
  }
  h->last_hits = nhits;
  if (nhits == 0) return COF_OK;
  // Sort hit keys into output order.
  COF_CUDA(h, h->hits_sorted.ensure(nhits * 8));
  COF_CUDA(h, h->row_bytes.ensure(nhits * 8));
  COF_CUDA(h, h->row_offsets.ensure(nhits * 8));
  COF_CUDA(h, h->row_count.ensure(nhits * 4));
  COF_CUDA(h, h->small.ensure(64));
  COF_CUDA(h, h->job_start.ensure((J + 1) * 4));
  COF_CUDA(h, h->job_bytes.ensure((J + 1) * 8));
  // Key bits the order depends on: strand (bit 7), position, variant id up to
  // the largest id in use.  The mismatch bits below never break a tie: a
  // (variant, position, strand) has one hit at most.
  int end_bit = 44;
  for (uint64_t v = h->job_gid0.empty() ? 1 : std::max<uint64_t>(h->job_gid0.back(), 2) - 1; v; v >>= 1) ++end_bit;
  end_bit = std::min(end_bit, 64);
  size_t tmp = 0;
  COF_CUDA(h, cub::DeviceRadixSort::SortKeys(nullptr, tmp, h->hits.as<uint64_t>(), h->hits_sorted.as<uint64_t>(),
                                             (int64_t)nhits, 7, end_bit, h->stream));
  size_t tmp2 = 0;
  COF_CUDA(h, cub::DeviceScan::ExclusiveSum(nullptr, tmp2, h->row_bytes.as<uint64_t>(), h->row_offsets.as<uint64_t>(),
                                            (int64_t)nhits, h->stream));
  size_t tmp3 = 0;
  COF_CUDA(h, cub::DeviceReduce::Sum(nullptr, tmp3, h->row_count.as<uint32_t>(), h->small.as<uint64_t>(),
                                     (int64_t)nhits, h->stream));
  COF_CUDA(h, h->sort_tmp.ensure(std::max(tmp, std::max(tmp2, tmp3))));
  tmp = h->sort_tmp.cap;
  if ((st = record_start(h, evs, "sort", (double)nhits, h->stream))) return st;
  COF_CUDA(h, cub::DeviceRadixSort::SortKeys(h->sort_tmp.p, tmp, h->hits.as<uint64_t>(), h->hits_sorted.as<uint64_t>(),
                                             (int64_t)nhits, 7, end_bit, h->stream));
  if ((st = record_stop(h, evs, h->stream))) return st;
  // Row sizes, offsets, per-job byte ranges, then the rows themselves.
  const GenomeView gv = h->genome.view();
  FormatTables ft{h->vfmt.as<VariantFmt>(), h->sfmt.as<ShapeFmt>(), h->pool.as<char>()};
  if ((st = record_start(h, evs, "format", (double)nhits, h->stream))) return st;
  launch_row_lengths(gv, ft, h->hits_sorted.as<uint64_t>(), nhits, h->row_bytes.as<uint64_t>(),
                     h->row_count.as<uint32_t>(), h->stream);
  tmp = h->sort_tmp.cap;
  COF_CUDA(h, cub::DeviceScan::ExclusiveSum(h->sort_tmp.p, tmp, h->row_bytes.as<uint64_t>(),
                                            h->row_offsets.as<uint64_t>(), (int64_t)nhits, h->stream));
  tmp = h->sort_tmp.cap;
  COF_CUDA(h, cub::DeviceReduce::Sum(h->sort_tmp.p, tmp, h->row_count.as<uint32_t>(), h->small.as<uint64_t>(),
                                     (int64_t)nhits, h->stream));
  COF_CUDA(h, cudaMemcpyAsync(h->job_start.p, h->job_gid0.data(), (J + 1) * 4, cudaMemcpyHostToDevice, h->stream));
  launch_job_bounds(h->hits_sorted.as<uint64_t>(), nhits, h->job_start.as<uint32_t>(), (uint32_t)J,
                    h->row_offsets.as<uint64_t>(), h->row_bytes.as<uint64_t>(), h->job_bytes.as<uint64_t>(),
                    h->stream);
  COF_CUDA(h, cudaMemcpyAsync(h->job_byte0.data(), h->job_bytes.p, (J + 1) * 8, cudaMemcpyDeviceToHost, h->stream));
  uint64_t nrows = 0;
  COF_CUDA(h, cudaMemcpyAsync(&nrows, h->small.p, 8, cudaMemcpyDeviceToHost, h->stream));
  // Rows returned in one buffer are written in about kRowChunks chunks of
  // hits, each a whole number of waves of the row writer (a chunk's launch
  // lasts as long as its last wave); each chunk's first byte offset comes
  // back with this sync.
  constexpr uint64_t kRowChunks = 8, kMinChunkHits = 1u << 16;
  const uint64_t wave = write_rows_wave_hits(h->sm_count);
  const uint64_t chunk_hits = std::max<uint64_t>(
      kMinChunkHits, ((nhits + kRowChunks - 1) / kRowChunks + wave - 1) / wave * wave);
  const uint64_t nck = sink ? 0 : (nhits + chunk_hits - 1) / chunk_hits;
  if (h->profiling) h->stats["rows.chunks"].units += (double)nck;  // row-writing launches
  std::vector<uint64_t> ck(nck + 1, 0);
  if (nck > 1)
    COF_CUDA(h, cudaMemcpy2DAsync(ck.data(), 8, h->row_offsets.as<uint64_t>(), chunk_hits * 8, 8, nck,
                                  cudaMemcpyDeviceToHost, h->stream));
  COF_CUDA(h, cudaStreamSynchronize(h->stream));
  const uint64_t bytes = h->job_byte0[J];
  // Rows are short; a size out of proportion means corrupted tables or keys.
  for (size_t j = 0; j < J; ++j)
    if (h->job_byte0[j] > h->job_byte0[j + 1])
      return fail(h, COF_ERR_DEVICE, "job row ranges out of order at job " + std::to_string(j));
  if (bytes > (nrows + 1) * (uint64_t)(1 << 20))
    return fail(h, COF_ERR_DEVICE, "row text of " + std::to_string(bytes) + " bytes for " + std::to_string(nrows) +
                                       " rows (" + std::to_string(nhits) + " hits)");
  if (!sink) {
    // Chunk k's rows are copied to the host on the second stream (idle once
    // the passes have joined) while chunk k + 1 is written.
    COF_CUDA(h, h->text.ensure(bytes + 1));
    COF_CUDA(h, h->host_text.ensure(bytes + 1));
    if (!h->stream_ev[0]) COF_CUDA(h, cudaEventCreateWithFlags(&h->stream_ev[0], cudaEventDisableTiming));
    ck[0] = 0;
    ck[nck] = bytes;
    // Profiled searches also time the row copies to the host (second stream).
    cudaEvent_t copy_ev[2] = {nullptr, nullptr};
    if (h->profiling)
      for (cudaEvent_t& e : copy_ev) COF_CUDA(h, cudaEventCreate(&e));
    for (uint64_t k = 0; k < nck; ++k) {
      const uint64_t i0 = k * chunk_hits, i1 = std::min(nhits, i0 + chunk_hits);
      launch_write_rows(gv, ft, h->hits_sorted.as<uint64_t>() + i0, i1 - i0, h->row_offsets.as<uint64_t>() + i0, 0,
                        ck[k + 1], h->text.as<char>(), h->stream);
      COF_CUDA(h, cudaEventRecord(h->stream_ev[0], h->stream));
      COF_CUDA(h, cudaStreamWaitEvent(h->stream2, h->stream_ev[0], 0));
      if (k == 0 && copy_ev[0]) COF_CUDA(h, cudaEventRecord(copy_ev[0], h->stream2));
      if (ck[k + 1] > ck[k])
        COF_CUDA(h, cudaMemcpyAsync((char*)h->host_text.p + ck[k], h->text.as<char>() + ck[k], ck[k + 1] - ck[k],
                                    cudaMemcpyDeviceToHost, h->stream2));
    }
    if (copy_ev[1]) COF_CUDA(h, cudaEventRecord(copy_ev[1], h->stream2));
    if ((st = record_stop(h, evs, h->stream))) return st;
    COF_CUDA(h, cudaGetLastError());
    COF_CUDA(h, cudaStreamSynchronize(h->stream2));
    COF_CUDA(h, cudaStreamSynchronize(h->stream));
    ((char*)h->host_text.p)[bytes] = 0;
    if (copy_ev[0]) {
      // From the first chunk's copy becoming ready to the last copy's end.
      float ms = 0;
      if (nck && cudaEventElapsedTime(&ms, copy_ev[0], copy_ev[1]) == cudaSuccess) {
        KernelStat& ks = h->stats["rows_to_host"];
        ks.launches += 1;
        ks.ms += ms;
        ks.units += (double)bytes;
      }
      for (cudaEvent_t e : copy_ev) cudaEventDestroy(e);
    }
  } else {
    // Rows in chunks of kBatch hits: chunk k+1 is formatted and copied while
    // the caller writes chunk k (two device and two pinned host buffers).
    if ((st = record_stop(h, evs, h->stream))) return st;
    constexpr uint64_t kBatch = 1ull << 20;
    const uint64_t nb = (nhits + kBatch - 1) / kBatch;
    std::vector<uint64_t> cut(nb + 1, 0);
    for (uint64_t k = 0; k < nb; ++k)
      COF_CUDA(h, cudaMemcpyAsync(&cut[k], h->row_offsets.as<uint64_t>() + k * kBatch, 8, cudaMemcpyDeviceToHost,
                                  h->stream));
    COF_CUDA(h, cudaStreamSynchronize(h->stream));
    cut[nb] = bytes;
    uint64_t most = 0;
    for (uint64_t k = 0; k < nb; ++k) most = std::max(most, cut[k + 1] - cut[k]);
    for (int b = 0; b < 2; ++b) {
      COF_CUDA(h, h->stream_dev[b].ensure(most + 16));
      COF_CUDA(h, h->stream_host[b].ensure(most + 16));
      if (!h->stream_ev[b]) COF_CUDA(h, cudaEventCreateWithFlags(&h->stream_ev[b], cudaEventDisableTiming));
    }
    for (uint64_t k = 0; k <= nb; ++k) {
      if (k < nb) {
        const int b = (int)(k & 1);
        const uint64_t i0 = k * kBatch, i1 = std::min(nhits, i0 + kBatch);
        launch_write_rows(gv, ft, h->hits_sorted.as<uint64_t>() + i0, i1 - i0, h->row_offsets.as<uint64_t>() + i0,
                          cut[k], cut[k + 1], h->stream_dev[b].as<char>(), h->stream);
        COF_CUDA(h, cudaGetLastError());
        COF_CUDA(h, cudaMemcpyAsync(h->stream_host[b].p, h->stream_dev[b].p, cut[k + 1] - cut[k],
                                    cudaMemcpyDeviceToHost, h->stream));
        COF_CUDA(h, cudaEventRecord(h->stream_ev[b], h->stream));
      }
      if (k >= 1) {
        const int pb = (int)((k - 1) & 1);
        const uint64_t len = cut[k] - cut[k - 1];
        COF_CUDA(h, cudaEventSynchronize(h->stream_ev[pb]));
        if (len && sink->fn(sink->ctx, (const char*)h->stream_host[pb].p, len) != 0) {
          cudaStreamSynchronize(h->stream);
          return fail(h, COF_ERR_IO, "the row writer failed after " + std::to_string(sink->written) + " bytes");
        }
        sink->written += len;
      }
    }
  }
  collect(h, evs);
  h->last_rows = nrows;
  if (h->summary_on && (st = summarise(h, nhits))) return st;
  if (!sink) {
    *rows = (const char*)h->host_text.p;
    *rows_len = bytes;
  }
  return COF_OK;
}

std::string summary_of(const std::map<std::string, unsigned long long>& table) {
  static const char* kHead[4] = {"Id", "Bulge Type", "Bulge Size", "Mismatches"};
  std::string out;
  for (const auto& kv : table) {
    std::string key = kv.first;
    out += "##";
    size_t cut;
    int col = 0;
    while ((cut = key.find(',')) != std::string::npos && col < 3) {
      out += std::string(kHead[col++]) + "=" + key.substr(0, cut) + ";";
      key.erase(0, cut + 1);
    }
    out += std::string(kHead[col]) + "=" + key + ";";
    out += "Number of Found Targets=" + std::to_string(kv.second) + "\n";
  }
  return out;
}

}  // namespace

extern "C" {

const char* cof_open_error(void) {
  std::lock_guard<std::mutex> g(g_open_mu);
  return g_open_err.c_str();
}

cof_status cof_open(int device, cof_handle** out) {
  if (!out) return COF_ERR_ARG;
  *out = nullptr;
  auto set_err = [](const std::string& m) {
    std::lock_guard<std::mutex> g(g_open_mu);
    g_open_err = m;
  };
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    set_err(std::string("no CUDA device: ") + cudaGetErrorString(e));
    return COF_ERR_CUDA;
  }
  if (device < 0 || device >= count) {
    set_err("device ordinal out of range");
    return COF_ERR_ARG;
  }
  if ((e = cudaSetDevice(device)) != cudaSuccess) {
    set_err(std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    return COF_ERR_CUDA;
  }
  cof_handle* h = new cof_handle();
  h->device = device;
  cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, device);
  e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream2, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream3, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_start, cudaEventDisableTiming);
  for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
    e = cudaEventCreateWithFlags(&h->ev_found[i], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_used[i], cudaEventDisableTiming);
  }
  if (e != cudaSuccess) {
    set_err(std::string("stream/event creation: ") + cudaGetErrorString(e));
    cof_close(h);
    return COF_ERR_CUDA;
  }
  *out = h;
  return COF_OK;
}

void cof_close(cof_handle* h) {
  if (!h) return;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->stream2) cudaStreamSynchronize(h->stream2);
  if (h->stream3) cudaStreamSynchronize(h->stream3);
  cudaStream_t s = h->stream, s2 = h->stream2, s3 = h->stream3;
  for (cudaEvent_t e : h->upload_ev) cudaEventDestroy(e);
  cudaEvent_t evs[7] = {h->timer_a, h->timer_b, h->ev_start, h->ev_found[0], h->ev_found[1], h->ev_used[0],
                        h->ev_used[1]};
  for (cudaEvent_t e : h->event_pool) cudaEventDestroy(e);
  if (h->pass_graph) cudaGraphExecDestroy(h->pass_graph);
  for (cudaEvent_t e : h->stream_ev)
    if (e) cudaEventDestroy(e);
  for (auto& kv : h->pinned_free) cudaFreeHost(kv.second);
  delete h;  // frees device buffers
  for (cudaEvent_t ev : evs)
    if (ev) cudaEventDestroy(ev);
  if (s) cudaStreamDestroy(s);
  if (s2) cudaStreamDestroy(s2);
  if (s3) cudaStreamDestroy(s3);
}

const char* cof_last_error(const cof_handle* h) { return h ? h->err.c_str() : "null handle"; }

cof_status cof_read_input(cof_handle* h, const char* text, size_t len) {
  if (!h || (!text && len)) return COF_ERR_ARG;
  h->err.clear();
  Job job;
  std::string err;
  if (!parse_job(text ? text : "", len, job, err)) return fail(h, COF_ERR_INPUT, err);
  if (!build_shapes(job, err)) return fail(h, COF_ERR_INPUT, err);
  h->jobs.clear();
  h->jobs.push_back(std::move(job));
  h->jobs_on_device = false;
  h->summaries.assign(1, {});
  h->job_byte0.clear();
  return COF_OK;
}

cof_status cof_batch_clear(cof_handle* h) {
  if (!h) return COF_ERR_ARG;
  h->jobs.clear();
  h->summaries.clear();
  h->job_byte0.clear();
  h->jobs_on_device = false;
  return COF_OK;
}

cof_status cof_batch_add_input(cof_handle* h, const char* text, size_t len, uint32_t* job_index) {
  if (!h || (!text && len)) return COF_ERR_ARG;
  h->err.clear();
  Job job;
  std::string err;
  if (!parse_job(text ? text : "", len, job, err)) return fail(h, COF_ERR_INPUT, err);
  if (!build_shapes(job, err)) return fail(h, COF_ERR_INPUT, err);
  if (job_index) *job_index = (uint32_t)h->jobs.size();
  h->jobs.push_back(std::move(job));
  h->summaries.emplace_back();
  h->job_byte0.clear();
  h->jobs_on_device = false;
  return COF_OK;
}

cof_status cof_batch_size(const cof_handle* h, uint32_t* n_jobs) {
  if (!h || !n_jobs) return COF_ERR_ARG;
  *n_jobs = (uint32_t)h->jobs.size();
  return COF_OK;
}

cof_status cof_job_rows(const cof_handle* h, uint32_t job, const char** rows, size_t* rows_len) {
  if (!h || !rows || !rows_len) return COF_ERR_ARG;
  if (job >= h->jobs.size() || h->job_byte0.size() != h->jobs.size() + 1) return COF_ERR_STATE;
  *rows = h->host_text.p ? (const char*)h->host_text.p + h->job_byte0[job] : "";
  *rows_len = h->job_byte0[job + 1] - h->job_byte0[job];
  return COF_OK;
}

const char* cof_genome_path(const cof_handle* h) {
  return (h && !h->jobs.empty()) ? h->jobs[0].genome_path.c_str() : "";
}

cof_status cof_input_info(const cof_handle* h, uint32_t* pattern_len, uint32_t* n_variants, uint32_t* n_bulge_records) {
  if (!h) return COF_ERR_ARG;
  if (h->jobs.empty()) return COF_ERR_STATE;
  if (pattern_len) *pattern_len = (uint32_t)h->jobs[0].pattern.size();
  uint32_t nv = 0, nb = 0;
  for (const Job& j : h->jobs) {
    nv += (uint32_t)j.variants.size();
    for (const Variant& v : j.variants) nb += (uint32_t)v.bulges.size();
  }
  if (n_variants) *n_variants = nv;
  if (n_bulge_records) *n_bulge_records = nb;
  return COF_OK;
}

cof_status cof_genome_load_file(cof_handle* h, const char* path) {
  if (!h || !path) return COF_ERR_ARG;
  h->err.clear();
  cudaSetDevice(h->device);
  PackedGenome g;
  if (load_fasta(path, g) != 0) {
    g = PackedGenome();
    if (load_twobit(path, g) != 0) return fail(h, COF_ERR_NOT_GENOME, std::string("Skipping non-acceptable file ") + path);
  }
  return upload_packed(h, h->genome, g);
}

cof_status cof_genome_load_text(cof_handle* h, const char* seq, uint64_t n, const char* const* names,
                                const uint64_t* starts, uint32_t n_records) {
  if (!h || (!seq && n) || (n_records && (!names || !starts))) return COF_ERR_ARG;
  h->err.clear();
  cudaSetDevice(h->device);
  PackedGenome g;
  g.n = n;
  const uint64_t W = plane_words(n);
  g.hi.assign(W, 0);
  g.lo.assign(W, 0);
  g.ot.assign(W, 0);
  pack_text(seq, n, g.hi.data(), g.lo.data(), g.ot.data(), &g.exc_pos, &g.exc_byte);
  for (uint32_t i = 0; i < n_records; ++i) {
    g.names.push_back(names[i] ? names[i] : "");
    g.starts.push_back(starts[i]);
  }
  return upload_packed(h, h->genome, g);
}

cof_status cof_genome_load_planes(cof_handle* h, const uint32_t* hi, const uint32_t* lo, const uint32_t* ot,
                                  uint64_t n, const uint64_t* exc_pos, const uint8_t* exc_byte, uint64_t n_exc,
                                  const char* const* names, const uint64_t* starts, uint32_t n_records) {
  if (!h || !hi || !lo || !ot || (n_exc && (!exc_pos || !exc_byte)) || (n_records && (!names || !starts)))
    return COF_ERR_ARG;
  h->err.clear();
  cudaSetDevice(h->device);
  std::vector<std::string> nm;
  std::vector<uint64_t> st;
  for (uint32_t i = 0; i < n_records; ++i) {
    nm.push_back(names[i] ? names[i] : "");
    st.push_back(starts[i]);
  }
  return upload_genome(h, h->genome, hi, lo, ot, n, exc_pos, exc_byte, n_exc, nm, st);
}

cof_status cof_genome_info(const cof_handle* h, uint64_t* n, uint32_t* n_records) {
  if (!h) return COF_ERR_ARG;
  if (!h->genome.loaded) return COF_ERR_STATE;
  if (n) *n = h->genome.n;
  if (n_records) *n_records = h->genome.n_rec;
  return COF_OK;
}

cof_status cof_search(cof_handle* h, const char** rows, size_t* rows_len) {
  if (!h || !rows || !rows_len) return COF_ERR_ARG;
  h->err.clear();
  cudaSetDevice(h->device);
  return do_search(h, rows, rows_len);
}

cof_status cof_search_stream(cof_handle* h, cof_write_fn write, void* ctx, uint64_t* bytes_written) {
  if (!h || !write) return COF_ERR_ARG;
  h->err.clear();
  cudaSetDevice(h->device);
  StreamSink sink{write, ctx, 0};
  const char* rows = "";
  size_t len = 0;
  const cof_status st = do_search(h, &rows, &len, &sink);
  if (bytes_written) *bytes_written = sink.written;
  return st;
}

cof_status cof_search_planes(cof_handle* h, const uint32_t* hi, const uint32_t* lo, const uint32_t* ot, uint64_t n,
                             const uint64_t* exc_pos, const uint8_t* exc_byte, uint64_t n_exc,
                             const char* const* names, const uint64_t* starts, uint32_t n_records,
                             const char** rows, size_t* rows_len) {
  if (!h || !hi || !lo || !ot || (n_exc && (!exc_pos || !exc_byte)) || (n_records && (!names || !starts)) || !rows ||
      !rows_len)
    return COF_ERR_ARG;
  h->err.clear();
  cudaSetDevice(h->device);
  std::vector<std::string> nm;
  std::vector<uint64_t> st;
  for (uint32_t i = 0; i < n_records; ++i) {
    nm.push_back(names[i] ? names[i] : "");
    st.push_back(starts[i]);
  }
  cof_status r = upload_genome(h, h->genome, hi, lo, ot, n, exc_pos, exc_byte, n_exc, nm, st, true);
  h->upload_pinned = true;
  for (const uint32_t* p : {hi, lo, ot}) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess || a.type != cudaMemoryTypeHost) h->upload_pinned = false;
  }
  cudaGetLastError();  // an unregistered pointer is not an error here
  if (r == COF_OK) r = do_search(h, rows, rows_len);
  // The whole genome stays resident (also when the search stopped early) and
  // the host planes are not read after this call returns.
  if (h->upload_pending) {
    const cof_status ri = issue_upload(h, h->upload_pending);
    cudaError_t e = cudaStreamSynchronize(h->stream3);
    const cudaError_t e2 = cudaStreamSynchronize(h->stream2);
    if (e == cudaSuccess) e = e2;
    h->upload_pending = h->upload_issued = 0;
    if (ri && r == COF_OK) return ri;
    if (e != cudaSuccess && r == COF_OK) return fail(h, COF_ERR_CUDA, cudaGetErrorString(e));
  }
  return r;
}

cof_status cof_last_hit_count(const cof_handle* h, uint64_t* n_hits, uint64_t* n_rows) {
  if (!h) return COF_ERR_ARG;
  if (n_hits) *n_hits = h->last_hits;
  if (n_rows) *n_rows = h->last_rows;
  return COF_OK;
}

cof_status cof_set_summary(cof_handle* h, int enable) {
  if (!h) return COF_ERR_ARG;
  h->summary_on = enable != 0;
  return COF_OK;
}

cof_status cof_summary_text(cof_handle* h, const char** text, size_t* len) {
  return cof_job_summary_text(h, 0, text, len);
}

cof_status cof_job_summary_text(cof_handle* h, uint32_t job, const char** text, size_t* len) {
  if (!h || !text || !len) return COF_ERR_ARG;
  h->summary_text = job < h->summaries.size() ? summary_of(h->summaries[job]) : std::string();
  *text = h->summary_text.c_str();
  *len = h->summary_text.size();
  return COF_OK;
}

const char* cof_header_text(void) {
  return "##Generated by Cas-OFFinder 3.0.0\n"
         "#Id\tBulge Type\tcrRNA\tDNA\tChromosome\tLocation\tDirection\tMismatches\tBulge Size\n";
}

cof_status cof_finder_chunk(cof_handle* h, const char* chr, uint64_t worksize, const char* pat, uint32_t patternlen,
                            uint32_t* loci, uint8_t* flag, uint32_t* entrycount) {
  if (!h || !chr || !pat || !loci || !flag || !entrycount || patternlen == 0) return COF_ERR_ARG;
  if (patternlen > (uint32_t)kMaxL) return fail(h, COF_ERR_UNSUPPORTED, "pattern too long");
  if (worksize >= (1ull << 31)) return fail(h, COF_ERR_ARG, "worksize must be below 2^31");
  h->err.clear();
  cudaSetDevice(h->device);
  *entrycount = 0;
  if (worksize == 0) return COF_OK;
  const uint64_t n = worksize + patternlen - 1;
  PackedGenome g;
  g.n = n;
  g.hi.assign(plane_words(n), 0);
  g.lo.assign(plane_words(n), 0);
  g.ot.assign(plane_words(n), 0);
  pack_text(chr, n, g.hi.data(), g.lo.data(), g.ot.data(), &g.exc_pos, &g.exc_byte);
  g.names.push_back("chunk");
  g.starts.push_back(0);
  cof_status st = upload_packed(h, h->scratch, g);
  if (st) return st;
  FinderPattern fp;
  make_finder_pattern(std::string(pat, patternlen), std::string(pat + patternlen, patternlen), fp);
  const uint64_t words = (worksize + 31) / 32;
  DevBuf q, qc;
  COF_CUDA(h, q.ensure(words * 64 * 4));
  COF_CUDA(h, qc.ensure(4));
  COF_CUDA(h, cudaMemsetAsync(qc.p, 0, 4, h->stream));
  launch_finder(h->scratch.view(), 0, words, fp, q.as<uint32_t>(), qc.as<uint32_t>(), h->stream);
  COF_CUDA(h, cudaGetLastError());
  uint32_t cnt = 0;
  COF_CUDA(h, cudaMemcpyAsync(&cnt, qc.p, 4, cudaMemcpyDeviceToHost, h->stream));
  COF_CUDA(h, cudaStreamSynchronize(h->stream));
  std::vector<uint32_t> e(cnt);
  if (cnt) COF_CUDA(h, cudaMemcpy(e.data(), q.p, (size_t)cnt * 4, cudaMemcpyDeviceToHost));
  std::sort(e.begin(), e.end());
  uint32_t out = 0;
  for (size_t i = 0; i < e.size();) {
    const uint32_t pos = e[i] >> 1;
    bool f = false, r = false;
    while (i < e.size() && (e[i] >> 1) == pos) {
      if (e[i] & 1) r = true;
      else f = true;
      ++i;
    }
    if (pos >= worksize) continue;
    loci[out] = pos;
    flag[out] = (f && r) ? 0 : (f ? 1 : 2);
    ++out;
  }
  *entrycount = out;
  return COF_OK;
}

cof_status cof_comparer_chunk(cof_handle* h, const char* chr, uint64_t chrlen, const uint32_t* loci,
                              const uint8_t* flag, uint32_t locicnt, const char* comp, uint32_t patternlen,
                              uint16_t threshold, uint32_t* mm_loci, uint16_t* mm_count, char* direction,
                              uint32_t* entrycount) {
  if (!h || !chr || (locicnt && (!loci || !flag)) || !comp || !mm_loci || !mm_count || !direction || !entrycount ||
      patternlen == 0)
    return COF_ERR_ARG;
  if (patternlen > (uint32_t)kMaxL) return fail(h, COF_ERR_UNSUPPORTED, "pattern too long");
  if (chrlen >= (1ull << 31)) return fail(h, COF_ERR_ARG, "chunk must be below 2^31 bytes");
  h->err.clear();
  cudaSetDevice(h->device);
  *entrycount = 0;
  std::vector<uint32_t> entries;
  for (uint32_t i = 0; i < locicnt; ++i) {
    if ((uint64_t)loci[i] + patternlen > chrlen) return fail(h, COF_ERR_ARG, "candidate window beyond the chunk");
    if (flag[i] == 0 || flag[i] == 1) entries.push_back(loci[i] << 1);
    if (flag[i] == 0 || flag[i] == 2) entries.push_back((loci[i] << 1) | 1u);
  }
  if (entries.empty()) return COF_OK;
  PackedGenome g;
  g.n = chrlen;
  g.hi.assign(plane_words(chrlen), 0);
  g.lo.assign(plane_words(chrlen), 0);
  g.ot.assign(plane_words(chrlen), 0);
  pack_text(chr, chrlen, g.hi.data(), g.lo.data(), g.ot.data(), &g.exc_pos, &g.exc_byte);
  g.names.push_back("chunk");
  g.starts.push_back(0);
  cof_status st = upload_packed(h, h->scratch, g);
  if (st) return st;
  const int nw = patternlen <= 32 ? 1 : 2;
  std::vector<unsigned char> vm(nw == 1 ? sizeof(VariantMask<1>) : sizeof(VariantMask<2>));
  const std::string cs(comp, patternlen);
  if (nw == 1) fill_mask<1>(*(VariantMask<1>*)vm.data(), cs, threshold, 0);
  else fill_mask<2>(*(VariantMask<2>*)vm.data(), cs, threshold, 0);
  DevBuf q, qc, vmd, hb, hc;
  const uint64_t cap = entries.size();
  COF_CUDA(h, q.ensure(entries.size() * 4));
  COF_CUDA(h, qc.ensure(4));
  COF_CUDA(h, vmd.ensure(vm.size()));
  COF_CUDA(h, hb.ensure(cap * 8));
  COF_CUDA(h, hc.ensure(8));
  const uint32_t ne = (uint32_t)entries.size();
  COF_CUDA(h, cudaMemcpyAsync(q.p, entries.data(), entries.size() * 4, cudaMemcpyHostToDevice, h->stream));
  COF_CUDA(h, cudaMemcpyAsync(qc.p, &ne, 4, cudaMemcpyHostToDevice, h->stream));
  COF_CUDA(h, cudaMemcpyAsync(vmd.p, vm.data(), vm.size(), cudaMemcpyHostToDevice, h->stream));
  COF_CUDA(h, cudaMemsetAsync(hc.p, 0, 8, h->stream));
  launch_comparer(h->scratch.view(), q.as<uint32_t>(), qc.as<uint32_t>(), 0, vmd.p, 1, nw, patternlen,
                  hb.as<uint64_t>(), hc.as<unsigned long long>(), cap, h->sm_count, h->stream);
  COF_CUDA(h, cudaGetLastError());
  uint64_t nh = 0;
  COF_CUDA(h, cudaMemcpyAsync(&nh, hc.p, 8, cudaMemcpyDeviceToHost, h->stream));
  COF_CUDA(h, cudaStreamSynchronize(h->stream));
  std::vector<uint64_t> keys(nh);
  if (nh) COF_CUDA(h, cudaMemcpy(keys.data(), hb.p, nh * 8, cudaMemcpyDeviceToHost));
  std::sort(keys.begin(), keys.end());
  for (uint64_t i = 0; i < nh; ++i) {
    mm_loci[i] = (uint32_t)((keys[i] >> kHitPosShift) & kHitPosMask);
    mm_count[i] = (uint16_t)(keys[i] & 0x7F);
    direction[i] = ((keys[i] >> 7) & 1) ? '-' : '+';
  }
  *entrycount = (uint32_t)nh;
  return COF_OK;
}

uint64_t cof_plane_words(uint64_t n) { return plane_words(n); }

int cofx_bs_programs(const char* input, size_t len, uint32_t* info, uint32_t* prog, size_t prog_cap, uint32_t* pgid,
                     size_t pgid_cap, char* keys, size_t keys_cap) {
  Job job;
  std::string err;
  if (!input || !info || !parse_job(input, len, job, err)) return 1;
  std::vector<const Variant*> vars;
  std::vector<uint32_t> gids;
  int maxpos = 0;
  std::vector<uint32_t> thr, npos;
  for (size_t v = 0; v < job.variants.size(); ++v) {
    vars.push_back(&job.variants[v]);
    gids.push_back((uint32_t)v);
    int c = 0;
    for (char ch : job.variants[v].key) c += bs_class_of((unsigned char)ch) != 0;
    maxpos = std::max(maxpos, c);
    thr.push_back(job.variants[v].threshold);
    npos.push_back((uint32_t)c);
  }
  const int S = bs_slots_for(maxpos);
  if (!S || vars.empty()) return 2;
  const uint32_t row = (uint32_t)bs_row_for((uint32_t)job.pattern.size());
  std::vector<uint32_t> pv, gv;
  uint32_t chunks = 0, m = 1;
  build_bs_programs(vars, gids, S, row, pv, gv, chunks, m, 0, nullptr);
  std::string kt;
  for (const Variant& v : job.variants) kt += v.key + "\t" + std::to_string(v.threshold) + "\n";
  info[0] = chunks;
  info[1] = m;
  info[2] = (uint32_t)S;
  info[3] = row;
  info[4] = (uint32_t)vars.size();
  info[5] = (uint32_t)kt.size();
  info[6] = bs_narrow_ok(S, thr.data(), npos.data(), thr.size()) ? 1u : 0u;
  if (prog && prog_cap >= pv.size()) std::memcpy(prog, pv.data(), pv.size() * 4);
  if (pgid && pgid_cap >= gv.size()) std::memcpy(pgid, gv.data(), gv.size() * 4);
  if (keys && keys_cap >= kt.size()) std::memcpy(keys, kt.data(), kt.size());
  return 0;
}

void cofx_mismatch_table(uint8_t* out) {
  if (!out) return;
  for (int p = 0; p < 256; ++p)
    for (int g = 0; g < 256; ++g) {
      const int cls = g == 'T' ? 0 : g == 'C' ? 1 : g == 'A' ? 2 : g == 'G' ? 3 : 4;
      out[p * 256 + g] = (uint8_t)((class_bits_of((unsigned char)p) >> cls) & 1u);
    }
}

uint64_t cof_pack_text(const char* seq, uint64_t n, uint32_t* hi, uint32_t* lo, uint32_t* ot, uint64_t* exc_pos,
                       uint8_t* exc_byte) {
  std::vector<uint64_t> ep;
  std::vector<uint8_t> eb;
  if (hi && lo && ot) {
    pack_text(seq, n, hi, lo, ot, &ep, &eb);
  } else {
    std::vector<uint32_t> a(plane_words(n)), b(plane_words(n)), c(plane_words(n));
    pack_text(seq, n, a.data(), b.data(), c.data(), &ep, &eb);
  }
  if (exc_pos && exc_byte) {
    std::copy(ep.begin(), ep.end(), exc_pos);
    std::copy(eb.begin(), eb.end(), exc_byte);
  }
  return ep.size();
}

cof_status cof_set_comparer(cof_handle* h, int kind) {
  if (!h || kind < 0 || kind > 2) return COF_ERR_ARG;
  h->force_popc = kind == 1;
  h->jobs_on_device = false;  // rebuild the comparer tables on the next search
  return COF_OK;
}

cof_status cof_set_autotune(cof_handle* h, int enable) {
  if (!h) return COF_ERR_ARG;
  h->autotune = enable != 0;
  h->jobs_on_device = false;  // choose again on the next search
  return COF_OK;
}

cof_status cof_schedule_text(cof_handle* h, const char** text, size_t* len) {
  if (!h || !text || !len) return COF_ERR_ARG;
  std::string t;
  for (const PatternGroup& g : h->groups) {
    char line[256];
    snprintf(line, sizeof line, "%s variants=%zu slots=%d", g.pattern.c_str(), g.gids.size(), g.bs_slots);
    t += line;
    if (g.bs_slots) {
      snprintf(line, sizeof line, " m=%u chunks=%u planes=%s", g.bs_m, g.bs_chunks,
               g.bs_narrow && g.bs_m > 1 ? "NB" : "NB+1");
      t += line;
      if (!g.bs_tuned.empty()) {
        t += " tuned:";
        for (const auto& x : g.bs_tuned) {
          snprintf(line, sizeof line, " m=%u %.1fus", x.first, x.second);
          t += line;
        }
      }
    } else {
      t += " popcount";
    }
    t += "\n";
  }
  h->summary_text = t;
  *text = h->summary_text.c_str();
  *len = h->summary_text.size();
  return COF_OK;
}

cof_status cof_comparer_info(const cof_handle* h, int* kind, int* slots) {
  if (!h) return COF_ERR_ARG;
  int k = 0, sl = 0;
  for (const PatternGroup& g : h->groups) {
    k = std::max(k, g.bs_slots ? 2 : 1);
    sl = std::max(sl, g.bs_slots);
  }
  if (kind) *kind = k ? k : 1;
  if (slots) *slots = sl;
  return COF_OK;
}

cof_status cof_set_profiling(cof_handle* h, int enable) {
  if (!h) return COF_ERR_ARG;
  h->profiling = enable != 0;
  return COF_OK;
}

cof_status cof_kernel_stats(const cof_handle* h, const char* name, uint64_t* launches, double* total_ms,
                            double* units) {
  if (!h || !name) return COF_ERR_ARG;
  auto it = h->stats.find(name);
  KernelStat s = it == h->stats.end() ? KernelStat() : it->second;
  if (launches) *launches = s.launches;
  if (total_ms) *total_ms = s.ms;
  if (units) *units = s.units;
  return COF_OK;
}

cof_status cof_reset_stats(cof_handle* h) {
  if (!h) return COF_ERR_ARG;
  h->stats.clear();
  return COF_OK;
}

cof_status cof_timer_start(cof_handle* h) {
  if (!h) return COF_ERR_ARG;
  cudaSetDevice(h->device);
  if (!h->timer_a) COF_CUDA(h, cudaEventCreate(&h->timer_a));
  if (!h->timer_b) COF_CUDA(h, cudaEventCreate(&h->timer_b));
  COF_CUDA(h, cudaEventRecord(h->timer_a, h->stream));
  return COF_OK;
}

cof_status cof_timer_stop(cof_handle* h, double* ms) {
  if (!h || !ms || !h->timer_a) return COF_ERR_ARG;
  COF_CUDA(h, cudaEventRecord(h->timer_b, h->stream));
  COF_CUDA(h, cudaEventSynchronize(h->timer_b));
  float f = 0;
  COF_CUDA(h, cudaEventElapsedTime(&f, h->timer_a, h->timer_b));
  *ms = f;
  return COF_OK;
}

cof_status cof_synchronize(cof_handle* h) {
  if (!h) return COF_ERR_ARG;
  COF_CUDA(h, cudaStreamSynchronize(h->stream));
  return COF_OK;
}

}  // extern "C"
