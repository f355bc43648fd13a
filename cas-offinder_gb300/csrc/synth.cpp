// Deterministic synthetic genome records (cofx_synth_record, include/cof_tools.h).
//
// Counter-based: every 64 Ki-base block draws from its own splitmix64 stream
// keyed by (seed, record, block), so blocks are generated in parallel and the
// result does not depend on the thread count or the platform.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "../../include/cof_tools.h"

namespace {

inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

struct Stream {
  uint64_t s;
  explicit Stream(uint64_t key) : s(mix64(key)) {}
  uint64_t next() { return mix64(s += 0x9E3779B97F4A7C15ull); }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

inline uint64_t key_of(uint64_t seed, uint64_t record, uint64_t lane, uint64_t index) {
  return mix64(seed * 0x9E3779B97F4A7C15ull ^ mix64(record + 0x632BE59BD9B4E019ull) ^ mix64(lane << 56 ^ index));
}

constexpr uint64_t kBlock = 1u << 16;

}  // namespace

extern "C" uint64_t cofx_synth_record(uint64_t seed, uint32_t record, uint64_t len, double gc, double gc_drift,
                                      uint32_t drift_window, double n_frac, uint32_t n_run_min, uint32_t n_run_max,
                                      char* out) {
  if (!out || len == 0) return 0;
  if (drift_window == 0) drift_window = 100000;
  const uint64_t nblocks = (len + kBlock - 1) / kBlock;
  auto gc_at = [&](uint64_t window) {
    double g = gc;
    if (gc_drift > 0) {
      Stream st(key_of(seed, record, 1, window));
      g += gc_drift * (2.0 * st.uniform() - 1.0);
    }
    return std::min(1.0, std::max(0.0, g));
  };
  auto work = [&](uint64_t b0, uint64_t b1) {
    for (uint64_t b = b0; b < b1; ++b) {
      Stream st(key_of(seed, record, 0, b));
      const uint64_t p0 = b * kBlock, p1 = std::min(len, p0 + kBlock);
      uint64_t window = ~0ull;
      uint32_t t_a = 0, t_c = 0, t_g = 0;
      uint64_t bits = 0;
      int left = 0;
      for (uint64_t p = p0; p < p1; ++p) {
        if (p / drift_window != window) {
          window = p / drift_window;
          const double g = gc_at(window);
          // Cumulative thresholds on a 32-bit draw: A < (1-g)/2 <= C < 1/2 <= G < (1+g)/2 <= T.
          const double two32 = 4294967296.0;
          t_a = (uint32_t)std::min(4294967295.0, std::floor((1.0 - g) / 2 * two32));
          t_c = 2147483648u;
          t_g = (uint32_t)std::min(4294967295.0, std::floor((1.0 + g) / 2 * two32));
        }
        if (left == 0) {
          bits = st.next();
          left = 2;
        }
        const uint32_t u = (uint32_t)bits;
        bits >>= 32;
        --left;
        out[p] = u < t_a ? 'A' : u < t_c ? 'C' : u < t_g ? 'G' : 'T';
      }
    }
  };
  unsigned T = std::thread::hardware_concurrency();
  if (T == 0) T = 4;
  T = (unsigned)std::min<uint64_t>(T, nblocks);
  std::vector<std::thread> pool;
  for (unsigned t = 1; t < T; ++t) pool.emplace_back(work, nblocks * t / T, nblocks * (t + 1) / T);
  work(0, nblocks / T);
  for (auto& th : pool) th.join();

  if (n_frac > 0 && n_run_max >= n_run_min && n_run_max > 0) {
    const double mean = 0.5 * ((double)n_run_min + (double)n_run_max);
    const uint64_t runs = (uint64_t)std::llround(n_frac * (double)len / mean);
    Stream st(key_of(seed, record, 2, 0));
    for (uint64_t r = 0; r < runs; ++r) {
      const uint64_t start = st.next() % len;
      const uint64_t span = (uint64_t)n_run_min + st.next() % ((uint64_t)n_run_max - n_run_min + 1);
      const uint64_t end = std::min(len, start + span);
      std::memset(out + start, 'N', end - start);
    }
  }
  std::vector<uint64_t> part(T, 0);
  auto count = [&](unsigned t) {
    const uint64_t a = len * t / T, z = len * (t + 1) / T;
    uint64_t c = 0;
    for (uint64_t p = a; p < z; ++p) c += out[p] == 'N';
    part[t] = c;
  };
  pool.clear();
  for (unsigned t = 1; t < T; ++t) pool.emplace_back(count, t);
  count(0);
  for (auto& th : pool) th.join();
  uint64_t nn = 0;
  for (uint64_t c : part) nn += c;
  return nn;
}
