// cof_search_chunk_static: search one genome chunk without allocating memory.
//
// Who needs this: callers that are not allowed to allocate device memory at
// the point where they search -- for example a host application that reserves
// all of its GPU memory up front in its own pool and forbids other
// allocations, or a latency-sensitive caller for whom the implicit device-wide
// synchronization of cudaMalloc/cudaFree would stall unrelated streams.  Such a
// caller owns the genome planes and the hit buffer (device memory it allocated
// earlier) and passes them in; the only other memory the search needs, the
// candidate queue between the PAM scan and the comparer, lives in a fixed
// file-scope device array instead of a per-call allocation.
//
// That array is `g_static_scratch` below: kStaticMaxPositions (2^21) start
// positions' worth of queue, 16 MiB, allocated by the CUDA runtime on every
// GPU that loads this library and held until the process exits.  Chunks longer
// than that are rejected with COF_ERR_TOO_LARGE.
//
// Host code cannot use the array's name as a device address: in host code it
// names a host-side shadow.  The first call on each device therefore looks up
// the device address with cudaGetSymbolAddress (with that device current),
// checks the result, and caches it per device; later calls reuse it.  Make the
// first call on a device before any stream capture begins.
//
// The pattern and compare string are upper-cased first, as the reference does
// with its input file; every other byte keeps its meaning (IUPAC codes, 'N'
// and any byte outside the IUPAC set never mismatch).  The compare string's
// masks are handed to the GPU as a kernel argument, so the call reads no host
// memory after it returns.
//
// Every call shares the one array, and the array keeps what the last call left
// in it: each call clears the queue counter (and the caller's hit counter)
// before use.  Two calls whose work overlaps on the GPU (different streams, or
// different host threads, without ordering between them) race on the array and
// give wrong results; order them, e.g. issue them on one stream.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "../../include/cof.h"
#include "cof_internal.h"
#include "kernels.cuh"

namespace {

using namespace cof;

constexpr uint64_t kStaticMaxPositions = 1ull << 21;
// Word layout of the scratch array: [0] queue counter, [16, 16 + 64) the
// compare variant's class masks, [kQueueOffset, ...) the candidate queue
// (at most 2 entries per start position, plus one word of rounding).
constexpr uint64_t kMaskOffset = 16;
constexpr uint64_t kQueueOffset = 128;
constexpr uint64_t kScratchWords = kQueueOffset + 2 * (kStaticMaxPositions + 32);

static __device__ __align__(256) uint32_t g_static_scratch[kScratchWords];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of g_static_scratch on the current device (set up once per device).
cudaError_t scratch_address(uint32_t** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[dev] = p;
  }
  *out = (uint32_t*)g_scratch_addr[dev];
  return cudaSuccess;
}

std::string revcomp_of(const std::string& s) {
  const size_t L = s.size();
  std::string r(L, 'N');
  for (size_t k = 0; k < L; ++k) r[k] = (char)complement_byte((unsigned char)s[L - 1 - k]);
  return r;
}

// The reference upper-cases the pattern and every guide before it builds its
// compare strings (cas-offinder.cpp:625, :640); so does this entry point.
std::string upper_of(const char* s, uint32_t L) {
  std::string r(s, L);
  for (char& c : r)
    if (c >= 'a' && c <= 'z') c = (char)(c - 32);
  return r;
}

// Writes one variant's class masks into the scratch array.  The masks travel
// as a kernel argument, so nothing on the host is read after the launch is
// queued.
template <int NW>
__global__ void store_mask_kernel(VariantMask<NW> vm, VariantMask<NW>* dst) {
  if (threadIdx.x == 0) *dst = vm;
}

template <int NW>
void fill_mask(VariantMask<NW>& vm, const std::string& comp, uint32_t L, uint32_t thr) {
  std::memset(&vm, 0, sizeof vm);
  for (uint32_t k = 0; k < L; ++k) {
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
  vm.gid = 0;
}

}  // namespace

extern "C" cof_status cof_search_chunk_static(const uint32_t* d_hi, const uint32_t* d_lo, const uint32_t* d_ot,
                                              uint64_t n, const char* pattern, const char* comp,
                                              uint32_t patternlen, uint16_t threshold, uint64_t* d_hits,
                                              uint64_t hit_cap, unsigned long long* d_hit_count, void* stream) {
  if (!d_hi || !d_lo || !d_ot || !pattern || !comp || !d_hits || !d_hit_count) return COF_ERR_ARG;
  if (patternlen == 0 || patternlen > (uint32_t)kMaxL) return COF_ERR_UNSUPPORTED;
  if (n > kStaticMaxPositions) return COF_ERR_TOO_LARGE;
  cudaStream_t st = (cudaStream_t)stream;
  // An unread error of the caller's own CUDA work is left for the caller:
  // nothing is queued, so every error this call reports after its launches
  // is its own.
  if (cudaPeekAtLastError() != cudaSuccess) return COF_ERR_CUDA;
  uint32_t* scratch = nullptr;
  if (scratch_address(&scratch) != cudaSuccess) return COF_ERR_CUDA;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return COF_ERR_CUDA;

  // Both counters start at zero on every call.
  if (cudaMemsetAsync(scratch, 0, sizeof(uint32_t), st) != cudaSuccess) return COF_ERR_CUDA;
  if (cudaMemsetAsync(d_hit_count, 0, sizeof(unsigned long long), st) != cudaSuccess) return COF_ERR_CUDA;
  const uint64_t npos = n >= patternlen ? n - patternlen + 1 : 0;
  if (npos == 0) return COF_OK;

  FinderPattern fp;
  std::memset(&fp, 0, sizeof fp);
  const std::string pat = upper_of(pattern, patternlen), cmp = upper_of(comp, patternlen);
  const std::string rev = revcomp_of(pat);
  fp.L = patternlen;
  for (uint32_t k = 0; k < patternlen; ++k) {
    const uint32_t mf = class_bits_of((unsigned char)pat[k]);
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
  const int nw = patternlen <= 32 ? 1 : 2;
  if (nw == 1) {
    VariantMask<1> vm;
    fill_mask<1>(vm, cmp, patternlen, threshold);
    store_mask_kernel<1><<<1, 32, 0, st>>>(vm, reinterpret_cast<VariantMask<1>*>(scratch + kMaskOffset));
  } else {
    VariantMask<2> vm;
    fill_mask<2>(vm, cmp, patternlen, threshold);
    store_mask_kernel<2><<<1, 32, 0, st>>>(vm, reinterpret_cast<VariantMask<2>*>(scratch + kMaskOffset));
  }
  if (cudaGetLastError() != cudaSuccess) return COF_ERR_CUDA;

  GenomeView g;
  std::memset(&g, 0, sizeof g);
  g.hi = d_hi;
  g.lo = d_lo;
  g.ot = d_ot;
  g.n = n;
  launch_finder(g, 0, (npos + 31) / 32, fp, scratch + kQueueOffset, scratch, st);
  launch_comparer(g, scratch + kQueueOffset, scratch, 0, scratch + kMaskOffset, 1, nw, patternlen, d_hits,
                  d_hit_count, hit_cap, sms, st);
  return cudaGetLastError() == cudaSuccess ? COF_OK : COF_ERR_CUDA;
}
