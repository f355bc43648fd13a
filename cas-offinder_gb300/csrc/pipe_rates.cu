// Integer-pipe throughput probe: libcofrates.so, a measurement library that
// bench.py loads beside the engine; it is not part of libcasoff.so.
//
// The comparer's roofline is set by the integer pipes, not by HBM or the tensor
// cores, so its denominator is measured here on the running GPU: sustained
// lane-operations per second of LOP3, POPC and IADD3, each from a kernel of
// many independent dependency chains (enough warps and chains to saturate the
// pipe), timed with CUDA events.
//
//   int cofx_pipe_rates(int device, double* lop3, double* popc, double* iadd);
// measures on CUDA device `device`, in lane-operations per second: LOP3
// (3-input logic), POPC (population count) and IADD (32-bit add).  Takes
// about a second.  Returns 0 on success.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

namespace {

constexpr int kChains = 8;
constexpr int kIters = 4096;
constexpr int kUnroll = 8;

__global__ void lop3_loop(uint32_t* sink, uint32_t seed) {
  uint32_t a[kChains];
  const uint32_t b = seed ^ threadIdx.x, c = seed * 3u + blockIdx.x;
#pragma unroll
  for (int i = 0; i < kChains; ++i) a[i] = seed + i * 0x9E3779B9u + threadIdx.x;
  for (int it = 0; it < kIters; ++it) {
#pragma unroll
    for (int u = 0; u < kUnroll; ++u)
#pragma unroll
      for (int i = 0; i < kChains; ++i) asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(a[i]) : "r"(b), "r"(c));
  }
  uint32_t x = 0;
#pragma unroll
  for (int i = 0; i < kChains; ++i) x ^= a[i];
  if (x == 0x12345678u) sink[0] = x;
}

__global__ void popc_loop(uint32_t* sink, uint32_t seed) {
  uint32_t a[kChains];
#pragma unroll
  for (int i = 0; i < kChains; ++i) a[i] = seed + i * 0x9E3779B9u + threadIdx.x;
  for (int it = 0; it < kIters; ++it) {
#pragma unroll
    for (int u = 0; u < kUnroll; ++u)
#pragma unroll
      for (int i = 0; i < kChains; ++i) asm volatile("popc.b32 %0, %0;" : "+r"(a[i]));
  }
  uint32_t x = 0;
#pragma unroll
  for (int i = 0; i < kChains; ++i) x ^= a[i];
  if (x == 0x12345678u) sink[0] = x;
}

__global__ void iadd3_loop(uint32_t* sink, uint32_t seed) {
  uint32_t a[kChains];
  const uint32_t b = seed ^ threadIdx.x, c = seed * 3u + blockIdx.x;
#pragma unroll
  for (int i = 0; i < kChains; ++i) a[i] = seed + i * 0x9E3779B9u + threadIdx.x;
  for (int it = 0; it < kIters; ++it) {
#pragma unroll
    for (int u = 0; u < kUnroll; ++u)
#pragma unroll
      for (int i = 0; i < kChains; ++i) asm volatile("add.u32 %0, %0, %1;\n\tadd.u32 %0, %0, %2;" : "+r"(a[i]) : "r"(b), "r"(c));
  }
  uint32_t x = 0;
#pragma unroll
  for (int i = 0; i < kChains; ++i) x ^= a[i];
  if (x == 0x12345678u) sink[0] = x;
}

template <typename K>
double rate(K kernel, int blocks, int threads, double ops_per_thread, uint32_t* sink) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  kernel<<<blocks, threads>>>(sink, 1u);  // warm-up
  cudaEventRecord(a);
  kernel<<<blocks, threads>>>(sink, 2u);
  cudaEventRecord(b);
  cudaEventSynchronize(b);
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (cudaGetLastError() != cudaSuccess || ms <= 0) return 0;
  return (double)blocks * threads * ops_per_thread / (ms * 1e-3);
}

// Device -> pinned host copy by the SMs: 16-byte loads from device memory,
// 16-byte stores to the host buffer's device-mapped address.
__global__ void sm_copy(const uint4* __restrict__ src, uint4* __restrict__ dst, size_t n16) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

}  // namespace

//   int cofx_d2h_rates(int device, size_t bytes, double* dma, double* sm, double* dma2);
// Device -> pinned host copy rates in bytes/s for a buffer of `bytes` (a
// multiple of 32): one cudaMemcpyAsync (copy engine), a kernel whose threads
// store into the mapped host buffer, and two copies of half the buffer each
// on two streams at once.  Best of three each.  Returns 0 on success.
extern "C" int cofx_d2h_rates(int device, size_t bytes, double* dma, double* sm, double* dma2) {
  if (cudaSetDevice(device) != cudaSuccess || bytes == 0 || bytes % 32) return 1;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  void *d = nullptr, *h = nullptr, *hd = nullptr;
  if (cudaMalloc(&d, bytes) != cudaSuccess) return 1;
  if (cudaHostAlloc(&h, bytes, cudaHostAllocMapped) != cudaSuccess) {
    cudaFree(d);
    return 1;
  }
  int rc = 0;
  if (cudaHostGetDevicePointer(&hd, h, 0) != cudaSuccess || cudaMemset(d, 1, bytes) != cudaSuccess) rc = 1;
  cudaEvent_t a, b, j;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventCreate(&j);
  cudaStream_t s2 = nullptr;
  if (cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking) != cudaSuccess) rc = 1;
  double best_dma = 0, best_sm = 0, best_dma2 = 0;
  for (int rep = 0; rc == 0 && rep < 4; ++rep) {  // the first of each is a warm-up
    float ms = 0;
    cudaEventRecord(a);
    cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, 0);
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    cudaEventElapsedTime(&ms, a, b);
    if (rep && ms > 0) best_dma = std::max(best_dma, bytes / (ms * 1e-3));
    cudaEventRecord(a);
    sm_copy<<<sms * 4, 512>>>((const uint4*)d, (uint4*)hd, bytes / 16);
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    cudaEventElapsedTime(&ms, a, b);
    if (rep && ms > 0) best_sm = std::max(best_sm, bytes / (ms * 1e-3));
    // Two halves at once, on the legacy stream and on s2.
    cudaEventRecord(a);
    cudaStreamWaitEvent(s2, a, 0);
    cudaMemcpyAsync(h, d, bytes / 2, cudaMemcpyDeviceToHost, 0);
    cudaMemcpyAsync((char*)h + bytes / 2, (const char*)d + bytes / 2, bytes / 2, cudaMemcpyDeviceToHost, s2);
    cudaEventRecord(j, s2);
    cudaStreamWaitEvent(0, j, 0);
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    cudaEventElapsedTime(&ms, a, b);
    if (rep && ms > 0) best_dma2 = std::max(best_dma2, bytes / (ms * 1e-3));
  }
  if (cudaGetLastError() != cudaSuccess) rc = 1;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaEventDestroy(j);
  if (s2) cudaStreamDestroy(s2);
  cudaFreeHost(h);
  cudaFree(d);
  if (dma) *dma = best_dma;
  if (sm) *sm = best_sm;
  if (dma2) *dma2 = best_dma2;
  return rc;
}

extern "C" int cofx_pipe_rates(int device, double* lop3, double* popc, double* iadd) {
  if (cudaSetDevice(device) != cudaSuccess) return 1;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  uint32_t* sink = nullptr;
  if (cudaMalloc(&sink, 4) != cudaSuccess) return 1;
  const int threads = 256, blocks = sms * 8;
  const double per = (double)kIters * kUnroll * kChains;
  if (lop3) *lop3 = rate(lop3_loop, blocks, threads, per, sink);
  if (popc) *popc = rate(popc_loop, blocks, threads, per, sink);
  // iadd3_loop issues two dependent add.u32 per chain step; ptxas may fuse them
  // into one IADD3, so count one operation per pair (a lower bound on adds).
  if (iadd) *iadd = rate(iadd3_loop, blocks, threads, per, sink);
  cudaFree(sink);
  return cudaGetLastError() == cudaSuccess ? 0 : 1;
}
