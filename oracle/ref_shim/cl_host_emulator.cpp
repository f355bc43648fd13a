/*
 * Host-only OpenCL emulator for running the reference Cas-OFFinder 3.0.0 here.
 *
 * TEST INFRASTRUCTURE (the oracle).  Nothing in the product links this file.
 *
 * The reference's host code talks to OpenCL through oclfunctions.cpp:5-296 and
 * launches four kernels written in OpenCL C (cas-offinder.cl:6-286).  This
 * container has no OpenCL driver, so this file provides the ~20 API entry
 * points those sources call, with plain host semantics:
 *   - buffers are malloc'd host memory; enqueue read/write is memcpy;
 *   - clCreateKernel binds the kernels of cas-offinder.cl itself, which is
 *     #included below and compiled as C++ (OpenCL qualifiers become empty
 *     macros, get_global_id() reads a thread-local work-item id, atomic_inc is a
 *     relaxed atomic fetch-add);
 *   - clEnqueueNDRangeKernel runs the NDRange with OpenMP.  The *_cpu kernels
 *     run one work-item per iteration; the work-group kernels (finder and
 *     comparer, which stage the pattern into __local memory) run one work-group
 *     per iteration, its work-items in order, so the li==0 copy precedes the
 *     reads that follow the barrier.
 *   - one platform with one CPU device and one GPU device; both run on the
 *     host.  CL_DEVICE_MAX_MEM_ALLOC_SIZE comes from COF_EMU_MAX_ALLOC (bytes,
 *     default 2^40), which sets the reference's chunk size
 *     (cas-offinder.cpp:189-194): a small value exercises its chunking.
 * With OMP_NUM_THREADS=1 the atomic append order is the work-item order, which
 * makes the reference's output deterministic.
 */
#include "CL/cl.h"

#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

// ---- the reference kernels, compiled as C++ -------------------------------
namespace refcl {
static thread_local size_t g_global_id = 0;
static thread_local size_t g_group_id = 0;
static thread_local size_t g_local_size = 1;
static inline size_t get_global_id(unsigned) { return g_global_id; }
static inline size_t get_group_id(unsigned) { return g_group_id; }
static inline size_t get_local_size(unsigned) { return g_local_size; }
static inline void barrier(int) {}
static inline unsigned int atomic_inc(unsigned int* p) {
  return __atomic_fetch_add(p, 1u, __ATOMIC_RELAXED);
}
#define CLK_LOCAL_MEM_FENCE 1
#define __kernel static
#define __global
#define __constant
#define __local
#pragma GCC diagnostic push
#pragma GCC diagnostic ignored "-Wunknown-pragmas"
#pragma GCC diagnostic ignored "-Wsign-compare"
#include COF_REFERENCE_KERNELS
#pragma GCC diagnostic pop
#undef __kernel
#undef __global
#undef __constant
#undef __local
}  // namespace refcl

// ---- object model ------------------------------------------------------------
struct _cl_platform_id { int dummy; };
struct _cl_device_id { cl_device_type type; const char* name; };
struct _cl_context { cl_device_id dev; };
struct _cl_command_queue { cl_context ctx; };
struct _cl_mem { void* data; size_t size; };
struct _cl_program { cl_context ctx; };
struct KernelArg { std::vector<unsigned char> bytes; size_t local_size = 0; bool is_local = false; };
struct _cl_kernel { std::string name; std::vector<KernelArg> args; };
struct _cl_event { int dummy; };

static _cl_platform_id g_platform;
static _cl_device_id g_cpu = {CL_DEVICE_TYPE_CPU, "Host emulator CPU device"};
static _cl_device_id g_gpu = {CL_DEVICE_TYPE_GPU, "Host emulator GPU device"};

static cl_int put_info(const void* src, size_t n, size_t cap, void* dst, size_t* ret) {
  if (ret) *ret = n;
  if (dst) {
    if (cap < n) return CL_INVALID_VALUE;
    std::memcpy(dst, src, n);
  }
  return CL_SUCCESS;
}

extern "C" {

cl_int clGetPlatformIDs(cl_uint num_entries, cl_platform_id* platforms, cl_uint* num_platforms) {
  if (platforms && num_entries > 0) platforms[0] = &g_platform;
  if (num_platforms) *num_platforms = 1;
  return CL_SUCCESS;
}

cl_int clGetPlatformInfo(cl_platform_id, cl_platform_info param_name, size_t sz, void* val, size_t* ret) {
  static const char name[] = "cof host OpenCL emulator";
  if (param_name == CL_PLATFORM_NAME) return put_info(name, sizeof(name), sz, val, ret);
  return CL_INVALID_VALUE;
}

cl_int clGetDeviceIDs(cl_platform_id, cl_device_type type, cl_uint num_entries, cl_device_id* devices,
                      cl_uint* num_devices) {
  cl_device_id d = nullptr;
  if (type & CL_DEVICE_TYPE_CPU) d = &g_cpu;
  else if (type & CL_DEVICE_TYPE_GPU) d = &g_gpu;
  if (!d) {
    if (num_devices) *num_devices = 0;
    return CL_DEVICE_NOT_FOUND;
  }
  if (devices && num_entries > 0) devices[0] = d;
  if (num_devices) *num_devices = 1;
  return CL_SUCCESS;
}

cl_int clGetDeviceInfo(cl_device_id dev, cl_device_info param_name, size_t sz, void* val, size_t* ret) {
  if (param_name == CL_DEVICE_MAX_MEM_ALLOC_SIZE) {
    cl_ulong v = 1ull << 40;
    if (const char* e = std::getenv("COF_EMU_MAX_ALLOC")) v = std::strtoull(e, nullptr, 10);
    return put_info(&v, sizeof(v), sz, val, ret);
  }
  if (param_name == CL_DEVICE_NAME) return put_info(dev->name, std::strlen(dev->name) + 1, sz, val, ret);
  return CL_INVALID_VALUE;
}

cl_context clCreateContext(const cl_context_properties*, cl_uint, const cl_device_id* devices,
                           void(CL_CALLBACK*)(const char*, const void*, size_t, void*), void*,
                           cl_int* err) {
  if (err) *err = CL_SUCCESS;
  return new _cl_context{devices[0]};
}
cl_int clReleaseContext(cl_context c) { delete c; return CL_SUCCESS; }

cl_command_queue clCreateCommandQueue(cl_context ctx, cl_device_id, cl_command_queue_properties, cl_int* err) {
  if (err) *err = CL_SUCCESS;
  return new _cl_command_queue{ctx};
}
cl_int clReleaseCommandQueue(cl_command_queue q) { delete q; return CL_SUCCESS; }

cl_mem clCreateBuffer(cl_context, cl_mem_flags, size_t size, void* host_ptr, cl_int* err) {
  void* p = std::calloc(size ? size : 1, 1);
  if (!p) {
    if (err) *err = CL_OUT_OF_HOST_MEMORY;
    return nullptr;
  }
  if (host_ptr) std::memcpy(p, host_ptr, size);
  if (err) *err = CL_SUCCESS;
  return new _cl_mem{p, size};
}
cl_int clReleaseMemObject(cl_mem m) {
  std::free(m->data);
  delete m;
  return CL_SUCCESS;
}

cl_program clCreateProgramWithSource(cl_context ctx, cl_uint, const char**, const size_t*, cl_int* err) {
  if (err) *err = CL_SUCCESS;
  return new _cl_program{ctx};
}
cl_int clBuildProgram(cl_program, cl_uint, const cl_device_id*, const char*, void(CL_CALLBACK*)(cl_program, void*),
                      void*) {
  return CL_SUCCESS;
}
cl_int clGetProgramBuildInfo(cl_program, cl_device_id, cl_program_build_info, size_t sz, void* val, size_t* ret) {
  return put_info("", 1, sz, val, ret);
}

cl_kernel clCreateKernel(cl_program, const char* name, cl_int* err) {
  std::string n(name);
  if (n != "finder" && n != "comparer" && n != "finder_cpu" && n != "comparer_cpu") {
    if (err) *err = CL_INVALID_KERNEL_NAME;
    return nullptr;
  }
  if (err) *err = CL_SUCCESS;
  auto* k = new _cl_kernel{n, {}};
  k->args.resize(13);
  return k;
}
cl_int clReleaseKernel(cl_kernel k) { delete k; return CL_SUCCESS; }

cl_int clSetKernelArg(cl_kernel k, cl_uint idx, size_t size, const void* value) {
  if (idx >= k->args.size()) return CL_INVALID_ARG_INDEX;
  KernelArg& a = k->args[idx];
  if (value == nullptr) {  // __local argument: size bytes per work-group
    a.is_local = true;
    a.local_size = size;
    a.bytes.clear();
  } else {
    a.is_local = false;
    a.bytes.assign((const unsigned char*)value, (const unsigned char*)value + size);
  }
  return CL_SUCCESS;
}

cl_int clEnqueueWriteBuffer(cl_command_queue, cl_mem buf, cl_bool, size_t off, size_t size, const void* ptr,
                            cl_uint, const cl_event*, cl_event* ev) {
  if (off + size > buf->size) return CL_INVALID_VALUE;
  std::memcpy((char*)buf->data + off, ptr, size);
  if (ev) *ev = nullptr;
  return CL_SUCCESS;
}

cl_int clEnqueueReadBuffer(cl_command_queue, cl_mem buf, cl_bool, size_t off, size_t size, void* ptr, cl_uint,
                           const cl_event*, cl_event* ev) {
  if (off + size > buf->size) return CL_INVALID_VALUE;
  std::memcpy(ptr, (char*)buf->data + off, size);
  if (ev) *ev = nullptr;
  return CL_SUCCESS;
}

cl_int clFinish(cl_command_queue) { return CL_SUCCESS; }

}  // extern "C"

template <typename T>
static T* mem_arg(const _cl_kernel* k, int i) {
  cl_mem m;
  std::memcpy(&m, k->args[i].bytes.data(), sizeof(cl_mem));
  return (T*)m->data;
}
template <typename T>
static T val_arg(const _cl_kernel* k, int i) {
  T v;
  std::memcpy(&v, k->args[i].bytes.data(), sizeof(T));
  return v;
}

extern "C" cl_int clEnqueueNDRangeKernel(cl_command_queue, cl_kernel k, cl_uint, const size_t*, const size_t* gws,
                                         const size_t* lws, cl_uint, const cl_event*, cl_event* ev) {
  const size_t n = gws[0];
  if (ev) *ev = nullptr;
  if (k->name == "finder_cpu") {
    char* chr = mem_arg<char>(k, 0);
    char* pat = mem_arg<char>(k, 1);
    int* pat_index = mem_arg<int>(k, 2);
    unsigned int plen = val_arg<unsigned int>(k, 3);
    char* flag = mem_arg<char>(k, 4);
    unsigned int* cnt = mem_arg<unsigned int>(k, 5);
    unsigned int* loci = mem_arg<unsigned int>(k, 6);
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)n; ++i) {
      refcl::g_global_id = (size_t)i;
      refcl::finder_cpu(chr, pat, pat_index, plen, flag, cnt, loci);
    }
    return CL_SUCCESS;
  }
  if (k->name == "comparer_cpu") {
    char* chr = mem_arg<char>(k, 0);
    unsigned int* loci = mem_arg<unsigned int>(k, 1);
    unsigned int* mm_loci = mem_arg<unsigned int>(k, 2);
    char* comp = mem_arg<char>(k, 3);
    int* comp_index = mem_arg<int>(k, 4);
    unsigned int plen = val_arg<unsigned int>(k, 5);
    unsigned short thr = val_arg<unsigned short>(k, 6);
    char* flag = mem_arg<char>(k, 7);
    unsigned short* mm_count = mem_arg<unsigned short>(k, 8);
    char* direction = mem_arg<char>(k, 9);
    unsigned int* cnt = mem_arg<unsigned int>(k, 10);
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)n; ++i) {
      refcl::g_global_id = (size_t)i;
      refcl::comparer_cpu(chr, loci, mm_loci, comp, comp_index, plen, thr, flag, mm_count, direction, cnt);
    }
    return CL_SUCCESS;
  }
  // Work-group kernels: the OpenCL runtime picks the local size when none is
  // given; 256 is used here.  A partial last group runs only its valid ids.
  const size_t ls = lws ? lws[0] : 256;
  const long long groups = (long long)((n + ls - 1) / ls);
  if (k->name == "finder") {
    char* chr = mem_arg<char>(k, 0);
    char* pat = mem_arg<char>(k, 1);
    int* pat_index = mem_arg<int>(k, 2);
    unsigned int plen = val_arg<unsigned int>(k, 3);
    char* flag = mem_arg<char>(k, 4);
    unsigned int* cnt = mem_arg<unsigned int>(k, 5);
    unsigned int* loci = mem_arg<unsigned int>(k, 6);
    const size_t l0 = k->args[7].local_size, l1 = k->args[8].local_size;
#pragma omp parallel
    {
      std::vector<char> lp(l0 + 1);
      std::vector<int> li((l1 + sizeof(int) - 1) / sizeof(int) + 1);
#pragma omp for schedule(static)
      for (long long g = 0; g < groups; ++g) {
        refcl::g_group_id = (size_t)g;
        refcl::g_local_size = ls;
        for (size_t t = 0; t < ls && g * ls + t < n; ++t) {
          refcl::g_global_id = g * ls + t;
          refcl::finder(chr, pat, pat_index, plen, flag, cnt, loci, lp.data(), li.data());
        }
      }
    }
    return CL_SUCCESS;
  }
  if (k->name == "comparer") {
    char* chr = mem_arg<char>(k, 0);
    unsigned int* loci = mem_arg<unsigned int>(k, 1);
    unsigned int* mm_loci = mem_arg<unsigned int>(k, 2);
    char* comp = mem_arg<char>(k, 3);
    int* comp_index = mem_arg<int>(k, 4);
    unsigned int plen = val_arg<unsigned int>(k, 5);
    unsigned short thr = val_arg<unsigned short>(k, 6);
    char* flag = mem_arg<char>(k, 7);
    unsigned short* mm_count = mem_arg<unsigned short>(k, 8);
    char* direction = mem_arg<char>(k, 9);
    unsigned int* cnt = mem_arg<unsigned int>(k, 10);
    const size_t l0 = k->args[11].local_size, l1 = k->args[12].local_size;
#pragma omp parallel
    {
      std::vector<char> lp(l0 + 1);
      std::vector<int> li((l1 + sizeof(int) - 1) / sizeof(int) + 1);
#pragma omp for schedule(static)
      for (long long g = 0; g < groups; ++g) {
        refcl::g_group_id = (size_t)g;
        refcl::g_local_size = ls;
        for (size_t t = 0; t < ls && g * ls + t < n; ++t) {
          refcl::g_global_id = g * ls + t;
          refcl::comparer(chr, loci, mm_loci, comp, comp_index, plen, thr, flag, mm_count, direction, cnt,
                          lp.data(), li.data());
        }
      }
    }
    return CL_SUCCESS;
  }
  return CL_INVALID_VALUE;
}
