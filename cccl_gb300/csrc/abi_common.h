// Host helpers shared by the radix-sort and segmented-sort C ABIs: CUDA error
// propagation, the primary-context push, embedded cubins, key codecs, driver-API launch
// and the build-result blob format.
#pragma once

#ifndef CCCL_C_EXPERIMENTAL
#  define CCCL_C_EXPERIMENTAL 1
#endif

#include <cuda.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include <cccl/c/types.h>

#include "sort_params.h"

namespace gb300
{

// A CUDA driver error carried as an exception inside the ABI; converted back to the
// CUresult at the boundary (the reference's check() in c/parallel/src/util/errors.cpp
// turns them into exceptions the same way).
struct cuda_error : std::runtime_error
{
  CUresult code;
  cuda_error(CUresult c, const std::string& what)
      : std::runtime_error(what)
      , code(c)
  {}
};

inline void check(CUresult r, const char* what)
{
  if (r != CUDA_SUCCESS)
  {
    const char* name = nullptr;
    cuGetErrorName(r, &name);
    throw cuda_error(r, std::string(what) + ": " + (name ? name : "unknown CUDA error"));
  }
}

// Pushes device 0's primary context when no context is current, as the reference does
// (c/parallel/src/util/context.cpp:14-31). Pops it again on destruction.
struct context_guard
{
  bool pushed = false;
  context_guard()
  {
    CUcontext ctx = nullptr;
    check(cuCtxGetCurrent(&ctx), "cuCtxGetCurrent");
    if (ctx == nullptr)
    {
      check(cuDevicePrimaryCtxRetain(&ctx, 0), "cuDevicePrimaryCtxRetain");
      check(cuCtxPushCurrent(ctx), "cuCtxPushCurrent");
      pushed = true;
    }
  }
  ~context_guard()
  {
    if (pushed)
    {
      CUcontext dummy;
      cuCtxPopCurrent(&dummy);
    }
  }
  context_guard(const context_guard&)            = delete;
  context_guard& operator=(const context_guard&) = delete;
};

// ---- embedded sm_103a images ----
struct image_ref
{
  const unsigned char* data;
  size_t size;
};
image_ref radix_image(int key_bytes); // one cubin per key width
image_ref segmented_image(int key_bytes); // one cubin per key width
image_ref learned_image(int key_bytes);   // 4- and 8-byte keys

// ---- key kinds ----
enum key_kind : int
{
  KIND_UNSIGNED = 0,
  KIND_SIGNED   = 1,
  KIND_FLOAT    = 2,
};

inline bool key_kind_of(cccl_type_enum t, int& kind, int& bytes)
{
  switch (t)
  {
    case CCCL_UINT8:
      kind = KIND_UNSIGNED, bytes = 1;
      return true;
    case CCCL_UINT16:
      kind = KIND_UNSIGNED, bytes = 2;
      return true;
    case CCCL_UINT32:
      kind = KIND_UNSIGNED, bytes = 4;
      return true;
    case CCCL_UINT64:
      kind = KIND_UNSIGNED, bytes = 8;
      return true;
    case CCCL_BOOLEAN:
      kind = KIND_UNSIGNED, bytes = 1;
      return true;
    case CCCL_INT8:
      kind = KIND_SIGNED, bytes = 1;
      return true;
    case CCCL_INT16:
      kind = KIND_SIGNED, bytes = 2;
      return true;
    case CCCL_INT32:
      kind = KIND_SIGNED, bytes = 4;
      return true;
    case CCCL_INT64:
      kind = KIND_SIGNED, bytes = 8;
      return true;
    case CCCL_FLOAT16:
      kind = KIND_FLOAT, bytes = 2;
      return true;
    case CCCL_FLOAT32:
      kind = KIND_FLOAT, bytes = 4;
      return true;
    case CCCL_FLOAT64:
      kind = KIND_FLOAT, bytes = 8;
      return true;
    default:
      return false;
  }
}

inline bool supported_value_bytes(size_t vb)
{
  return vb == 0 || vb == 1 || vb == 2 || vb == 4 || vb == 8 || vb == 16;
}

// Encoding of raw key bits to the sortable unsigned order, with descending order folded
// in as a bit inversion (cub/cub/util_type.cuh:893-963 and
// cub/cub/block/radix_rank_sort_operations.cuh:536-575 define the mapping).
// Integer kinds get fwd_pos == fwd_neg (one mask for both signs): the integer kernels'
// counting loops encode with fwd_pos alone (encode_key_for_count).
inline KeyCodec make_codec(int kind, int bytes, bool descending)
{
  const unsigned long long all  = bytes == 8 ? ~0ull : ((1ull << (8 * bytes)) - 1ull);
  const unsigned long long high = 1ull << (8 * bytes - 1);
  KeyCodec c{};
  switch (kind)
  {
    case KIND_UNSIGNED:
      c.fwd_pos = c.fwd_neg = c.inv_set = c.inv_clr = descending ? all : 0ull;
      break;
    case KIND_SIGNED:
      c.fwd_pos = c.fwd_neg = c.inv_set = c.inv_clr = descending ? (all ^ high) : high;
      break;
    default: // floating point
      if (!descending)
      {
        c.fwd_pos = high, c.fwd_neg = all, c.inv_set = high, c.inv_clr = all;
      }
      else
      {
        c.fwd_pos = all ^ high, c.fwd_neg = 0ull, c.inv_set = 0ull, c.inv_clr = all ^ high;
      }
      break;
  }
  return c;
}

// ---- kernels ----
struct kernel_ref
{
  CUkernel k = nullptr;
};

inline CUfunction function_of(CUkernel k)
{
  CUfunction f = nullptr;
  check(cuKernelGetFunction(&f, k), "cuKernelGetFunction");
  return f;
}

// Optional launch observer (include/cccl_gb300/sort_trace.h).
using launch_observer_fn = void (*)(void*, const char*, int, CUstream);
void notify_launch(const char* role, int phase, CUstream stream);

template <class Params>
inline void launch(
  const char* role, CUkernel kernel, unsigned grid, unsigned block, size_t smem, CUstream stream, const Params& p)
{
  CUfunction f = function_of(kernel);
  // dynamic shared memory near the 48 KB default leaves no room for a kernel's static shared
  // memory: opt in above 47 KB
  if (smem > 47 * 1024)
  {
    check(cuFuncSetAttribute(f, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, int(smem)),
          "cuFuncSetAttribute(max dynamic shared memory)");
  }
  void* args[] = {const_cast<Params*>(&p)};
  notify_launch(role, 0, stream);
  check(cuLaunchKernel(f, grid, 1, 1, block, 1, 1, unsigned(smem), stream, args, nullptr), "cuLaunchKernel");
  notify_launch(role, 1, stream);
}

// Cooperative launch: every CTA of the grid is resident at once (the persistent kernels
// wait on each other's tiles, so co-residency is required for forward progress).
template <class Params>
inline void launch_cooperative(
  const char* role, CUkernel kernel, unsigned grid, unsigned block, size_t smem, CUstream stream, const Params& p)
{
  CUfunction f = function_of(kernel);
  if (smem > 48 * 1024)
  {
    check(cuFuncSetAttribute(f, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, int(smem)),
          "cuFuncSetAttribute(max dynamic shared memory)");
  }
  void* args[] = {const_cast<Params*>(&p)};
  notify_launch(role, 0, stream);
  check(cuLaunchCooperativeKernel(f, grid, 1, 1, block, 1, 1, unsigned(smem), stream, args),
        "cuLaunchCooperativeKernel");
  notify_launch(role, 1, stream);
}

// Resident CTAs per SM of a kernel at the given block size and dynamic shared memory.
inline int occupancy(CUkernel kernel, int block, size_t smem)
{
  CUfunction f = function_of(kernel);
  if (smem > 48 * 1024)
  {
    check(cuFuncSetAttribute(f, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, int(smem)),
          "cuFuncSetAttribute(max dynamic shared memory)");
  }
  int n = 0;
  check(cuOccupancyMaxActiveBlocksPerMultiprocessor(&n, f, block, smem), "cuOccupancyMaxActiveBlocksPerMultiprocessor");
  if (n < 1)
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "kernel cannot be resident on an SM");
  }
  return n;
}

inline int sm_count()
{
  CUdevice dev;
  check(cuCtxGetDevice(&dev), "cuCtxGetDevice");
  int n = 0;
  check(cuDeviceGetAttribute(&n, CU_DEVICE_ATTRIBUTE_MULTIPROCESSOR_COUNT, dev), "cuDeviceGetAttribute");
  return n;
}

inline char* dup_cstr(const std::string& s)
{
  char* p = new char[s.size() + 1];
  std::memcpy(p, s.c_str(), s.size() + 1);
  return p;
}

// ---- build-result blob: "GB3S" | version | algo | payload kind | cc | fields ... ----
constexpr uint32_t BLOB_MAGIC   = 0x53334247u; // "GB3S"
constexpr uint32_t BLOB_VERSION = 1u;

struct blob_writer
{
  std::vector<unsigned char> buf;
  void bytes(const void* p, size_t n)
  {
    const auto* c = static_cast<const unsigned char*>(p);
    buf.insert(buf.end(), c, c + n);
  }
  template <class T>
  void pod(const T& v)
  {
    bytes(&v, sizeof(T));
  }
  void blob(const void* p, size_t n)
  {
    pod<uint64_t>(n);
    bytes(p, n);
  }
  void cstr(const char* s)
  {
    const uint32_t n = s ? uint32_t(std::strlen(s)) : 0u;
    pod<uint32_t>(n);
    bytes(s, n);
  }
  void type_info(const cccl_type_info& t)
  {
    pod<uint64_t>(t.size);
    pod<uint64_t>(t.alignment);
    pod<uint32_t>(uint32_t(t.type));
  }
  void release(void** out, size_t* out_size)
  {
    void* p = std::malloc(buf.size());
    if (p == nullptr)
    {
      throw cuda_error(CUDA_ERROR_OUT_OF_MEMORY, "serialization buffer");
    }
    std::memcpy(p, buf.data(), buf.size());
    *out      = p;
    *out_size = buf.size();
  }
};

struct blob_reader
{
  const unsigned char* p;
  size_t left;
  void need(size_t n)
  {
    if (n > left)
    {
      throw cuda_error(CUDA_ERROR_INVALID_VALUE, "serialization blob: truncated");
    }
  }
  void bytes(void* out, size_t n)
  {
    need(n);
    std::memcpy(out, p, n);
    p += n;
    left -= n;
  }
  template <class T>
  T pod()
  {
    T v;
    bytes(&v, sizeof(T));
    return v;
  }
  void* blob_new(size_t* n)
  {
    const uint64_t sz = pod<uint64_t>();
    need(sz);
    char* out = new char[sz ? sz : 1];
    bytes(out, sz);
    *n = sz;
    return out;
  }
  char* cstr_new()
  {
    const uint32_t n = pod<uint32_t>();
    need(n);
    char* s = new char[n + 1];
    bytes(s, n);
    s[n] = '\0';
    return s;
  }
  cccl_type_info type_info()
  {
    cccl_type_info t{};
    t.size      = pod<uint64_t>();
    t.alignment = pod<uint64_t>();
    t.type      = cccl_type_enum(pod<uint32_t>());
    return t;
  }
};

inline void write_header(blob_writer& w, uint32_t algo, cccl_payload_kind_t kind, int cc)
{
  w.pod<uint32_t>(BLOB_MAGIC);
  w.pod<uint32_t>(BLOB_VERSION);
  w.pod<uint32_t>(algo);
  w.pod<uint32_t>(uint32_t(kind));
  w.pod<int32_t>(cc);
}

struct blob_header
{
  uint32_t payload_kind;
  int32_t cc;
};

inline blob_header read_header(blob_reader& r, uint32_t algo)
{
  if (r.pod<uint32_t>() != BLOB_MAGIC)
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "serialization blob: bad magic");
  }
  if (r.pod<uint32_t>() != BLOB_VERSION)
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "serialization blob: unsupported version");
  }
  if (r.pod<uint32_t>() != algo)
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "serialization blob: built for another algorithm");
  }
  blob_header h{};
  h.payload_kind = r.pod<uint32_t>();
  h.cc           = r.pod<int32_t>();
  if (h.payload_kind != CCCL_PAYLOAD_CUBIN)
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "serialization blob: payload is not a cubin");
  }
  return h;
}

// Prints the exception like the reference's ABI does and maps it to a CUresult.
inline CUresult report(const char* fn, const std::exception& e)
{
  fflush(stderr);
  printf("\nEXCEPTION in %s(): %s\n", fn, e.what());
  fflush(stdout);
  if (const auto* ce = dynamic_cast<const cuda_error*>(&e))
  {
    return ce->code;
  }
  return CUDA_ERROR_UNKNOWN;
}

inline size_t align_up(size_t x, size_t a)
{
  return (x + a - 1) / a * a;
}

} // namespace gb300
