// Segment offsets given as iterators (offset_iterators.h).
#include "offset_iterators.h"

#include <dlfcn.h>

#include <cctype>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "abi_common.h"

namespace gb300
{

namespace
{

// The few NVRTC and nvJitLink entry points used, opened once with dlopen (so the library
// needs neither unless a caller passes iterator offsets).
struct JitApi
{
  int (*nvrtcCreateProgram)(void**, const char*, const char*, int, const char* const*, const char* const*);
  int (*nvrtcCompileProgram)(void*, int, const char* const*);
  int (*nvrtcGetProgramLogSize)(void*, size_t*);
  int (*nvrtcGetProgramLog)(void*, char*);
  int (*nvrtcGetCUBINSize)(void*, size_t*);
  int (*nvrtcGetCUBIN)(void*, char*);
  int (*nvrtcGetLTOIRSize)(void*, size_t*);
  int (*nvrtcGetLTOIR)(void*, char*);
  int (*nvrtcDestroyProgram)(void**);
  int (*nvJitLinkCreate)(void**, uint32_t, const char**);
  int (*nvJitLinkAddData)(void*, int, const void*, size_t, const char*);
  int (*nvJitLinkComplete)(void*);
  int (*nvJitLinkGetLinkedCubinSize)(void*, size_t*);
  int (*nvJitLinkGetLinkedCubin)(void*, void*);
  int (*nvJitLinkGetErrorLogSize)(void*, size_t*);
  int (*nvJitLinkGetErrorLog)(void*, char*);
  int (*nvJitLinkDestroy)(void**);
  bool nvrtc_ok = false;
  bool link_ok  = false;
};

void* open_first(const char* const* names)
{
  for (const char* const* n = names; *n != nullptr; ++n)
  {
    if (void* h = dlopen(*n, RTLD_NOW | RTLD_LOCAL))
    {
      return h;
    }
  }
  return nullptr;
}

const JitApi& jit_api()
{
  static JitApi api{};
  static std::once_flag once;
  std::call_once(once, [] {
    const char* nvrtc_names[] = {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13", nullptr};
    const char* link_names[]  = {"libnvJitLink.so.13", "libnvJitLink.so", "/usr/local/cuda/lib64/libnvJitLink.so.13",
                                 nullptr};
    if (void* h = open_first(nvrtc_names))
    {
      bool ok = true;
      auto sym = [&](auto& fn, const char* name) {
        fn = reinterpret_cast<std::remove_reference_t<decltype(fn)>>(dlsym(h, name));
        ok = ok && fn != nullptr;
      };
      sym(api.nvrtcCreateProgram, "nvrtcCreateProgram");
      sym(api.nvrtcCompileProgram, "nvrtcCompileProgram");
      sym(api.nvrtcGetProgramLogSize, "nvrtcGetProgramLogSize");
      sym(api.nvrtcGetProgramLog, "nvrtcGetProgramLog");
      sym(api.nvrtcGetCUBINSize, "nvrtcGetCUBINSize");
      sym(api.nvrtcGetCUBIN, "nvrtcGetCUBIN");
      sym(api.nvrtcGetLTOIRSize, "nvrtcGetLTOIRSize");
      sym(api.nvrtcGetLTOIR, "nvrtcGetLTOIR");
      sym(api.nvrtcDestroyProgram, "nvrtcDestroyProgram");
      api.nvrtc_ok = ok;
    }
    if (void* h = open_first(link_names))
    {
      bool ok = true;
      auto sym = [&](auto& fn, const char* name) {
        fn = reinterpret_cast<std::remove_reference_t<decltype(fn)>>(dlsym(h, name));
        ok = ok && fn != nullptr;
      };
      sym(api.nvJitLinkCreate, "nvJitLinkCreate");
      sym(api.nvJitLinkAddData, "nvJitLinkAddData");
      sym(api.nvJitLinkComplete, "nvJitLinkComplete");
      sym(api.nvJitLinkGetLinkedCubinSize, "nvJitLinkGetLinkedCubinSize");
      sym(api.nvJitLinkGetLinkedCubin, "nvJitLinkGetLinkedCubin");
      sym(api.nvJitLinkGetErrorLogSize, "nvJitLinkGetErrorLogSize");
      sym(api.nvJitLinkGetErrorLog, "nvJitLinkGetErrorLog");
      sym(api.nvJitLinkDestroy, "nvJitLinkDestroy");
      api.link_ok = ok;
    }
  });
  return api;
}

constexpr int NVJITLINK_INPUT_LTOIR = 3; // nvJitLinkInputType (nvJitLink.h)

const char* offset_type_name(cccl_type_enum t)
{
  switch (t)
  {
    case CCCL_INT32:
      return "int";
    case CCCL_UINT32:
      return "unsigned int";
    case CCCL_INT64:
      return "long long";
    case CCCL_UINT64:
      return "unsigned long long";
    default:
      return nullptr;
  }
}

bool valid_name(const char* s)
{
  if (s == nullptr || *s == '\0')
  {
    return false;
  }
  for (const char* c = s; *c; ++c)
  {
    if (!(std::isalnum(static_cast<unsigned char>(*c)) || *c == '_'))
    {
      return false;
    }
  }
  return true;
}

std::string program_log(const JitApi& api, void* prog)
{
  size_t n = 0;
  api.nvrtcGetProgramLogSize(prog, &n);
  std::string log(n, '\0');
  if (n > 0)
  {
    api.nvrtcGetProgramLog(prog, log.data());
  }
  return log;
}

} // namespace

namespace
{

// NVRTC program -> LTO-IR for sm_<arch>a; throws with the compiler's log.
std::vector<char> source_to_ltoir(const JitApi& api, const std::string& src, const char* name, const std::string& arch)
{
  void* prog = nullptr;
  if (api.nvrtcCreateProgram(&prog, src.c_str(), name, 0, nullptr, nullptr) != 0)
  {
    throw cuda_error(CUDA_ERROR_UNKNOWN, "nvrtcCreateProgram failed");
  }
  const char* opts[] = {arch.c_str(), "-dlto", "-rdc=true"};
  if (api.nvrtcCompileProgram(prog, 3, opts) != 0)
  {
    const std::string log = program_log(api, prog);
    api.nvrtcDestroyProgram(&prog);
    throw cuda_error(CUDA_ERROR_INVALID_SOURCE, std::string("compilation of ") + name + " failed: " + log);
  }
  size_t n = 0;
  api.nvrtcGetLTOIRSize(prog, &n);
  std::vector<char> ltoir(n);
  api.nvrtcGetLTOIR(prog, ltoir.data());
  api.nvrtcDestroyProgram(&prog);
  return ltoir;
}

} // namespace

bool has_code(const cccl_op_t& op)
{
  return op.code != nullptr && (op.code_size > 0 || op.code[0] != '\0');
}

void compile_offset_iterator(
  const cccl_iterator_t& it_in, const cccl_iterator_t* sibling, int cc_major, int cc_minor, OffsetIteratorKernel& out)
{
  out = OffsetIteratorKernel{};
  // an operation given by name only takes its code from the sibling iterator's operation of
  // the same name (the end offsets are often the begin iterator's type, state advanced by one)
  cccl_iterator_t it = it_in;
  for (cccl_op_t* op : {&it.advance, &it.dereference})
  {
    if (!has_code(*op) && sibling != nullptr && sibling->type == CCCL_ITERATOR && op->name != nullptr)
    {
      for (const cccl_op_t* sop : {&sibling->advance, &sibling->dereference})
      {
        if (has_code(*sop) && sop->name != nullptr && std::strcmp(sop->name, op->name) == 0)
        {
          *op = *sop;
        }
      }
    }
  }
  const char* vt = offset_type_name(it.value_type.type);
  const size_t vsize = (it.value_type.type == CCCL_INT32 || it.value_type.type == CCCL_UINT32) ? 4u : 8u;
  if (it.type != CCCL_ITERATOR || vt == nullptr || it.value_type.size != vsize)
  {
    throw cuda_error(CUDA_ERROR_NOT_SUPPORTED, "offset iterators must yield 32- or 64-bit integers");
  }
  if (!valid_name(it.advance.name) || !valid_name(it.dereference.name) || !has_code(it.advance)
      || !has_code(it.dereference) || it.size == 0 || it.size > MAX_OFFSET_STATE_BYTES || it.alignment == 0
      || it.alignment > 16 || (it.alignment & (it.alignment - 1)) != 0 || it.size % it.alignment != 0)
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "offset iterator without named advance/dereference code or state");
  }
  const JitApi& api = jit_api();
  if (!api.nvrtc_ok || !api.link_ok)
  {
    throw cuda_error(CUDA_ERROR_NOT_SUPPORTED,
                     "iterator offsets need NVRTC and nvJitLink (libnvrtc.so.13, libnvJitLink.so.13), which are not available");
  }
  const std::string arch = "-arch=sm_" + std::to_string(cc_major) + std::to_string(cc_minor) + "a";
  // the evaluation kernel, declaring the operations with the prototypes the reference's
  // iterator mapping uses; each operation is a separate LTO-IR module (a C++ source is
  // compiled alone, as its own translation unit, since it carries its own state struct)
  const std::string kernel =
    "extern \"C\" __device__ void " + std::string(it.advance.name) + "(void*, const void*);\n"
    + "extern \"C\" __device__ void " + std::string(it.dereference.name) + "(const void*, void*);\n"
    + "struct __align__(" + std::to_string(it.alignment) + ") gb300_offset_state { char data["
    + std::to_string(it.size) + "]; };\n"
    + "extern \"C\" __global__ void __launch_bounds__(256) gb300_evaluate_offsets(gb300_offset_state st, "
      "unsigned long long n, " + vt + "* out)\n{\n"
      "  const unsigned long long i = blockIdx.x * 256ull + threadIdx.x;\n"
      "  if (i < n)\n  {\n"
      "    gb300_offset_state s = st;\n"
      "    unsigned long long d = i;\n    "
    + std::string(it.advance.name) + "(&s, &d);\n    " + vt + " v;\n    " + std::string(it.dereference.name)
    + "(&s, &v);\n    out[i] = v;\n  }\n}\n";
  std::vector<std::vector<char>> modules;
  std::vector<std::string> module_names;
  modules.push_back(source_to_ltoir(api, kernel, "gb300_offsets.cu", arch));
  module_names.emplace_back("gb300_offsets");
  const cccl_op_t* ops[] = {&it.advance, &it.dereference};
  for (int o = 0; o < 2; ++o)
  {
    const cccl_op_t* op = ops[o];
    if (o == 1 && op->code == ops[0]->code && op->code_type == ops[0]->code_type)
    {
      continue; // one module holding both operations
    }
    if (op->code_type == CCCL_OP_CPP_SOURCE)
    {
      const std::string src(op->code, op->code_size ? op->code_size : std::strlen(op->code));
      modules.push_back(source_to_ltoir(api, src, op->name, arch));
    }
    else if (op->code_type == CCCL_OP_LTOIR && op->code_size > 0)
    {
      modules.emplace_back(op->code, op->code + op->code_size);
    }
    else
    {
      throw cuda_error(CUDA_ERROR_INVALID_VALUE, "iterator operation without code");
    }
    module_names.emplace_back(op->name);
    for (size_t e = 0; e < op->num_extra_ltoirs; ++e)
    {
      if (op->extra_ltoirs == nullptr || op->extra_ltoir_sizes == nullptr || op->extra_ltoirs[e] == nullptr)
      {
        throw cuda_error(CUDA_ERROR_INVALID_VALUE, "iterator operation: missing extra LTO-IR");
      }
      if (op->extra_code_types != nullptr && op->extra_code_types[e] == CCCL_OP_CPP_SOURCE)
      {
        const std::string src(op->extra_ltoirs[e], op->extra_ltoir_sizes[e]);
        modules.push_back(source_to_ltoir(api, src, op->name, arch));
      }
      else
      {
        modules.emplace_back(op->extra_ltoirs[e], op->extra_ltoirs[e] + op->extra_ltoir_sizes[e]);
      }
      module_names.emplace_back(op->name);
    }
  }
  const char* lopts[] = {arch.c_str(), "-lto"};
  void* h             = nullptr;
  if (api.nvJitLinkCreate(&h, 2, lopts) != 0)
  {
    throw cuda_error(CUDA_ERROR_UNKNOWN, "nvJitLinkCreate failed");
  }
  auto fail = [&](const std::string& what) {
    size_t ln = 0;
    api.nvJitLinkGetErrorLogSize(h, &ln);
    std::string log(ln, '\0');
    if (ln > 0)
    {
      api.nvJitLinkGetErrorLog(h, log.data());
    }
    api.nvJitLinkDestroy(&h);
    throw cuda_error(CUDA_ERROR_INVALID_SOURCE, what + ": " + log);
  };
  for (size_t m = 0; m < modules.size(); ++m)
  {
    if (api.nvJitLinkAddData(h, NVJITLINK_INPUT_LTOIR, modules[m].data(), modules[m].size(), module_names[m].c_str())
        != 0)
    {
      fail("nvJitLinkAddData(" + module_names[m] + ")");
    }
  }
  if (api.nvJitLinkComplete(h) != 0)
  {
    fail("nvJitLinkComplete");
  }
  size_t n = 0;
  api.nvJitLinkGetLinkedCubinSize(h, &n);
  out.cubin = std::malloc(n);
  if (out.cubin == nullptr)
  {
    api.nvJitLinkDestroy(&h);
    throw cuda_error(CUDA_ERROR_OUT_OF_MEMORY, "offset iterator image");
  }
  api.nvJitLinkGetLinkedCubin(h, out.cubin);
  api.nvJitLinkDestroy(&h);
  out.cubin_size      = n;
  out.state_size      = it.size;
  out.state_alignment = it.alignment;
  out.value_size      = vsize;
}

void load_offset_iterator(OffsetIteratorKernel& k)
{
  if (k.cubin == nullptr || k.library != nullptr)
  {
    return;
  }
  check(cuLibraryLoadData(&k.library, k.cubin, nullptr, nullptr, 0, nullptr, nullptr, 0), "cuLibraryLoadData(offsets)");
  check(cuLibraryGetKernel(&k.kernel, k.library, "gb300_evaluate_offsets"), "cuLibraryGetKernel(gb300_evaluate_offsets)");
}

void free_offset_iterator(OffsetIteratorKernel& k)
{
  if (k.library != nullptr)
  {
    cuLibraryUnload(k.library);
  }
  std::free(k.cubin);
  k = OffsetIteratorKernel{};
}

void evaluate_offset_iterator(
  const OffsetIteratorKernel& k, const cccl_iterator_t& it, uint64_t n, void* out, CUstream stream)
{
  if (k.kernel == nullptr)
  {
    throw cuda_error(CUDA_ERROR_NOT_INITIALIZED, "offset iterator kernel not loaded");
  }
  if (it.type != CCCL_ITERATOR || it.size != k.state_size || it.state == nullptr)
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "offset iterator differs from the one the build compiled");
  }
  if (n == 0)
  {
    return;
  }
  // the state travels by value: copy it into a buffer with the state's alignment
  alignas(16) unsigned char state[MAX_OFFSET_STATE_BYTES];
  std::memcpy(state, it.state, size_t(k.state_size));
  unsigned long long nn = n;
  void* args[]          = {state, &nn, &out};
  CUfunction f          = nullptr;
  check(cuKernelGetFunction(&f, k.kernel), "cuKernelGetFunction(offsets)");
  if ((n + 255) / 256 > 0x7fffffffull)
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "too many segments");
  }
  const unsigned grid = unsigned((n + 255) / 256);
  notify_launch("segment_offsets", 0, stream);
  check(cuLaunchKernel(f, grid, 1, 1, 256, 1, 1, 0, stream, args, nullptr), "cuLaunchKernel(offsets)");
  notify_launch("segment_offsets", 1, stream);
}

} // namespace gb300
