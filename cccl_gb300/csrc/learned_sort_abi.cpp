// C ABI of the learned-partition sort: cccl_gb300_learned_sort_{build,stats,cleanup} and
// the run entry cccl_gb300_learned_sort (include/cccl_gb300/learned_sort.h). The run takes
// the arguments of cccl_device_radix_sort (c/parallel/src/radix_sort.cu:582-698) and
// rejects what it rejects: non-pointer iterators (CUDA_ERROR_UNKNOWN with a message),
// custom decomposers, a null selector or size pointer.
#include <cccl_gb300/learned_sort.h>

#include <memory>

#include "abi_common.h"
#include "learned_plan.h"
#include "sort_policy.h"

using namespace gb300;

namespace
{

constexpr uint32_t SETUP_MAGIC = 0x4c425047u; // "GPBL"

bool is_keys_only(const cccl_iterator_t& values)
{
  return values.type == CCCL_POINTER && values.state == nullptr;
}

bool has_decomposer(const cccl_op_t& op)
{
  return op.name != nullptr && op.name[0] != '\0';
}

CUkernel get_kernel(CUlibrary lib, const std::string& name)
{
  CUkernel k = nullptr;
  check(cuLibraryGetKernel(&k, lib, name.c_str()), name.c_str());
  return k;
}

const LearnedSetup& setup_of(const cccl_gb300_learned_sort_build_result_t& b)
{
  if (b.setup == nullptr || b.setup_size != sizeof(LearnedSetup)
      || static_cast<const LearnedSetup*>(b.setup)->magic != SETUP_MAGIC)
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "build result is not a learned-sort build");
  }
  return *static_cast<const LearnedSetup*>(b.setup);
}

void unload_all(cccl_gb300_learned_sort_build_result_t* b)
{
  for (CUlibrary* l : {&b->radix_library, &b->segmented_library, &b->learned_library})
  {
    if (*l != nullptr)
    {
      cuLibraryUnload(*l);
      *l = nullptr;
    }
  }
  std::free(b->setup);
  b->setup      = nullptr;
  b->setup_size = 0;
}

RadixCall make_call(const cccl_gb300_learned_sort_build_result_t& build,
                    void* d_temp_storage,
                    size_t* temp_storage_bytes,
                    const cccl_iterator_t& keys_in,
                    const cccl_iterator_t& keys_out,
                    const cccl_iterator_t& values_in,
                    const cccl_iterator_t& values_out,
                    uint64_t num_items,
                    int begin_bit,
                    int end_bit,
                    bool overwrite,
                    CUstream stream)
{
  RadixCall call{};
  call.keys[0]            = keys_in.state;
  call.keys[1]            = keys_out.state;
  call.values[0]          = values_in.state;
  call.values[1]          = values_out.state;
  call.num_items          = num_items;
  call.begin_bit          = begin_bit;
  call.end_bit            = end_bit;
  call.overwrite          = overwrite;
  call.descending         = build.order == CCCL_DESCENDING;
  call.d_temp_storage     = d_temp_storage;
  call.temp_storage_bytes = temp_storage_bytes;
  call.stream             = stream;
  return call;
}

bool all_pointers(const cccl_iterator_t& a, const cccl_iterator_t& b, const cccl_iterator_t& c, const cccl_iterator_t& d)
{
  return a.type == CCCL_POINTER && b.type == CCCL_POINTER && c.type == CCCL_POINTER && d.type == CCCL_POINTER;
}

} // namespace

extern "C" {

CCCL_GB300_API CUresult cccl_gb300_learned_sort_build(
  cccl_gb300_learned_sort_build_result_t* build,
  cccl_sort_order_t sort_order,
  cccl_iterator_t input_keys_it,
  cccl_iterator_t input_values_it,
  int cc_major,
  int cc_minor)
{
  if (build == nullptr || (sort_order != CCCL_ASCENDING && sort_order != CCCL_DESCENDING))
  {
    return CUDA_ERROR_INVALID_VALUE;
  }
  if (cc_major * 10 + cc_minor != 103)
  {
    printf("\nERROR in cccl_gb300_learned_sort_build(): kernels are built for sm_103a only (requested %d.%d)\n",
           cc_major,
           cc_minor);
    return CUDA_ERROR_NOT_SUPPORTED;
  }
  int kind = 0, kb = 0;
  if (!key_kind_of(input_keys_it.value_type.type, kind, kb) || input_keys_it.value_type.size != size_t(kb)
      || (kb != 4 && kb != 8))
  {
    printf("\nERROR in cccl_gb300_learned_sort_build(): keys must be 4- or 8-byte integers or floats\n");
    return CUDA_ERROR_NOT_SUPPORTED;
  }
  const size_t vb = is_keys_only(input_values_it) ? 0 : input_values_it.value_type.size;
  if (!(vb == 0 || vb == 4 || vb == 8))
  {
    printf("\nERROR in cccl_gb300_learned_sort_build(): value size %zu is not supported (0, 4 or 8)\n", vb);
    return CUDA_ERROR_NOT_SUPPORTED;
  }
  cccl_gb300_learned_sort_build_result_t r{};
  try
  {
    context_guard ctx;
    auto* s = static_cast<LearnedSetup*>(std::calloc(1, sizeof(LearnedSetup)));
    if (s == nullptr)
    {
      return CUDA_ERROR_OUT_OF_MEMORY;
    }
    r.setup       = s;
    r.setup_size  = sizeof(LearnedSetup);
    r.cc          = cc_major * 10 + cc_minor;
    r.key_type    = input_keys_it.value_type;
    r.value_type  = input_values_it.value_type;
    r.order       = sort_order;
    s->magic       = SETUP_MAGIC;
    s->key_bytes   = kb;
    s->value_bytes = int(vb);
    s->key_kind    = kind;
    s->pass_tpb    = persistent_tpb(kb, int(vb));
    s->pass_items  = learned_items(kb, int(vb));
    s->pass_smem   = learned_pass_smem(kb, int(vb));
    s->route_policy = LEARNED_POLICY_COST_MODEL;

    auto load = [](CUlibrary* lib, const image_ref& img) {
      check(cuLibraryLoadData(lib, img.data, nullptr, nullptr, 0, nullptr, nullptr, 0), "cuLibraryLoadData");
    };
    load(&r.radix_library, radix_image(kb));
    load(&r.segmented_library, segmented_image(kb));
    load(&r.learned_library, learned_image(kb));

    auto radix = [&](int rvb, int rkind, RadixPolicy& pol, RadixKernels& ks) {
      pol                       = make_radix_policy(kb, rvb, rkind);
      const RadixKernelNames nm = radix_kernel_names(kb, rvb, rkind, rkind == KIND_FLOAT && sort_order == CCCL_DESCENDING);
      ks.init                   = get_kernel(r.radix_library, nm.init);
      ks.histogram              = get_kernel(r.radix_library, nm.histogram);
      ks.onesweep               = get_kernel(r.radix_library, nm.onesweep);
      ks.onesweep_first         = get_kernel(r.radix_library, nm.onesweep_first);
      ks.onesweep_dyn           = get_kernel(r.radix_library, nm.onesweep_dyn);
      ks.single_tile            = get_kernel(r.radix_library, nm.single_tile);
    };
    radix(int(vb), kind, s->plain_pol, s->plain_ks);
    radix(0, KIND_UNSIGNED, s->sample_pol, s->sample_ks);

    s->seg_pol = make_segmented_policy(kb, int(vb), kind);
    char names[SK_COUNT][64];
    segmented_kernel_names(kb, int(vb), kind, sort_order == CCCL_DESCENDING, names);
    for (int i = 0; i < SK_COUNT; ++i)
    {
      s->seg_ks.k[i] = get_kernel(r.segmented_library, names[i]);
    }

    const std::string k  = std::to_string(kb);
    const std::string fs = kind == KIND_FLOAT ? "f" : "i";
    s->lk.init   = get_kernel(r.learned_library, "gb300_init");
    s->lk.status_fold = get_kernel(r.learned_library, "gb300_status_fold");
    s->lk.sample = get_kernel(r.learned_library, "gb300_learned_sample_k" + k + "_" + fs);
    s->lk.fit    = get_kernel(r.learned_library, "gb300_learned_fit_k" + k);
    s->lk.cells  = get_kernel(r.learned_library, "gb300_learned_cells_k" + k);
    s->lk.route  = get_kernel(r.learned_library, "gb300_learned_route_k" + k + "_" + fs);
    s->lk.hist   = get_kernel(r.learned_library, "gb300_learned_hist_k" + k + "_" + fs);
    s->lk.pass   = get_kernel(r.learned_library, "gb300_learned_pass_k" + k + "_v" + std::to_string(vb) + "_" + fs);
    s->lk.bounds = get_kernel(r.learned_library, "gb300_learned_bounds_k" + k + "_" + fs);
    const std::string kvf = "_k" + k + "_v" + std::to_string(vb) + "_" + fs;
    s->lk.bucket4k        = get_kernel(r.learned_library, "gb300_learned_bucket4096" + kvf);
    s->lk.bucket8k        = get_kernel(r.learned_library, "gb300_learned_bucket8192" + kvf);
    *build = r;
    return CUDA_SUCCESS;
  }
  catch (const std::exception& e)
  {
    unload_all(&r);
    return report("cccl_gb300_learned_sort_build", e);
  }
}

CCCL_GB300_API CUresult cccl_gb300_learned_sort(
  cccl_gb300_learned_sort_build_result_t build,
  void* d_temp_storage,
  size_t* temp_storage_bytes,
  cccl_iterator_t d_keys_in,
  cccl_iterator_t d_keys_out,
  cccl_iterator_t d_values_in,
  cccl_iterator_t d_values_out,
  cccl_op_t decomposer,
  uint64_t num_items,
  int begin_bit,
  int end_bit,
  bool is_overwrite_okay,
  int* selector,
  CUstream stream)
{
  if (!all_pointers(d_keys_in, d_keys_out, d_values_in, d_values_out))
  {
    fflush(stderr);
    printf("\nERROR in cccl_gb300_learned_sort(): radix sort input must be a pointer\n");
    fflush(stdout);
    return CUDA_ERROR_UNKNOWN;
  }
  if (temp_storage_bytes == nullptr || selector == nullptr)
  {
    return CUDA_ERROR_INVALID_VALUE;
  }
  if (has_decomposer(decomposer))
  {
    return CUDA_ERROR_NOT_SUPPORTED;
  }
  try
  {
    context_guard ctx;
    const LearnedSetup& s = setup_of(build);
    const RadixCall call  = make_call(build, d_temp_storage, temp_storage_bytes, d_keys_in, d_keys_out, d_values_in,
                                     d_values_out, num_items, begin_bit, end_bit, is_overwrite_okay, stream);
    int sel = 0;
    learned_sort_dispatch(s, call, &sel);
    *selector = sel;
    return CUDA_SUCCESS;
  }
  catch (const std::exception& e)
  {
    return report("cccl_gb300_learned_sort", e);
  }
}

CCCL_GB300_API CUresult cccl_gb300_learned_sort_stats(
  cccl_gb300_learned_sort_build_result_t build,
  void* d_temp_storage,
  cccl_iterator_t d_keys_in,
  cccl_iterator_t d_keys_out,
  cccl_iterator_t d_values_in,
  cccl_iterator_t d_values_out,
  uint64_t num_items,
  int begin_bit,
  int end_bit,
  bool is_overwrite_okay,
  cccl_gb300_learned_sort_stats_t* stats)
{
  if (stats == nullptr || !all_pointers(d_keys_in, d_keys_out, d_values_in, d_values_out))
  {
    return CUDA_ERROR_INVALID_VALUE;
  }
  try
  {
    context_guard ctx;
    const LearnedSetup& s = setup_of(build);
    const RadixCall call  = make_call(build, d_temp_storage, nullptr, d_keys_in, d_keys_out, d_values_in, d_values_out,
                                     num_items, begin_bit, end_bit, is_overwrite_okay, nullptr);
    const LearnedStats st = learned_sort_stats(s, call);
    stats->learned          = st.learned;
    stats->bucket_log2      = st.bucket_log2;
    stats->partition_passes = st.partition_passes;
    stats->block_buckets    = st.block_buckets;
    stats->device_buckets   = st.device_buckets;
    stats->device_items     = st.device_items;
    return CUDA_SUCCESS;
  }
  catch (const std::exception& e)
  {
    return report("cccl_gb300_learned_sort_stats", e);
  }
}

CCCL_GB300_API CUresult cccl_gb300_learned_sort_set_route(cccl_gb300_learned_sort_build_result_t* build, int route)
{
  if (build == nullptr || build->setup == nullptr || build->setup_size != sizeof(LearnedSetup)
      || (route != CCCL_GB300_LEARNED_ROUTE_COST_MODEL && route != CCCL_GB300_LEARNED_ROUTE_ALWAYS))
  {
    return CUDA_ERROR_INVALID_VALUE;
  }
  auto* s = static_cast<LearnedSetup*>(build->setup);
  if (s->magic != SETUP_MAGIC)
  {
    return CUDA_ERROR_INVALID_VALUE;
  }
  s->route_policy = route == CCCL_GB300_LEARNED_ROUTE_ALWAYS ? LEARNED_POLICY_ALWAYS : LEARNED_POLICY_COST_MODEL;
  return CUDA_SUCCESS;
}

CCCL_GB300_API CUresult cccl_gb300_learned_sort_cleanup(cccl_gb300_learned_sort_build_result_t* build)
{
  if (build == nullptr)
  {
    return CUDA_ERROR_INVALID_VALUE;
  }
  try
  {
    context_guard ctx;
    unload_all(build);
    return CUDA_SUCCESS;
  }
  catch (const std::exception& e)
  {
    return report("cccl_gb300_learned_sort_cleanup", e);
  }
}

} // extern "C"
