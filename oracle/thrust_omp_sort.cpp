// The reference library's own CPU sort, timed as the CPU baseline: thrust::sort /
// thrust::sort_by_key on thrust's OpenMP backend (thrust/thrust/system/omp/detail/sort.h
// in the reference tree: per-thread sequential radix sort of a uniform decomposition,
// then pairwise merges). Built with g++ -fopenmp against the thrust headers of the CUDA
// toolkit on the machine (CCCL, the same library as the reference); no GPU is involved.
// TEST/BENCH INFRASTRUCTURE ONLY. It is a timing baseline, not a bit-exact oracle:
// its -0.0/+0.0 order and descending stability differ from cub::DeviceRadixSort.
#include <thrust/functional.h>
#include <thrust/sort.h>
#include <thrust/system/omp/execution_policy.h>

#include <cstdint>

#include <omp.h>

namespace
{
template <class K, class V>
int sort_impl(K* keys, V* values, uint64_t n, int descending)
{
  if (values == nullptr)
  {
    if (descending)
    {
      thrust::sort(thrust::omp::par, keys, keys + n, thrust::greater<K>());
    }
    else
    {
      thrust::sort(thrust::omp::par, keys, keys + n);
    }
  }
  else
  {
    if (descending)
    {
      thrust::sort_by_key(thrust::omp::par, keys, keys + n, values, thrust::greater<K>());
    }
    else
    {
      thrust::sort_by_key(thrust::omp::par, keys, keys + n, values);
    }
  }
  return 0;
}

template <class K>
int by_value(void* k, void* v, uint64_t vb, uint64_t n, int desc)
{
  switch (vb)
  {
    case 0:
      return sort_impl<K, uint32_t>(static_cast<K*>(k), nullptr, n, desc);
    case 4:
      return sort_impl<K, uint32_t>(static_cast<K*>(k), static_cast<uint32_t*>(v), n, desc);
    case 8:
      return sort_impl<K, uint64_t>(static_cast<K*>(k), static_cast<uint64_t*>(v), n, desc);
    default:
      return 2;
  }
}
} // namespace

extern "C" {

// In-place sort. key_type uses the cccl_type_enum codes; value_bytes 0, 4 or 8.
int thrust_omp_sort(int key_type, void* keys, uint64_t value_bytes, void* values, uint64_t n, int descending, int threads)
{
  if (threads > 0)
  {
    omp_set_num_threads(threads);
  }
  switch (key_type)
  {
    case 2:
      return by_value<int32_t>(keys, values, value_bytes, n, descending);
    case 3:
      return by_value<int64_t>(keys, values, value_bytes, n, descending);
    case 6:
      return by_value<uint32_t>(keys, values, value_bytes, n, descending);
    case 7:
      return by_value<uint64_t>(keys, values, value_bytes, n, descending);
    case 9:
      return by_value<float>(keys, values, value_bytes, n, descending);
    case 10:
      return by_value<double>(keys, values, value_bytes, n, descending);
    default:
      return 1;
  }
}

int thrust_omp_max_threads()
{
  return omp_get_max_threads();
}
}
