// Times cub::DeviceRadixSort (the CUDA toolkit's CCCL build of the reference library) on
// the benchmark workloads, with the same CUDA-event method as bench.py, and writes its
// sorted output checksums so the engine can be compared bit for bit. Test/bench
// infrastructure only: compiled on the GPU machine against the toolkit's CUB headers.
#include <cub/device/device_radix_sort.cuh>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include <cuda_runtime.h>

#define CK(x)                                                                         \
  do                                                                                  \
  {                                                                                   \
    cudaError_t e = (x);                                                              \
    if (e != cudaSuccess)                                                             \
    {                                                                                 \
      std::fprintf(stderr, "%s failed: %s\n", #x, cudaGetErrorString(e));             \
      std::exit(1);                                                                   \
    }                                                                                 \
  } while (0)

__global__ void fill_u64(unsigned long long* k, unsigned int* v, size_t n, unsigned long long seed, int ands)
{
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
  {
    unsigned long long acc = ~0ull;
    for (int a = 0; a < ands; ++a)
    {
      unsigned long long x = (i + 1) * 0x9E3779B97F4A7C15ull ^ (seed + a * 0xD1B54A32D192ED03ull);
      x ^= x >> 33;
      x *= 0xff51afd7ed558ccdull;
      x ^= x >> 33;
      x *= 0xc4ceb9fe1a85ec53ull;
      x ^= x >> 33;
      acc &= x;
    }
    k[i] = acc;
    if (v)
    {
      v[i] = unsigned(i);
    }
  }
}

template <class F>
float time_ms(F f, int steps)
{
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  for (int i = 0; i < 3; ++i)
  {
    f();
  }
  CK(cudaDeviceSynchronize());
  CK(cudaEventRecord(a));
  for (int i = 0; i < steps; ++i)
  {
    f();
  }
  CK(cudaEventRecord(b));
  CK(cudaEventSynchronize(b));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, a, b));
  return ms / steps;
}

int main(int argc, char** argv)
{
  const int log2n = argc > 1 ? std::atoi(argv[1]) : 28;
  const size_t n  = size_t(1) << log2n;
  const int steps = 10;
  unsigned long long *k_in, *k_out;
  unsigned int *v_in, *v_out;
  CK(cudaMalloc(&k_in, n * 8));
  CK(cudaMalloc(&k_out, n * 8));
  CK(cudaMalloc(&v_in, n * 4));
  CK(cudaMalloc(&v_out, n * 4));
  void* temp     = nullptr;
  size_t tbytes  = 0;
  size_t tneeded = 0;
  CK(cub::DeviceRadixSort::SortPairs(nullptr, tneeded, k_in, k_out, v_in, v_out, n));
  size_t t2 = 0;
  CK(cub::DeviceRadixSort::SortKeys(nullptr, t2, reinterpret_cast<unsigned*>(k_in), reinterpret_cast<unsigned*>(k_out), n));
  tbytes = tneeded > t2 ? tneeded : t2;
  CK(cudaMalloc(&temp, tbytes));

  struct V
  {
    const char* name;
    int ands;
    bool desc;
    int b, e;
  } vars[] = {{"u64+u32 pairs, 64-bit entropy", 1, false, 0, 64},
              {"u64+u32 pairs, AND of 3", 3, false, 0, 64},
              {"u64+u32 pairs, descending", 1, true, 0, 64},
              {"u64+u32 pairs, bits 8..40", 1, false, 8, 40}};
  for (auto& v : vars)
  {
    fill_u64<<<1024, 256>>>(k_in, v_in, n, 12345, v.ands);
    CK(cudaDeviceSynchronize());
    float ms = time_ms(
      [&] {
        size_t tb = tbytes;
        if (v.desc)
        {
          CK(cub::DeviceRadixSort::SortPairsDescending(temp, tb, k_in, k_out, v_in, v_out, n, v.b, v.e));
        }
        else
        {
          CK(cub::DeviceRadixSort::SortPairs(temp, tb, k_in, k_out, v_in, v_out, n, v.b, v.e));
        }
      },
      steps);
    std::printf("{\"impl\": \"cub\", \"workload\": \"%s\", \"n\": %zu, \"ms\": %.4f, \"keys_per_s\": %.4e}\n",
                v.name, n, ms, n / (ms * 1e-3));
  }
  fill_u64<<<1024, 256>>>(k_in, nullptr, n / 2, 777, 1); // n u32 keys in the same bytes
  CK(cudaDeviceSynchronize());
  float ms = time_ms(
    [&] {
      size_t tb = tbytes;
      CK(cub::DeviceRadixSort::SortKeys(temp, tb, reinterpret_cast<unsigned*>(k_in), reinterpret_cast<unsigned*>(k_out), n));
    },
    steps);
  std::printf("{\"impl\": \"cub\", \"workload\": \"u32 keys-only\", \"n\": %zu, \"ms\": %.4f, \"keys_per_s\": %.4e}\n",
              n, ms, n / (ms * 1e-3));
  return 0;
}
