// Runs cub::DeviceSegmentedSort::StableSortPairs(Descending) from the CUDA toolkit's CCCL on
// binary inputs, to pin the segmented-sort oracle against CUB itself on the GPU machine.
// Test infrastructure only (compiled there by tests/test_cub_segmented_gpu.py).
//
// usage: cub_segmented <n> <num_segments> <descending> <in.bin> <out.bin> [timing reps]
//   in.bin  = n f32 keys, n i32 values, num_segments i32 begin offsets, num_segments i32 end offsets
//   out.bin = n f32 keys, n i32 values (positions outside segments keep the input)
#include <cub/device/device_segmented_sort.cuh>

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <vector>

#define CK(x)                                                               \
  do                                                                        \
  {                                                                         \
    cudaError_t err_ = (x);                                                 \
    if (err_ != cudaSuccess)                                                \
    {                                                                       \
      std::fprintf(stderr, "%s: %s\n", #x, cudaGetErrorString(err_));       \
      return 1;                                                             \
    }                                                                       \
  } while (0)

int main(int argc, char** argv)
{
  if (argc != 6 && argc != 7)
  {
    return 2;
  }
  const int reps = argc == 7 ? std::atoi(argv[6]) : 0;
  const long n    = std::atol(argv[1]);
  const long nseg = std::atol(argv[2]);
  const bool desc = std::atoi(argv[3]) != 0;
  std::ifstream in(argv[4], std::ios::binary);
  std::vector<float> keys(n);
  std::vector<int> vals(n), b(nseg), e(nseg);
  in.read(reinterpret_cast<char*>(keys.data()), n * 4);
  in.read(reinterpret_cast<char*>(vals.data()), n * 4);
  in.read(reinterpret_cast<char*>(b.data()), nseg * 4);
  in.read(reinterpret_cast<char*>(e.data()), nseg * 4);
  float *ki, *ko;
  int *vi, *vo, *db, *de;
  CK(cudaMalloc(&ki, n * 4));
  CK(cudaMalloc(&ko, n * 4));
  CK(cudaMalloc(&vi, n * 4));
  CK(cudaMalloc(&vo, n * 4));
  CK(cudaMalloc(&db, nseg * 4));
  CK(cudaMalloc(&de, nseg * 4));
  CK(cudaMemcpy(ki, keys.data(), n * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ko, keys.data(), n * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(vi, vals.data(), n * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(vo, vals.data(), n * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(db, b.data(), nseg * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(de, e.data(), nseg * 4, cudaMemcpyHostToDevice));
  size_t bytes = 0;
  void* temp   = nullptr;
  for (int pass = 0; pass < 2; ++pass)
  {
    if (desc)
    {
      CK(cub::DeviceSegmentedSort::StableSortPairsDescending(temp, bytes, ki, ko, vi, vo, n, nseg, db, de));
    }
    else
    {
      CK(cub::DeviceSegmentedSort::StableSortPairs(temp, bytes, ki, ko, vi, vo, n, nseg, db, de));
    }
    if (pass == 0)
    {
      CK(cudaMalloc(&temp, bytes));
    }
  }
  CK(cudaDeviceSynchronize());
  if (reps > 0)
  {
    cudaEvent_t a, z;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&z));
    CK(cudaEventRecord(a));
    for (int r = 0; r < reps; ++r)
    {
      CK(desc ? cub::DeviceSegmentedSort::StableSortPairsDescending(temp, bytes, ki, ko, vi, vo, n, nseg, db, de)
              : cub::DeviceSegmentedSort::StableSortPairs(temp, bytes, ki, ko, vi, vo, n, nseg, db, de));
    }
    CK(cudaEventRecord(z));
    CK(cudaEventSynchronize(z));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, a, z));
    std::printf("{\"impl\": \"cub\", \"ms\": %.4f}\n", ms / reps);
  }
  CK(cudaMemcpy(keys.data(), ko, n * 4, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(vals.data(), vo, n * 4, cudaMemcpyDeviceToHost));
  std::ofstream out(argv[5], std::ios::binary);
  out.write(reinterpret_cast<const char*>(keys.data()), n * 4);
  out.write(reinterpret_cast<const char*>(vals.data()), n * 4);
  return 0;
}
