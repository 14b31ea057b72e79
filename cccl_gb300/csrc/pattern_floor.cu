// Memory-pattern floor of a digit pass (measurement only; not part of the sort library).
//
// A stable 8-bit digit pass reads a tile, stages it in shared memory in digit order and writes
// every digit's run of the tile to that digit's region of the output. These kernels keep the
// pass's launch shape (one CTA per SM walking tiles blockIdx.x, blockIdx.x + gridDim.x, ...),
// its tile (the persistent pass's main threads x items per thread, from sort_policy.h) and its
// write-out address computation (digit of the staged slot, the digit's per-tile delta in shared
// memory, a bounds-checked streaming store), and leave out the ranking and the look-back:
//   runs = 1:   the staged tile is written back to its own place (contiguous stores);
//   runs = R:   slot s of the staged tile belongs to run r(s), the R runs' lengths being the same
//               in every tile (TILE / R each, the remainder spread); tile t's run r goes to r's
//               region at offset t * len(r) (+ shift keys), the write pattern of a pass over
//               uniform keys when R = 256.
// The time with 256 runs is what the pass's access pattern costs before any ranking work; the
// difference to one run is what the runs' partially written 32-byte sectors cost.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>

#include "sort_policy.h"

namespace
{
using namespace gb300;

constexpr int FLOOR_MAX_RUNS = 1024;

template <int KB>
struct word_of;
template <>
struct word_of<4>
{
  using type = uint32_t;
};
template <>
struct word_of<8>
{
  using type = unsigned long long;
};

template <int KB, int VB, int MT, int ITEMS>
__global__ void __launch_bounds__(MT, 1) pattern_floor_kernel(
  const void* keys_in, void* keys_out, const uint32_t* values_in, uint32_t* values_out, uint32_t ntiles, int runs, int shift)
{
  using K             = typename word_of<KB>::type;
  constexpr int TILE  = MT * ITEMS;
  extern __shared__ __align__(16) unsigned char smem[];
  K* kst              = reinterpret_cast<K*>(smem);
  uint32_t* vst       = reinterpret_cast<uint32_t*>(smem + sizeof(K) * TILE);
  uint16_t* run_of    = reinterpret_cast<uint16_t*>(smem + (sizeof(K) + (VB > 0 ? 4 : 0)) * TILE);
  __shared__ int64_t gdelta[FLOOR_MAX_RUNS];
  __shared__ int run_start[FLOOR_MAX_RUNS + 1]; // first slot of every run (and TILE)
  const K* kin        = static_cast<const K*>(keys_in);
  K* kout             = static_cast<K*>(keys_out);
  const int tid       = threadIdx.x;
  const uint64_t nout = uint64_t(ntiles) * TILE + uint64_t(shift);
  for (int r = tid; r <= runs; r += MT)
  {
    run_start[r] = int(int64_t(TILE) * r / runs);
  }
  __syncthreads();
  for (int r = 0; r < runs; ++r)
  {
    for (int s = run_start[r] + tid; s < run_start[r + 1]; s += MT)
    {
      run_of[s] = uint16_t(r);
    }
  }
  __syncthreads();
  for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x)
  {
    K k[ITEMS];
    uint32_t v[VB > 0 ? ITEMS : 1];
#pragma unroll
    for (int i = 0; i < ITEMS; ++i)
    {
      k[i] = kin[uint64_t(t) * TILE + i * MT + tid];
      if constexpr (VB > 0)
      {
        v[i] = values_in[uint64_t(t) * TILE + i * MT + tid];
      }
    }
#pragma unroll
    for (int i = 0; i < ITEMS; ++i)
    {
      kst[i * MT + tid] = k[i];
      if constexpr (VB > 0)
      {
        vst[i * MT + tid] = v[i];
      }
    }
    for (int r = tid; r < runs; r += MT)
    {
      const int64_t s0  = run_start[r];
      const int64_t len = run_start[r + 1] - s0;
      gdelta[r]         = s0 * ntiles + int64_t(t) * len - s0 + shift;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < ITEMS; ++j)
    {
      const uint32_t s = j * MT + tid;
      const K key      = kst[s];
      const uint64_t g = uint64_t(gdelta[run_of[s]] + int64_t(s));
      if (g < nout)
      {
        __stcs(kout + g, key);
        if constexpr (VB > 0)
        {
          __stcs(values_out + g, vst[s]);
        }
      }
    }
    __syncthreads();
  }
}

template <int KB, int VB>
int run_floor(uint64_t num_items, int runs, int shift, int reps, float* ms_out)
{
  constexpr int MT      = persistent_main(KB, VB);
  constexpr int ITEMS   = persistent_items(KB, VB);
  constexpr int TILE    = MT * ITEMS;
  const uint32_t ntiles = uint32_t(num_items / TILE);
  const uint64_t n      = uint64_t(ntiles) * TILE;
  const uint64_t nout   = n + uint64_t(shift);
  const size_t smem     = (size_t(KB) + (VB > 0 ? 4 : 0) + 2) * TILE;
  auto kern             = pattern_floor_kernel<KB, VB, MT, ITEMS>;
  void *kin = nullptr, *kout = nullptr;
  uint32_t *vin = nullptr, *vout = nullptr;
  int sms       = 0;
  cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (e == cudaSuccess) e = cudaMalloc(&kin, n * KB);
  if (e == cudaSuccess) e = cudaMalloc(&kout, nout * KB);
  if (e == cudaSuccess && VB > 0) e = cudaMalloc(&vin, n * 4);
  if (e == cudaSuccess && VB > 0) e = cudaMalloc(&vout, nout * 4);
  if (e == cudaSuccess) e = cudaMemset(kin, 0x5a, n * KB);
  if (e == cudaSuccess && VB > 0) e = cudaMemset(vin, 0x33, n * 4);
  cudaEvent_t a = nullptr, b = nullptr;
  if (e == cudaSuccess) e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  float best = 1e30f;
  for (int r = 0; e == cudaSuccess && r <= reps; ++r)
  {
    cudaEventRecord(a);
    kern<<<sms, MT, smem>>>(kin, kout, vin, vout, ntiles, runs, shift);
    cudaEventRecord(b);
    e = cudaEventSynchronize(b);
    if (e == cudaSuccess) e = cudaGetLastError();
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
    if (r > 0 && ms < best) best = ms; // the first launch is a warm-up
  }
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  cudaFree(kin);
  cudaFree(kout);
  cudaFree(vin);
  cudaFree(vout);
  if (e != cudaSuccess)
  {
    fprintf(stderr, "pattern floor: %s\n", cudaGetErrorString(e));
    return int(e);
  }
  ms_out[0] = best;
  ms_out[1] = float(TILE);
  ms_out[2] = float(n);
  return 0;
}
} // namespace

// Times the pattern for the persistent pass's tile of (key_bytes, value_bytes) with `runs`
// runs per tile (1: contiguous; 256: a digit pass) whose regions start `shift` keys into the
// output: out[0] = best of `reps` launches after one warm-up (ms), out[1] = keys per tile,
// out[2] = keys moved. Returns 0 or a CUDA error code. Shapes: u32 keys only, u64 keys + u32
// values, 4-byte keys + u32 values.
extern "C" __attribute__((visibility("default"))) int cccl_gb300_pattern_floor(
  int key_bytes, int value_bytes, unsigned long long num_items, int runs, int shift, int reps, float* out)
{
  if (runs < 1 || runs > FLOOR_MAX_RUNS || shift < 0 || shift > 64 || reps < 1 || out == nullptr)
  {
    return int(cudaErrorInvalidValue);
  }
  if (key_bytes == 4 && value_bytes == 0)
  {
    return run_floor<4, 0>(num_items, runs, shift, reps, out);
  }
  if (key_bytes == 8 && value_bytes == 4)
  {
    return run_floor<8, 4>(num_items, runs, shift, reps, out);
  }
  if (key_bytes == 4 && value_bytes == 4)
  {
    return run_floor<4, 4>(num_items, runs, shift, reps, out);
  }
  return int(cudaErrorInvalidValue);
}
