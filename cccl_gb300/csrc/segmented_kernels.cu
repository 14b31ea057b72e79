// Segmented-sort kernels (size-class binning, warp/block classes). Placeholder until the
// batched path lands.
#include "radix_kernels.cuh"

extern "C" __global__ void __launch_bounds__(256) gb300_init(const gb300::InitParams p)
{
  gb300::init_body(p);
}
