// Learned-partition sort kernels for 8-byte keys.
#include "learned_instances.cuh"

GB300_LEARNED(8, false, i)
GB300_LEARNED(8, true, f)
GB300_LEARNED_FIT(8)
