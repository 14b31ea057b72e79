// Learned-partition sort kernels for 4-byte keys.
#include "learned_instances.cuh"

GB300_LEARNED(4, false, i)
GB300_LEARNED(4, true, f)
GB300_LEARNED_FIT(4)
