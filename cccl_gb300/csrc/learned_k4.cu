// Learned-partition sort kernels for 4-byte keys.
#include "learned_instances.cuh"

GB300_LEARNED(4, gb300::FP_NONE, i)
GB300_LEARNED(4, gb300::FP_ONESWEEP, f)
GB300_LEARNED_FIT(4)
