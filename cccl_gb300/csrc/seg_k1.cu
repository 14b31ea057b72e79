// Batched segmented sort kernels for 1-byte keys.
#include "segmented_instances.cuh"

GB300_SEG_VALUES(1, gb300::FP_NONE, i)
GB300_SEG_NET_VALUES(1, 0, u)
GB300_SEG_NET_VALUES(1, 1, i)
GB300_SEG_HIST(1, gb300::FP_NONE, i)
GB300_SEG_RNET_VALUES(1, gb300::NET_RADIX + gb300::FP_NONE, ri)
