// Batched segmented sort kernels for 8-byte keys.
#include "segmented_instances.cuh"

GB300_SEG_VALUES(8, false, i)
GB300_SEG_NET_VALUES(8, 0, u)
GB300_SEG_NET_VALUES(8, 1, i)
GB300_SEG_HIST(8, false, i)
GB300_SEG_VALUES(8, true, f)
GB300_SEG_NET_VALUES(8, 2, f)
GB300_SEG_HIST(8, true, f)
