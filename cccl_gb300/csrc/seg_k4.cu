// Batched segmented sort kernels for 4-byte keys.
#include "segmented_instances.cuh"

GB300_SEG_VALUES(4, false, i)
GB300_SEG_NET_VALUES(4, 0, u)
GB300_SEG_NET_VALUES(4, 1, i)
GB300_SEG_HIST(4, false, i)
GB300_SEG_VALUES(4, true, f)
GB300_SEG_NET_VALUES(4, 2, f)
GB300_SEG_HIST(4, true, f)
