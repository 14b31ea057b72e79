// Batched segmented sort kernels for 2-byte keys.
#include "segmented_instances.cuh"

GB300_SEG_VALUES(2, false, i)
GB300_SEG_NET_VALUES(2, 0, u)
GB300_SEG_NET_VALUES(2, 1, i)
GB300_SEG_HIST(2, false, i)
GB300_SEG_VALUES(2, true, f)
GB300_SEG_NET_VALUES(2, 2, f)
GB300_SEG_HIST(2, true, f)
