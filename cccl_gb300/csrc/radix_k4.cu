// Plain-path kernels for 4-byte keys (integer and floating-point key kinds).
#include "radix_instances.cuh"

GB300_ALL_VALUES(4, false, i)
GB300_ONESWEEP_FIRST(4)
GB300_ALL_VALUES(4, true, f)
