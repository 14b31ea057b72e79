// Plain-path kernels for 8-byte keys (integer and floating-point key kinds).
#include "radix_instances.cuh"

GB300_ALL_VALUES(8, false, i)
GB300_ONESWEEP_FIRST(8)
GB300_ALL_VALUES(8, true, f)
