// Plain-path kernels for 1-byte keys (integer key kinds).
#include "radix_instances.cuh"

GB300_ALL_VALUES(1, gb300::FP_NONE, i)
GB300_ONESWEEP_FIRST(1)

