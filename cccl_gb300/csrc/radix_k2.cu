// Plain-path kernels for 2-byte keys (integer and floating-point key kinds).
#include "radix_instances.cuh"

GB300_ALL_VALUES(2, gb300::FP_NONE, i)
GB300_ONESWEEP_FIRST(2)
GB300_ALL_VALUES(2, gb300::FP_ONESWEEP, f)
GB300_SINGLE_TILE_DESC_FP(2)
