"""GB300-native sort engine with the C ABI and Python API of CCCL's sort path.

``cccl_gb300.build()`` compiles the sm_103a kernels and the host library in-tree;
``radix_sort`` / ``make_radix_sort`` (and the segmented and learned-partition
counterparts) call the library's C ABI. There is no CPU fallback: without the built library every call raises.
"""

from .build import build, library_path
from .radix_sort import DoubleBuffer, SortOrder, make_radix_sort, radix_sort, sort_status
from .segmented_sort import make_segmented_radix_sort, make_segmented_sort, segmented_radix_sort, segmented_sort
from .learned_sort import learned_sort, make_learned_sort
from .distributed_sort import distributed_sort

__all__ = [
    "build",
    "library_path",
    "DoubleBuffer",
    "SortOrder",
    "make_radix_sort",
    "radix_sort",
    "sort_status",
    "make_segmented_sort",
    "segmented_sort",
    "make_segmented_radix_sort",
    "segmented_radix_sort",
    "make_learned_sort",
    "learned_sort",
    "distributed_sort",
]
