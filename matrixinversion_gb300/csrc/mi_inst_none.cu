// Instantiations of the contiguous-batch inverse kernel for n = 1..32,
// pivot mode none.
#include "mi_launch.cuh"

namespace mi {
MI_TABLE(kTableNone, kModeNone);
}  // namespace mi
