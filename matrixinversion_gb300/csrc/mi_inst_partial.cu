// Instantiations of the contiguous-batch inverse kernel for n = 1..32,
// pivot mode partial.
#include "mi_launch.cuh"

namespace mi {
MI_TABLE(kTablePartial, kModePartial);
}  // namespace mi
