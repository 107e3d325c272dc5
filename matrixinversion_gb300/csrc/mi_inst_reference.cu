// Instantiations of the contiguous-batch inverse kernel for n = 1..32,
// pivot mode reference.
#include "mi_launch.cuh"

namespace mi {
MI_TABLE(kTableReference, kModeReference);
}  // namespace mi
