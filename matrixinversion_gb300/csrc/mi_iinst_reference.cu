// Instantiations of the indexed (descriptor bucket) inverse kernel for
// n = 1..32, pivot mode reference.
#include "mi_launch.cuh"

namespace mi {
MI_ITABLE(kITableReference, kModeReference);
}  // namespace mi
