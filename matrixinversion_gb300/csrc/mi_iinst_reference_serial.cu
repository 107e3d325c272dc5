// Instantiations of the indexed (descriptor bucket) inverse kernel for
// n = 1..32, pivot mode reference_serial.
#include "mi_launch.cuh"

namespace mi {
MI_ITABLE(kITableReferenceSerial, kModeReferenceSerial);
}  // namespace mi
