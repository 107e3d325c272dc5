// Walks of the single persistent descriptor launch for pivot mode reference_serial,
// n = 1..32 (relocatable device code, linked with mi_descr_persist.cu).
#include "mi_persist.cuh"

namespace mi {
MI_PWALK_EACH_N(MI_PWALK_DEF, 2)
}  // namespace mi
