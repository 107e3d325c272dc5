// Emulation unit: parallel_pivot kernel (column argmax by a shared-memory tree).
#define EMU_PREFIX ref_emu_parallel_pivot
#include "emu_variant.inc"
