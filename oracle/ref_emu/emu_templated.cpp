// Emulation unit: templated kernel (no pivoting).
#define EMU_PREFIX ref_emu_templated
#define EMU_NO_PIVOTS 1
#include "emu_variant.inc"
