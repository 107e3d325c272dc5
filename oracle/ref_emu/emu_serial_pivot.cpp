// Emulation unit: serial_pivot kernel (thread-0 argmax and swap).
#define EMU_PREFIX ref_emu_serial_pivot
#include "emu_variant.inc"
