/* Host-thread stand-in for the CUDA header of the same name (oracle pinning only). */
#pragma once
#include "emu_cuda.h"
