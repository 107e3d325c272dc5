// Thread/barrier runtime for the host-thread CUDA stand-in (see shim/emu_cuda.h).
#include <barrier>
#include "shim/emu_cuda.h"

thread_local emu_dim3 emu_threadIdx;
thread_local emu_dim3 emu_blockIdx;
std::barrier<>* emu_block_barrier = nullptr;

void emu_syncthreads() { emu_block_barrier->arrive_and_wait(); }
