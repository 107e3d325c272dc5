/*
 * emu_cuda.h -- just enough of the CUDA execution model, on host threads, to
 * compile the reference's kernel headers unchanged with g++ and run one block
 * at a time: each CUDA thread is a std::thread, __syncthreads is a
 * std::barrier, dynamic shared memory is one file-scope array per translation
 * unit.  TEST INFRASTRUCTURE ONLY: it pins the oracle's pivot replay against
 * the reference's own device code; nothing in the product uses it.
 */
#pragma once
#include <cmath>
#include <cstdio>
#include <cstdlib>

struct emu_dim3 { unsigned x, y, z; };
extern thread_local emu_dim3 emu_threadIdx;
extern thread_local emu_dim3 emu_blockIdx;
void emu_syncthreads();

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __launch_bounds__(...)
#define __shared__
#define __syncthreads() emu_syncthreads()
#define threadIdx emu_threadIdx
#define blockIdx emu_blockIdx
