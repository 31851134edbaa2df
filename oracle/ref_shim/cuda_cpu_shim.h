// CPU execution shim for the reference's CUDA kernels.  TEST INFRASTRUCTURE ONLY.
//
// oracle/build_ref.sh feeds each reference kernel file (volume-rendering-jax/lib/impl/*.cu) to
// g++ through this header, with its `<<<...>>>` launch configurations stripped, followed by a
// driver (oracle/ref_driver_*.cpp) that runs every CUDA thread of every block on the CPU.  The
// reference sources are read where they lie and are never copied; the result lands only in
// oracle/_ref/.
#pragma once
#include <cuda_runtime_api.h>

#include <algorithm>
#include <barrier>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <thread>
#include <vector>

#undef __host__
#undef __device__
#undef __global__
#undef __shared__
#undef __forceinline__
#define __host__
#define __device__
#define __global__
#define __forceinline__ inline
#define __shared__ static
#ifndef __CUDACC__
#define __CUDACC__ 1
#endif

// per-CPU-thread emulation of the CUDA built-in indices
extern thread_local uint3 blockIdx, threadIdx;
extern uint3 blockDim, gridDim;
extern thread_local std::barrier<> *g_block_barrier;

static inline std::uint32_t atomicAdd(std::uint32_t *p, std::uint32_t v) {
    return __atomic_fetch_add(p, v, __ATOMIC_SEQ_CST);
}
static inline void __syncthreads() { g_block_barrier->arrive_and_wait(); }
#define __expf(x) expf(x)  // glibc already declares a __expf; route the CUDA intrinsic to expf
static inline int min(int a, int b) { return a < b ? a : b; }
static inline int max(int a, int b) { return a > b ? a : b; }
static inline unsigned min(unsigned a, unsigned b) { return a < b ? a : b; }
static inline unsigned max(unsigned a, unsigned b) { return a > b ? a : b; }

// Run kernel body `fn` for every thread of a 1-D grid.  Blocks run one after another.  With
// `concurrent_threads`, each block's threads run as real CPU threads sharing one barrier, so
// `__syncthreads` and block-shared counters behave as on the GPU (exited threads drop out of the
// barrier, as exited warps do); otherwise threads run in index order, which is one legal schedule
// for kernels that use neither.
void run_grid(std::uint32_t n_blocks, std::uint32_t block_size, bool concurrent_threads,
              const std::function<void()> &fn);
