// Out-of-line part of oracle/ref_shim/cuda_cpu_shim.h.  TEST INFRASTRUCTURE ONLY.
#include "cuda_cpu_shim.h"

thread_local uint3 blockIdx, threadIdx;
uint3 blockDim, gridDim;
thread_local std::barrier<> *g_block_barrier = nullptr;

void run_grid(std::uint32_t n_blocks, std::uint32_t block_size, bool concurrent_threads,
              const std::function<void()> &fn) {
    blockDim = {block_size, 1, 1};
    gridDim = {n_blocks, 1, 1};
    for (std::uint32_t b = 0; b < n_blocks; ++b) {
        if (!concurrent_threads) {
            for (std::uint32_t t = 0; t < block_size; ++t) {
                blockIdx = {b, 0, 0};
                threadIdx = {t, 0, 0};
                fn();
            }
            continue;
        }
        std::barrier<> bar((std::ptrdiff_t)block_size);
        std::vector<std::thread> th;
        th.reserve(block_size);
        for (std::uint32_t t = 0; t < block_size; ++t) {
            th.emplace_back([&, b, t]() {
                blockIdx = {b, 0, 0};
                threadIdx = {t, 0, 0};
                g_block_barrier = &bar;
                fn();
                bar.arrive_and_drop();
            });
        }
        for (auto &x : th) x.join();
    }
}

// The reference launchers call these runtime functions; the drivers never call the launchers,
// so the stubs only satisfy the linker.
extern "C" {
cudaError_t cudaMemsetAsync(void *, int, size_t, cudaStream_t) { std::abort(); }
cudaError_t cudaMemcpyAsync(void *, const void *, size_t, enum cudaMemcpyKind, cudaStream_t) { std::abort(); }
cudaError_t cudaStreamSynchronize(cudaStream_t) { std::abort(); }
cudaError_t cudaGetLastError(void) { return cudaSuccess; }
const char *cudaGetErrorString(cudaError_t) { return "cpu shim"; }
}
