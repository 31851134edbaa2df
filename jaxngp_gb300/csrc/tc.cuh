// Fifth-generation tensor-core helpers for sm_103a: tensor-memory allocation, tcgen05.mma with
// shared-memory operand descriptors, completion through mbarriers, and tensor-memory loads.
//
// Operands are staged in shared memory without swizzling, in the canonical "core matrix" layout:
// a core matrix is 8 rows of 16 contiguous bytes (128 bytes).  A buffer that holds a matrix
// X[rows][cols] is stored row-block by row-block: core matrix (r/8, c/E) (E = 16 bytes / element
// size) sits at (r/8) * (cols/E) * 128 + (c/E) * 128, row r%8 at +16*(r%8).  The same bytes serve
// an MMA two ways:
//   * K-major operand with MN = rows, K = cols:  LBO = 128 (next core matrix along K),
//     SBO = (cols/E) * 128 (next 8 rows), one instruction's 32 bytes of K = +256 bytes;
//   * MN-major operand with MN = cols, K = rows: SBO = 128 (next E columns along MN),
//     LBO = (cols/E) * 128 (next 8 rows along K), one instruction's 16 K-rows (16-bit types) =
//     +2 * LBO.
#pragma once

#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_fp16.h>

namespace ngp {
namespace tc {

__device__ __forceinline__ std::uint32_t smem_addr(const void *p) {
    return static_cast<std::uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor (no swizzle, version 1, base offset 0).
__device__ __forceinline__ std::uint64_t sdesc(std::uint32_t saddr, std::uint32_t lbo, std::uint32_t sbo) {
    return (std::uint64_t)((saddr >> 4) & 0x3FFFu) | ((std::uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((std::uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((std::uint64_t)1 << 46);
}

// A shared-memory descriptor as its two 32-bit halves.  The low half holds the start address (bits
// 0-13, in 16-byte units) and the LBO; the descriptor of an offset of `b` bytes into the same buffer
// is the low half plus b / 16 (shared addresses stay below 2^18 bytes, so the address field never
// carries into the LBO), which makes a run of MMAs over one buffer one add per operand each.
struct SDesc {
    std::uint32_t lo, hi;
};

__device__ __forceinline__ SDesc sdesc2(std::uint32_t saddr, std::uint32_t lbo, std::uint32_t sbo) {
    const std::uint64_t v = sdesc(saddr, lbo, sbo);
    return {static_cast<std::uint32_t>(v), static_cast<std::uint32_t>(v >> 32)};
}

// Instruction descriptor of kind::f16 with an FP32 accumulator; `fmt` is the operand format of
// both A and B (0 = FP16, 1 = BF16: one instruction never mixes them).
__host__ __device__ constexpr std::uint32_t idesc_kf16(int M, int N, std::uint32_t fmt, bool a_mn, bool b_mn) {
    return (1u << 4) | (fmt << 7) | (fmt << 10) | ((a_mn ? 1u : 0u) << 15) | ((b_mn ? 1u : 0u) << 16) |
           ((std::uint32_t)(N >> 3) << 17) | ((std::uint32_t)(M >> 4) << 24);
}

__host__ __device__ constexpr std::uint32_t idesc_bf16(int M, int N, bool a_mn, bool b_mn) {
    return idesc_kf16(M, N, 1u, a_mn, b_mn);
}

__host__ __device__ constexpr std::uint32_t idesc_f16(int M, int N) { return idesc_kf16(M, N, 0u, false, false); }

static_assert(idesc_f16(128, 64) == ((1u << 4) | (8u << 17) | (8u << 24)), "FP16 descriptor");
static_assert(idesc_bf16(64, 16, true, true) == ((1u << 4) | (1u << 7) | (1u << 10) | (1u << 15) | (1u << 16) | (2u << 17) | (4u << 24)),
              "BF16 descriptor");

// kind::f16 MMA (BF16 or FP16 operands, as the instruction descriptor says).
__device__ __forceinline__ void mma_bf16(std::uint32_t d_tmem, std::uint64_t a, std::uint64_t b, std::uint32_t idesc,
                                         bool accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        :: "r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(accumulate ? 1u : 0u) : "memory");
}

// The same MMA with the operand descriptors given as halves: (a_lo + a_off, a_hi) and (b_lo + b_off,
// b_hi), the offsets in 16-byte units (see SDesc).
__device__ __forceinline__ void mma_bf16(std::uint32_t d_tmem, SDesc a, std::uint32_t a_off, SDesc b,
                                         std::uint32_t b_off, std::uint32_t idesc, bool accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t.reg .b64 da, db;\n\t"
        "mov.b64 da, {%1, %2};\n\tmov.b64 db, {%3, %4};\n\t"
        "setp.ne.b32 p, %6, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], da, db, %5, p;\n\t}"
        :: "r"(d_tmem), "r"(a.lo + a_off), "r"(a.hi), "r"(b.lo + b_off), "r"(b.hi), "r"(idesc),
           "r"(accumulate ? 1u : 0u) : "memory");
}

// Arrive on `bar` once every MMA issued so far by this thread has completed.
__device__ __forceinline__ void commit(std::uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 :: "r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void mbar_init(std::uint64_t *bar, std::uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// Waits for the phase with parity `parity` to complete; gives up after `limit` polls.
__device__ __forceinline__ bool mbar_wait(std::uint64_t *bar, std::uint32_t parity, std::uint32_t limit) {
    const std::uint32_t a = smem_addr(bar);
    for (std::uint32_t it = 0; it < limit; ++it) {
        std::uint32_t ok;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(ok) : "r"(a), "r"(parity) : "memory");
        if (ok) return true;
    }
    return false;
}

// The next phase of `bar` also waits for `bytes` of asynchronous copies (one arrival).
__device__ __forceinline__ void mbar_expect_tx(std::uint64_t *bar, std::uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(smem_addr(bar)), "r"(bytes) : "memory");
}

// Tensor-map tile load (TMA) of a 4-D box at coordinates {c0, c1, c2, c3} into shared memory;
// completion is signalled on `bar` as transferred bytes.  `map` is the address of a
// __grid_constant__ CUtensorMap kernel parameter.  c0, the innermost coordinate, must keep the
// copy's start 16-byte aligned (callers pass 0).
__device__ __forceinline__ void tma_load_4d(void *dst, const void *map, int c0, int c1, int c2, int c3,
                                            std::uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];"
        :: "r"(smem_addr(dst)), "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_addr(bar)) : "memory");
}

// Generic-proxy shared-memory writes become visible to the tensor cores.
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Named barrier over `count` threads (a warpgroup: 128).
__device__ __forceinline__ void bar_sync(int id, int count) {
    asm volatile("bar.sync %0, %1;" :: "r"(id), "r"(count) : "memory");
}

// One warp allocates `ncols` (power of two, >= 32) tensor-memory columns and writes the base address to *dst.
__device__ __forceinline__ void tmem_alloc(std::uint32_t *dst, std::uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" :: "r"(smem_addr(dst)), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_free(std::uint32_t base, std::uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(base), "r"(ncols) : "memory");
}

// Tensor-memory loads, 32 lanes x N columns: thread `lane` of the warp receives row (lane base of
// the warp's sub-partition + lane), columns [col, col + N) of `taddr`.  The load and its
// completion wait are one asm statement, so nothing can read the registers before they land.
__device__ __forceinline__ void ld16(std::uint32_t taddr, float *v) {
    std::uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr) : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void ld32(std::uint32_t taddr, float *v) {
    std::uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr) : "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void ld64(std::uint32_t taddr, float *v) {
    std::uint32_t r[64];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x64.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%64];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]), "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
        : "r"(taddr) : "memory");
#pragma unroll
    for (int i = 0; i < 64; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ std::uint32_t pack_f16(float a, float b) {
    const __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<const std::uint32_t *>(&h);
}

__device__ __forceinline__ std::uint32_t pack_bf16(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const std::uint32_t *>(&h);
}

}  // namespace tc
}  // namespace ngp
