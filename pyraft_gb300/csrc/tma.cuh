// tma.cuh -- TMA tile loads and bounded mbarrier waits, shared by the
// TMA-staged kernels (radon_tma.cu, gather_rot.cu).
//
// Every wait is bounded: mbar_wait gives up after kTmWaitNs of global time
// (strips and windows normally land within microseconds) and returns false,
// so a kernel can set its error flag and leave instead of hanging.
#pragma once

#include <cuda.h>

namespace rg {

constexpr int kTmWaitLimit = 1 << 24;                    // polls (backstop)
constexpr unsigned long long kTmWaitNs = 200000000ull;    // 0.2 s per wait

__device__ __forceinline__ unsigned smem_addr(const void *p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(unsigned bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Wait on phase `parity` of an mbarrier for at most kTmWaitNs; false if the
// time ran out.
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity)
{
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (int it = 0; it < kTmWaitLimit; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 63) == 63 && global_ns() - t0 > kTmWaitNs) return false;
    }
    return false;
}

// Order this thread's earlier generic-proxy accesses to shared memory
// before async-proxy (TMA) writes that it issues next.
__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void tma_load_3d(unsigned dst, const CUtensorMap *tm, int x, int y,
                                            int z, unsigned bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
        "l"(reinterpret_cast<unsigned long long>(tm)), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

// cuTensorMapEncodeTiled from the driver (null when the driver lacks it).
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn tensor_map_encoder();

}  // namespace rg
