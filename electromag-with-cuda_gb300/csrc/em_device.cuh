// Device-side helpers shared by the tracer kernels: mbarrier waits with a
// time limit, bulk (TMA) copies global -> shared, streaming stores.
//
// Every wait in this library is bounded: after EM_WAIT_LIMIT_NS of waiting
// the kernel records EM_DEVERR_TIMEOUT in its error word and returns instead
// of spinning forever.  No kernel traps or asserts.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "em_internal.h"

namespace em {

// electro_k of include/Electrostatics.h:27 (Coulomb constant, SI units).
constexpr double kElectroK = 8.987551787E9;

// 2 s: far above any legitimate wait (one charge tile takes microseconds).
constexpr uint64_t EM_WAIT_LIMIT_NS = 2000000000ull;

__device__ __forceinline__ uint64_t globaltimer_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// Arrives on the pending phase and leaves: later phases expect one arrival
// fewer (a consumer that will read no further tiles).
__device__ __forceinline__ void mbar_arrive_drop(uint32_t bar)
{
    asm volatile("mbarrier.arrive_drop.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(bar), "r"(parity)
                 : "memory");
    return ok != 0;
}

// Waits for the phase with the given parity to complete.  Returns false
// (and records a timeout in *err) if it has not completed within limit_ns.
__device__ __forceinline__ bool mbar_wait_limit(uint32_t bar, uint32_t parity, int *err,
                                                uint64_t limit_ns)
{
    if (mbar_try_wait(bar, parity))
        return true;
    const uint64_t t0 = globaltimer_ns();
    for (;;) {
        for (int i = 0; i < 64; ++i)
            if (mbar_try_wait(bar, parity))
                return true;
        if (globaltimer_ns() - t0 > limit_ns) {
            atomicCAS(err, 0, EM_DEVERR_TIMEOUT);
            return false;
        }
        if (*(volatile int *)err != 0)
            return false; // another warp already gave up
    }
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int *err)
{
    return mbar_wait_limit(bar, parity, err, EM_WAIT_LIMIT_NS);
}

// Bulk copy of `bytes` (multiple of 16, both addresses 16-B aligned) from
// global to this CTA's shared memory, completing on mbarrier `bar`.
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes,
                                         uint32_t bar)
{
    asm volatile("cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes "
                 "[%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

__device__ __forceinline__ void store_stream(float *p, float v) { __stcs(p, v); }
__device__ __forceinline__ void store_stream(double *p, double v) { __stcs(p, v); }

} // namespace em
