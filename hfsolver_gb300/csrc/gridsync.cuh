// Grid-wide barrier for cooperative launches: a counter that only grows.
// Barrier number `epoch` (1, 2, ...) completes when the count reaches
// epoch * nblocks; the arrival is a release and the wait an acquire, so the
// writes a block made before the barrier are visible to every block after it
// (no separate fences).  The wait gives up after limit_ns (2 s unless the caller
// says otherwise) and sets *err, so a grid that was not co-resident cannot spin
// forever.
#pragma once
#include <cstdint>

namespace hfgpu {

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void red_add_release(unsigned* p, unsigned v)
{
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// called by one thread per block; true unless the wait timed out (then *err = 1)
__device__ __forceinline__ bool grid_arrive_wait(unsigned* count, int* err, unsigned nblocks, unsigned epoch,
                                                 uint64_t limit_ns = 2000000000ull)
{
    red_add_release(count, 1u);
    const unsigned target = epoch * nblocks;
    unsigned spins = 0;
    uint64_t t0 = 0;
    while ((int)(ld_acquire(count) - target) < 0) {
        if ((++spins & 1023u) == 0) {
            if (t0 == 0) {
                t0 = global_ns();
            } else if (global_ns() - t0 > limit_ns) {
                atomicExch(err, 1);
                break;
            }
        }
    }
    return *(volatile int*)err == 0;
}

}  // namespace hfgpu
