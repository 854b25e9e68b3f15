// Device-side helpers shared by the kernels of libkcore.so (sm_103a).
#pragma once

#include <cstdint>

#define KC_FULL_MASK 0xffffffffu

namespace kc {

// Nanoseconds from the GPU global timer; used to bound every spin-wait.
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned int ld_acquire(const unsigned int *p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned long long ld_acquire64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(unsigned int *p, unsigned int v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned int ld_relaxed(const unsigned int *p) {
    unsigned int v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned long long ld_relaxed64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_relaxed64(unsigned long long *p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Grid-wide barrier for a cooperative (co-resident) launch.  Arrivals count
// up in *count; the last arrival resets it and bumps *gen.  Waiters spin on
// *gen with a wall-clock limit; on timeout *err is set and false returned,
// after which callers must leave the kernel.
__device__ __forceinline__ bool grid_barrier(unsigned int *count, unsigned int *gen, unsigned int nblocks,
                                             unsigned int *err, unsigned int err_code,
                                             unsigned long long timeout_ns) {
    __shared__ unsigned int ok_sh;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int g = ld_acquire(gen);
        __threadfence();
        unsigned int arrived = atomicAdd(count, 1u);
        unsigned int ok = 1;
        if (arrived == nblocks - 1) {
            atomicExch(count, 0u);
            __threadfence();
            st_release(gen, g + 1);
        } else {
            unsigned long long t0 = global_ns();
            unsigned int spins = 0;
            while (ld_acquire(gen) == g) {
                if (ld_relaxed(err) != 0) { ok = 0; break; }
                if ((++spins & 63u) == 0 && global_ns() - t0 > timeout_ns) {
                    atomicCAS(err, 0u, err_code);
                    ok = 0;
                    break;
                }
                __nanosleep(32);
            }
        }
        if (ld_relaxed(err) != 0) ok = 0;
        ok_sh = ok;
    }
    __syncthreads();
    return ok_sh != 0;
}

__device__ __forceinline__ unsigned int warp_excl_scan(unsigned int x, unsigned int lane, unsigned int &total) {
    unsigned int v = x;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        unsigned int y = __shfl_up_sync(KC_FULL_MASK, v, d);
        if (lane >= (unsigned)d) v += y;
    }
    total = __shfl_sync(KC_FULL_MASK, v, 31);
    return v - x;
}

}  // namespace kc
