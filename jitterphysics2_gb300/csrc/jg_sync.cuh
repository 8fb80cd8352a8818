// Grid-wide barrier for persistent (cooperatively launched) kernels.  Every wait is
// bounded: a block that spins longer than the limit records JG_ERR_TIMEOUT in the
// status word and returns false, and every other block sees that status in its own spin
// and leaves too, so a lost block can never hang the GPU.
#pragma once
#include "jg_world.cuh"

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ld_relaxed_int(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Returns false when the barrier timed out or another block reported a failure.
__device__ __forceinline__ bool grid_sync(unsigned* count, unsigned* gen, int* status) {
    __shared__ int ok_flag;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        unsigned g = ld_acquire(gen);
        __threadfence();
        unsigned arrived = atomicAdd(count, 1u);
        if (arrived == gridDim.x - 1) {
            atomicExch(count, 0u);
            __threadfence();
            atomicAdd(gen, 1u);
        } else {
            // about 2^22 polls with back-off (about a second), far above any legitimate wait
            unsigned spins = 0;
            while (ld_acquire(gen) == g) {
                if (ld_relaxed_int(status) == JG_ERR_TIMEOUT) { ok = 0; break; }
                if (++spins > (1u << 22)) {
                    atomicCAS(status, 0, JG_ERR_TIMEOUT);
                    ok = 0;
                    break;
                }
                __nanosleep(spins < 64 ? 0 : 64);
            }
        }
        __threadfence();
        ok_flag = ok;
    }
    __syncthreads();
    return ok_flag != 0;
}
