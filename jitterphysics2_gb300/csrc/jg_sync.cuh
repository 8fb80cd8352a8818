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

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned atom_add_release(unsigned* p, unsigned v) {
    unsigned old;
    asm volatile("atom.add.release.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

// Returns false when the barrier timed out or another block reported a failure.
// The counter only grows (it is zeroed before each cooperative launch): barrier k of
// the launch is passed when it reaches (k + 1) * gridDim.x, so an arrival is one
// release atomic and the wait one acquire load per poll.
__device__ __forceinline__ bool grid_sync(unsigned* count, unsigned* gen, int* status) {
    (void)gen;
    __shared__ int ok_flag;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        __threadfence();
        unsigned old = atom_add_release(count, 1u);
        unsigned target = (old / gridDim.x + 1) * gridDim.x;
        // Polls are spaced by a short sleep: back-to-back polls from every block saturate
        // the L2 slice that holds the counter, which delays the arrivals and every other
        // access that maps to that slice.  The wait gives up after one second (or 2^22
        // polls), far above any legitimate wait.
        const unsigned long long t0 = globaltimer_ns();
        unsigned spins = 0;
        while ((int)(ld_acquire(count) - target) < 0) {
            ++spins;
            if ((spins & 63) == 0) {
                if (ld_relaxed_int(status) == JG_ERR_TIMEOUT) { ok = 0; break; }
                if (globaltimer_ns() - t0 > 1000000000ull || spins > (1u << 22)) {
                    atomicCAS(status, 0, JG_ERR_TIMEOUT);
                    ok = 0;
                    break;
                }
            }
            __nanosleep(spins < 4 ? 20 : 80);
        }
        ok_flag = ok;
    }
    __syncthreads();
    return ok_flag != 0;
}
