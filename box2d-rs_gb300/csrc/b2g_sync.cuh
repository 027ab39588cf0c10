/*
 * b2g_sync.cuh — grid-wide barrier for the cooperative (persistent) kernels.
 *
 * Sense-by-generation barrier over the co-resident blocks of a cooperative launch. Thread 0
 * of each block arrives with an acquire-release add on a counter; the last arrival resets the
 * counter and publishes the next generation with a release store; the others spin on an
 * acquire load and check a clock64 limit (~1 s at 2 GHz) every 256 polls. __syncthreads
 * around it orders the rest of the block. On timeout the block sets ST_BARRIER_TIMEOUT in the
 * status word; once set, every later barrier returns false at once, so all blocks leave the
 * kernel within one limit and the host reports B2G_ERR_TIMEOUT. Thread 0 decides for its block
 * and broadcasts through shared memory, so all threads of a block see the same result.
 */
#ifndef B2G_SYNC_CUH
#define B2G_SYNC_CUH

#include "b2g_internal.h"

namespace b2g {

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned atom_add_acq_rel_gpu(unsigned* p, unsigned v) {
    unsigned old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}
__device__ __forceinline__ void st_release_gpu(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

/* cnt: the world's counter block (uses CNT_BARRIER, CNT_BARRIER + 1 and CNT_STATUS) */
__device__ __forceinline__ bool grid_barrier(int* cnt) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = (((volatile int*)cnt)[CNT_STATUS] & ST_BARRIER_TIMEOUT) == 0;
        if (ok) {
            unsigned* count = (unsigned*)&cnt[CNT_BARRIER];
            unsigned* gen_ptr = (unsigned*)&cnt[CNT_BARRIER + 1];
            const unsigned gen = ld_acquire_gpu(gen_ptr);
            const unsigned arrived = atom_add_acq_rel_gpu(count, 1u);
            if (arrived == gridDim.x - 1) {
                atomicExch(count, 0u);
                st_release_gpu(gen_ptr, gen + 1u);
            } else {
                const long long t0 = clock64();
                unsigned polls = 0;
                while (ld_acquire_gpu(gen_ptr) == gen) {
                    if ((++polls & 255u) == 0u && clock64() - t0 > 2000000000LL) {
                        atomicOr((unsigned*)&cnt[CNT_STATUS], ST_BARRIER_TIMEOUT);
                        break;
                    }
                }
            }
            ok = (((volatile int*)cnt)[CNT_STATUS] & ST_BARRIER_TIMEOUT) == 0;
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

__device__ __forceinline__ bool grid_barrier(const DevWorld& w) { return grid_barrier(w.cnt); }

}  // namespace b2g
#endif
