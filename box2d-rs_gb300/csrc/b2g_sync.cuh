/*
 * b2g_sync.cuh — grid-wide barrier for the cooperative (persistent) kernels.
 *
 * Counting barrier over the co-resident blocks of a cooperative launch. The launcher zeroes the
 * counter before every launch (a memset node in the step graph), so the k-th barrier of the
 * launch completes when the counter reaches (k + 1) x gridDim.x. Thread 0 of each block keeps k in
 * shared memory, arrives with one fire-and-forget release add and polls the counter with acquire
 * loads; nobody resets anything, so the last block to arrive waits for no extra round trip, and a
 * barrier costs one arrival and the polls (the launch's settings are read once, at its first
 * barrier). Each wait is bounded: a clock64 limit checked every 256 polls, cnt[CNT_BARRIER_LIMIT] x
 * 1024 cycles (b2g_set_barrier_limit; 0 means 2e9 cycles, ~1 s at 2 GHz). cnt[CNT_BARRIER_HOLD] (0
 * unless a test sets it) is added to every wait's target: arrivals that never come, so the wait runs
 * out its limit; it exists to test the timeout path without a fault. On timeout the block sets
 * ST_BARRIER_TIMEOUT in the status word and leaves the kernel; a block waiting at any barrier sees
 * the status at its next check (every 256 polls) and leaves too, so all blocks leave within one
 * limit and the host reports B2G_ERR_TIMEOUT (kernels launched later return at once). Thread 0
 * decides for its block and broadcasts through shared memory, so all threads of a block see the
 * same result. Every cooperative kernel calls grid_barrier_start() first.
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

__device__ __forceinline__ void red_release_add_gpu(unsigned* p, unsigned v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

/* barriers this block has passed in the current launch, and the launch's wait limit and held
 * arrivals (used by thread 0) */
static __shared__ unsigned b2g_barrier_epoch;
static __shared__ long long b2g_barrier_limit;
static __shared__ unsigned b2g_barrier_hold;

__device__ __forceinline__ void grid_barrier_start() {
    if (threadIdx.x == 0) b2g_barrier_epoch = 0u;  /* ordered by the barrier's first __syncthreads */
}

/* cnt: the counter block (uses CNT_BARRIER, zeroed by the launcher, and CNT_STATUS) */
__device__ __forceinline__ bool grid_barrier(int* cnt) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        if (b2g_barrier_epoch == 0u) {
            int2 lim_hold;
            asm volatile("ld.volatile.global.v2.s32 {%0, %1}, [%2];"
                         : "=r"(lim_hold.x), "=r"(lim_hold.y) : "l"(&cnt[CNT_BARRIER_LIMIT]) : "memory");
            b2g_barrier_limit = lim_hold.x > 0 ? (long long)lim_hold.x << 10 : 2000000000LL;
            b2g_barrier_hold = (unsigned)max(lim_hold.y, 0);
        }
        unsigned* count = (unsigned*)&cnt[CNT_BARRIER];
        const unsigned target = (b2g_barrier_epoch + 1u) * gridDim.x + b2g_barrier_hold;
        ++b2g_barrier_epoch;
        red_release_add_gpu(count, 1u);
        const long long t0 = clock64();
        unsigned polls = 0;
        int ok = 1;
        while ((int)(ld_acquire_gpu(count) - target) < 0) {
            if ((++polls & 255u) == 0u) {
                if (((volatile int*)cnt)[CNT_STATUS] & ST_BARRIER_TIMEOUT) {
                    ok = 0;
                    break;
                }
                if (clock64() - t0 > b2g_barrier_limit) {
                    atomicOr((unsigned*)&cnt[CNT_STATUS], ST_BARRIER_TIMEOUT);
                    ok = 0;
                    break;
                }
            }
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

__device__ __forceinline__ bool grid_barrier(const DevWorld& w) { return grid_barrier(w.cnt); }

}  // namespace b2g
#endif
