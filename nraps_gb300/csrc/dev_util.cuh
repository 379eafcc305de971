/* dev_util.cuh — warp/block scan and aggregated-atomic helpers. */
#ifndef NRAPS_DEV_UTIL_CUH
#define NRAPS_DEV_UTIL_CUH
#include <stdint.h>

namespace nrdev {

/* Programmatic dependent launch (sm_90+).  A kernel launched with
   programmatic stream serialization may start while the kernel before it
   in the stream is still finishing; pdl_wait() blocks until that kernel
   has completed and its memory is visible, so everything a kernel reads or
   writes that the one before it produces or reads comes after it (reading
   tables no kernel writes may come before).  A kernel launched without the
   attribute returns from it at once.  pdl_trigger() lets the next kernel
   launch as soon as every block of this one has started. */
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
    int lane = threadIdx.x & 31;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t n = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += n;
    }
    return v;
}

/* Block-wide exclusive scan of one value per thread; every thread of the
   block must call it.  smem_warp needs 33 words.  Returns the block total. */
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* excl, uint32_t* smem_warp) {
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t inc = warp_incl_scan(v);
    if (lane == 31) smem_warp[w] = inc;
    __syncthreads();
    if (w == 0) {
        uint32_t t = lane < nw ? smem_warp[lane] : 0u;
        uint32_t ti = warp_incl_scan(t);
        if (lane < nw) smem_warp[lane] = ti - t;
        if (lane == 31) smem_warp[32] = ti;
    }
    __syncthreads();
    *excl = inc - v + smem_warp[w];
    uint32_t total = smem_warp[32];
    __syncthreads();
    return total;
}

/* Each calling lane gets a distinct slot: one atomic per group of
   converged lanes. */
__device__ __forceinline__ unsigned long long agg_inc(unsigned long long* ctr) {
    unsigned mask = __activemask();
    int lane = threadIdx.x & 31;
    int leader = __ffs(mask) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(ctr, (unsigned long long)__popc(mask));
    base = __shfl_sync(mask, base, leader);
    return base + (unsigned long long)__popc(mask & ((1u << lane) - 1u));
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

/* Fire-and-forget global reductions.  Written as PTX `red.global` so that a
   pointer the compiler cannot prove global (one read from shared memory, say)
   still becomes a global reduction rather than a generic atomic that returns
   the old value. */
__device__ __forceinline__ void red_add_f64(double* p, double v) {
    asm volatile("red.global.add.f64 [%0], %1;" ::"l"(__cvta_generic_to_global(p)), "d"(v) : "memory");
}
__device__ __forceinline__ void red_add_u32(uint32_t* p, uint32_t v) {
    asm volatile("red.global.add.u32 [%0], %1;" ::"l"(__cvta_generic_to_global(p)), "r"(v) : "memory");
}

}  // namespace nrdev
#endif
