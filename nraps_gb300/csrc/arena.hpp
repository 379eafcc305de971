/*
 * arena.hpp — device memory for a session's small buffers at fixed strides.
 *
 * The event transport's time per launch on single_large ranged over 0.10 to
 * 0.14 ms depending only on where cudaMalloc placed the session's small
 * buffers (tallies, counters, the instance descriptor and tables, the
 * per-history counts and queues): the same process, the same kernels, more
 * or less memory allocated beforehand.  Every buffer of up to ITEM_MAX bytes
 * is therefore taken from one arena, each starting on its own 64 KB
 * boundary; with that layout the launch time measured 0.099-0.100 ms whatever
 * was allocated before the session.  Buffers are not freed one by one: the
 * arena's chunks are freed when the arena is destroyed (its owner outlives
 * every buffer it hands out).
 */
#ifndef NRAPS_ARENA_HPP
#define NRAPS_ARENA_HPP
#include <cuda_runtime.h>

#include <cstddef>
#include <vector>

struct DeviceArena {
    static constexpr size_t ALIGN = 64u << 10;      /* every buffer on its own 64 KB */
    static constexpr size_t ITEM_MAX = 4u << 20;    /* larger buffers: cudaMalloc */
    static constexpr size_t CHUNK = 64u << 20;
    std::vector<void*> chunks;
    char* cur = nullptr;
    size_t off = 0, cap = 0;
    DeviceArena() = default;
    DeviceArena(const DeviceArena&) = delete;
    DeviceArena& operator=(const DeviceArena&) = delete;
    ~DeviceArena() { for (void* c : chunks) cudaFree(c); }
    /* bytes <= ITEM_MAX from the arena (a new chunk when the current one is
       full); the caller never frees it */
    cudaError_t take(size_t bytes, void** p) {
        const size_t need = (bytes + ALIGN - 1) / ALIGN * ALIGN;
        if (!cur || off + need > cap) {
            void* c = nullptr;
            cudaError_t e = cudaMalloc(&c, CHUNK);
            if (e != cudaSuccess) return e;
            chunks.push_back(c);
            cur = static_cast<char*>(c);
            off = 0;
            cap = CHUNK;
        }
        *p = cur + off;
        off += need;
        return cudaSuccess;
    }
};
#endif
