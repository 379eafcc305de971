/*
 * engine_internal.hpp — host-side pieces shared by sessions, batches and the
 * request server: the context, device buffers of one problem instance, and
 * the conversion of an instance's FP64 device results into SolutionResults.
 */
#ifndef NRAPS_ENGINE_INTERNAL_HPP
#define NRAPS_ENGINE_INTERNAL_HPP

#include <cuda_runtime.h>

#include <array>
#include <map>
#include <string>

#include "../../include/nraps_gpu.h"
#include "engine.cuh"
#include "arena.hpp"
#include "event.cuh"
#include "host_common.hpp"

struct nraps_ctx {
    nraps_opts opts;
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    uint64_t launches = 0;
    /* launch shape the autotuner chose, per problem shape (materials,
       groups, cells, histories, mode, log): a later session of the same
       shape on this context starts with it instead of tuning again */
    std::map<std::array<uint64_t, 6>, EvParams> tuned;
    /* stream-ordered memory pool of this context's device (created on first
       use, kept until the context is destroyed) */
    cudaMemPool_t pool = nullptr;
};

namespace nrint {

inline int set_err(nraps_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg; else nraps_host::set_error(msg);
    return code;
}

inline int cuda_status(cudaError_t e) {
    return e == cudaErrorMemoryAllocation ? NRAPS_ERR_NOMEM : NRAPS_ERR_CUDA;
}

/* Device memory: cudaMalloc, or (alloc with a pool) stream-ordered from a
   memory pool, which neither synchronises the device nor returns memory to
   the driver, and is freed in the same stream's order. */
struct DevMem {
    void* p = nullptr;
    size_t n = 0;
    cudaStream_t fs = nullptr;          /* stream-ordered: the stream it is freed on */
    bool pooled = false;
    bool in_arena = false;              /* owned by a DeviceArena: never freed here */
    DevMem() = default;
    DevMem(const DevMem&) = delete;
    DevMem& operator=(const DevMem&) = delete;
    ~DevMem() { release(); }
    void release() {
        if (p && !in_arena) { if (pooled) cudaFreeAsync(p, fs); else cudaFree(p); }
        p = nullptr;
        pooled = false;
        in_arena = false;
    }
    /* a small buffer from the arena, a large one from cudaMalloc */
    cudaError_t alloc_in(DeviceArena& a, size_t bytes) {
        if (bytes == 0 || bytes > DeviceArena::ITEM_MAX) return alloc(bytes);
        release();
        n = bytes;
        in_arena = true;
        return a.take(bytes, &p);
    }
    cudaError_t alloc(size_t bytes, cudaMemPool_t pool = nullptr, cudaStream_t s = nullptr) {
        release();
        n = bytes;
        if (bytes == 0) return cudaSuccess;
        if (pool) {
            pooled = true;
            fs = s;
            return cudaMallocFromPoolAsync(&p, bytes, pool, s);
        }
        return cudaMalloc(&p, bytes);
    }
    template <class T> T* as() const { return reinterpret_cast<T*>(p); }
};

/* Device buffers of one problem instance of the event engine. */
struct InstBuffers {
    DevMem tally, flux_acc, flux_sum, flux_sq, fs_acc, k64, entropy, bank0, bank1, hist, own_state;
    GenState* st = nullptr;
    uint64_t G = 0, nc = 0, gens = 0, cap = 0;
    uint32_t tally_shift = 0;     /* tally bin b at word b << tally_shift */
    /* st_ext: a GenState slot owned by the caller, or nullptr to own one;
       pool: allocate stream-ordered on s from this pool (no device-wide
       synchronisation: the request server admits and retires many
       instances), or nullptr for cudaMalloc; arena: small buffers from it
       at 64 KB strides (batches) */
    cudaError_t alloc(uint64_t G_, uint64_t nc_, uint64_t gens_, uint64_t N, double bank_factor, bool bank,
                      double k0, GenState* st_ext, cudaStream_t s, cudaMemPool_t pool = nullptr,
                      DeviceArena* arena = nullptr);
    EvBuffers view(uint64_t skip, uint64_t seed) const;
    uint64_t bytes() const;
};

/* What is needed to turn an instance's device results into SolutionResults. */
struct ResultsView {
    uint64_t G, nc, gens, skip, numass, done, histories;
    const double *flux_acc, *flux_sum, *flux_sq, *fs_acc, *k64, *entropy;
    const GenState* st;
    double transport_ms, total_ms;
    uint64_t transport_launches, gpu_launches;
};

/* The context's memory pool (created on first call; nullptr on failure). */
cudaMemPool_t ctx_pool(nraps_ctx* ctx);

/* Copies device results into `out` (synchronous on the current device). */
int fetch_results(nraps_ctx* ctx, const ResultsView& v, nraps_result* out);

/* Problem validation shared by every entry point. */
int validate_problem(nraps_ctx* ctx, const nraps_problem* p, const nraps_opts& o);

}  // namespace nrint

#endif
