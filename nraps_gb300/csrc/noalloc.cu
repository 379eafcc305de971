/*
 * noalloc.cu — one PHYSICS-mode generation of the plain FP32 kernel that
 * allocates no device memory.
 *
 * Some callers cannot call cudaMalloc: code running inside another
 * framework's memory pool (where every byte of device memory is already
 * handed out by the host application and a stray allocation fails or
 * fragments the pool), callers that replay work from a pre-planned memory
 * layout, and callers that must not risk an allocation failure in the middle
 * of a job.  They own all device memory themselves.  This entry point takes
 * the problem already resident on the device, writes the results into device
 * buffers the caller provides, and keeps its own working state (the derived
 * cross-section tables and the generation's counters) in the fixed array
 * below, which every GPU that loads this library holds until the process
 * exits.
 *
 * Host code cannot use `g_noalloc_scratch` as a device address: its name on
 * the host is only a stand-in.  The device address is looked up once per
 * device with cudaGetSymbolAddress, with that device current, on the first
 * call made on that device; make that first call before any stream capture.
 * Every call also waits for its input check on the caller's stream (one copy
 * into host memory and a stream synchronisation), so no call can be made
 * while that stream is being captured.
 *
 * Every call shares the one array and the previous call's contents remain in
 * it.  Each call rewrites the tables and clears the counters before its
 * kernels run, on the caller's stream.  Two calls whose work overlaps on the
 * GPU (different streams, or several host threads) race on the array: the
 * caller must order them.  The race covers the input check too: an
 * overlapping call can clear or set the flags between another call's check
 * and its read, so that call may be rejected for the other's inputs or pass
 * with bad ones of its own.
 */
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "engine.cuh"
#include "host_common.hpp"
#include "nr_math.h"

namespace {

/* limits of the fixed array */
constexpr uint32_t NOALLOC_MAX_XS = 1024;      /* (material, group) pairs     */
constexpr uint32_t NOALLOC_MAX_SCAT = 16384;   /* (material, group, group')   */
constexpr size_t NOALLOC_FLOATS = 4 * NOALLOC_MAX_XS + NOALLOC_MAX_SCAT;
constexpr size_t NOALLOC_BYTES = 256 + NOALLOC_FLOATS * sizeof(float);

/* layout: [GenState | flags | pad to 256][nsf][nsf_sigtr][pabs][chi_cdf][phys_cdf] */
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
unsigned char* g_addr[MAX_DEVICES] = {nullptr};

#define NOALLOC_BAD_MAT  1u
#define NOALLOC_BAD_FUEL 2u

struct Flags { unsigned int bad; };

/* the state and the flags must fit the 256-byte header ahead of the tables */
static_assert(sizeof(GenState) + sizeof(Flags) <= 256, "GenState and Flags outgrew the array's header");
static_assert(NOALLOC_BYTES % alignof(float) == 0 && 256 % alignof(GenState) == 0, "table alignment");

/* derived tables (same arithmetic as the packed FP32 tables), cleared state,
   and a range check of the device inputs into the (pre-cleared) flags */
__global__ void noalloc_setup(nraps_device_problem p, uint64_t generation, unsigned char* base) {
    GenState* st = reinterpret_cast<GenState*>(base);
    Flags* fl = reinterpret_cast<Flags*>(base + sizeof(GenState));
    float* f = reinterpret_cast<float*>(base + 256);
    const uint32_t M = p.mattypes, G = p.energygroups, nx = M * G;
    float* nsf = f;
    float* nsfs = nsf + NOALLOC_MAX_XS;
    float* pabs = nsfs + NOALLOC_MAX_XS;
    float* chi = pabs + NOALLOC_MAX_XS;
    float* phys = chi + NOALLOC_MAX_XS;
    if (blockIdx.x == 0) {
        for (uint32_t i = threadIdx.x; i < nx; i += blockDim.x) {
            nsf[i] = p.nut[i] * p.sigf[i];
            nsfs[i] = nsf[i] * p.inv_sigtr[i];
            pabs[i] = p.siga[i] * p.inv_sigtr[i];
        }
        for (uint32_t m = threadIdx.x; m < M; m += blockDim.x) {
            float c = 0.0f;
            for (uint32_t g = 0; g < G; ++g) { c += p.chit[m + M * g]; chi[m * G + g] = c; }
        }
        for (uint32_t j = threadIdx.x; j < nx; j += blockDim.x) {
            uint32_t m = j / G, g = j % G, xs = m + M * g;
            float cum[NR_MAXG];
            float c = 0.0f;
            for (uint32_t e = 0; e < G; ++e) {
                float s = p.scat_matrix[(uint64_t)G * G * m + (uint64_t)G * g + e];
                if (e == g) s = s - p.mu[xs] * p.sigs[xs];
                if (s < 0.0f) s = 0.0f;
                c = c + s; cum[e] = c;
            }
            for (uint32_t e = 0; e < G; ++e) phys[(m * G + g) * G + e] = (c > 0.0f) ? cum[e] / c : 1.0f;
        }
        if (threadIdx.x == 0) {
            GenState z = {};
            z.gen = generation;
            z.k = 1.0;
            z.inv_kf = 1.0f;
            *st = z;
        }
    }
    /* inputs that would index out of range are reported, not followed */
    uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < p.n_cells; c += stride)
        if (p.matid[c] >= M) atomicOr(&fl->bad, NOALLOC_BAD_MAT);
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < p.n_fuel; i += stride)
        if (p.fuel_indices[i] >= p.n_cells) atomicOr(&fl->bad, NOALLOC_BAD_FUEL);
}

__global__ void noalloc_finish(const unsigned char* base, uint64_t histories, double* d_k, uint32_t* d_error) {
    const GenState* st = reinterpret_cast<const GenState*>(base);
    d_k[0] = nr_unfix(st->kq) / (double)histories;
    if (d_error) d_error[0] = st->error;
}

}  // namespace

extern "C" int nraps_physics_generation_noalloc(const nraps_device_problem* p, uint64_t seed,
                                                uint64_t generation, uint64_t max_events,
                                                double* d_tally, double* d_k, uint32_t* d_error,
                                                void* stream) {
    using nraps_host::set_error;
    if (!p || !d_tally || !d_k) { set_error("NULL argument"); return NRAPS_ERR_INVALID; }
    const nraps_device_problem& q = *p;
    if (!q.sigt || !q.sigs || !q.mu || !q.siga || !q.sigf || !q.nut || !q.chit || !q.scat_matrix ||
        !q.inv_sigtr || !q.matid || !q.delta_x || !q.mesh_left || !q.mesh_right || !q.fuel_indices) {
        set_error("a device input pointer is NULL");
        return NRAPS_ERR_INVALID;
    }
    if (q.mattypes == 0 || q.energygroups == 0 || q.n_cells == 0 || q.n_fuel == 0 || q.histories == 0) {
        set_error("empty problem");
        return NRAPS_ERR_INVALID;
    }
    if (q.energygroups > NR_MAXG) { set_error("at most 16 energy groups"); return NRAPS_ERR_INVALID; }
    uint64_t nx = (uint64_t)q.mattypes * q.energygroups;
    if (nx > NOALLOC_MAX_XS || nx * q.energygroups > NOALLOC_MAX_SCAT) {
        set_error("MatTypes*EnergyGroups exceeds 1024 or MatTypes*EnergyGroups^2 exceeds 16384, "
                  "the limits of the fixed working array of the no-allocation entry point");
        return NRAPS_ERR_INVALID;
    }
    if (q.histories >= (1ULL << 32)) { set_error("at most 2^32-1 histories"); return NRAPS_ERR_INVALID; }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) { set_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e)); return NRAPS_ERR_NO_DEVICE; }
    if (dev < 0 || dev >= MAX_DEVICES) { set_error("device ordinal beyond 63"); return NRAPS_ERR_INVALID; }
    unsigned char* base;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_addr[dev]) {
            void* ptr = nullptr;
            e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
            if (e != cudaSuccess || !ptr) {
                set_error(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
                return NRAPS_ERR_CUDA;
            }
            g_addr[dev] = static_cast<unsigned char*>(ptr);
        }
        base = g_addr[dev];
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    /* the validation flags start at zero before any block can set one */
    e = cudaMemsetAsync(base + sizeof(GenState), 0, sizeof(Flags), s);
    if (e != cudaSuccess) { set_error(std::string("flag clear: ") + cudaGetErrorString(e)); return NRAPS_ERR_CUDA; }
    noalloc_setup<<<64, 256, 0, s>>>(q, generation, base);
    e = cudaGetLastError();
    if (e != cudaSuccess) { set_error(std::string("setup launch: ") + cudaGetErrorString(e)); return NRAPS_ERR_CUDA; }
    Flags fl{0};
    e = cudaMemcpyAsync(&fl, base + sizeof(GenState), sizeof fl, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { set_error(std::string("setup: ") + cudaGetErrorString(e)); return NRAPS_ERR_CUDA; }
    if (fl.bad & NOALLOC_BAD_MAT) { set_error("a matid is not below MatTypes"); return NRAPS_ERR_INVALID; }
    if (fl.bad & NOALLOC_BAD_FUEL) { set_error("a fuel index is not below n_cells"); return NRAPS_ERR_INVALID; }

    const uint32_t M = q.mattypes, G = q.energygroups;
    float* f = reinterpret_cast<float*>(base + 256);
    PlainArgs<float> a{};
    a.sigt = q.sigt; a.sigs = q.sigs; a.siga = q.siga; a.inv_sigtr = q.inv_sigtr;
    a.nsf = f; a.nsf_sigtr = f + NOALLOC_MAX_XS; a.pabs = f + 2 * NOALLOC_MAX_XS;
    a.scat = q.scat_matrix; a.chi_cdf = f + 3 * NOALLOC_MAX_XS; a.phys_cdf = f + 4 * NOALLOC_MAX_XS;
    a.left = q.mesh_left; a.right = q.mesh_right; a.dx = q.delta_x;
    a.mat = q.matid; a.fuel = q.fuel_indices;
    a.M = M; a.G = G; a.nc = q.n_cells; a.nfuel = q.n_fuel;
    a.dx_fuel = 0.0f; a.boundl = q.boundl; a.boundr = q.boundr;
    a.base_seed = seed; a.n_hist = q.histories; a.N = q.histories;
    a.max_events = max_events ? max_events : (1ULL << 24);
    a.st = reinterpret_cast<GenState*>(base);
    a.tally = d_tally;
    a.bank[0] = a.bank[1] = nullptr;
    a.records = nullptr;
    e = cudaMemsetAsync(d_tally, 0, (size_t)G * q.n_cells * sizeof(double), s);
    if (e != cudaSuccess) { set_error(std::string("tally clear: ") + cudaGetErrorString(e)); return NRAPS_ERR_CUDA; }
    if (launch_plain<float>(a, NRAPS_MODE_PHYSICS, 256, s) < 0) {
        set_error(std::string("transport launch: ") + cudaGetErrorString(cudaGetLastError()));
        return NRAPS_ERR_CUDA;
    }
    noalloc_finish<<<1, 1, 0, s>>>(base, q.histories, d_k, d_error);
    e = cudaGetLastError();
    if (e != cudaSuccess) { set_error(std::string("finish launch: ") + cudaGetErrorString(e)); return NRAPS_ERR_CUDA; }
    return NRAPS_OK;
}
