/*
 * engine.cuh — device-side structures shared by the engine's translation units.
 *
 * HBM layout of one problem ("session"):
 *   tables   one packed buffer: cross sections per (material, group) in the
 *            transport precision T, cumulative chi and scatter CDFs, the cell
 *            mesh (left, right, width, material) and the fuel-cell list.
 *   tally    G*cells FP64, [g*cells + c], cleared by the finalize kernel.
 *   sites    unordered fission sites of the running generation (SoA:
 *            x f32, cell u32, group u32, parent u32, seq u32) + per-history
 *            site counts, an exclusive scan of them, and two ordered banks
 *            (nraps_site, 16 B) used ping-pong by generation parity.
 *   GenState scalars read and advanced on the device, so one generation is a
 *            fixed launch sequence that a CUDA graph can replay.
 */
#ifndef NRAPS_ENGINE_CUH
#define NRAPS_ENGINE_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/nraps_gpu.h"

#define NR_MAXG 16            /* groups supported by the kernels            */
#define NR_ERR_CAPACITY 1u    /* GenState.error bits                        */
#define NR_ERR_EMPTY    2u
#define NR_ERR_CAPPED   4u
#define NR_ERR_STALLED  8u    /* a bounded device wait ran out              */

struct GenState {
    uint64_t gen;             /* generation being run                        */
    double   k;               /* k of the previous generation                */
    unsigned long long kq;    /* fixed-point k score of this generation      */
    unsigned long long n_sites; /* unordered sites appended (may exceed cap) */
    unsigned long long n_bank;  /* ordered sites available as source        */
    unsigned long long n_bank_next;
    unsigned int error;
    float inv_kf;             /* (float)(1/k), read by the FP32 event kernels */
    double h_acc;             /* entropy accumulator of the event finalize    */
    /* per-generation counters (zeroed by finalize) */
    unsigned long long collisions, virtual_collisions, crossings, absorbed, leaked, capped;
    /* run totals */
    unsigned long long tot_collisions, tot_virtual, tot_crossings, tot_absorbed,
        tot_leaked, tot_capped, tot_sites, tot_histories;
    /* k over the active generations so far: sum, sum of squares, count */
    double ksum, ksum2;
    unsigned long long nactive;
    /* deferred end of generation (event engine, one instance): the
       generation whose tallies and site histogram still wait to be folded
       (by extra blocks of the next transport launch, or a flush), the k in
       effect during it, its bank size and its entropy accumulator */
    unsigned long long fold_pending, fold_gen, fold_B;
    double fold_k, fold_h;
    unsigned long long pad2;
};

/* Unordered site stream written by the transport kernels. */
struct SiteSink {
    float* x;
    uint32_t* cell;
    uint32_t* group;
    uint32_t* parent;
    uint32_t* seq;
    uint64_t cap;
    uint32_t* count;          /* per history: sites it banked                */
};

template <class T>
struct PlainArgs {
    const T *sigt, *sigs, *siga, *inv_sigtr, *nsf, *nsf_sigtr, *pabs;
    const T *scat;            /* [G*G*m + G*g + g'] raw                       */
    const T *chi_cdf;         /* [m*G + g]                                    */
    const T *phys_cdf;        /* [(m*G + g)*G + g']                           */
    const T *left, *right, *dx;
    const uint8_t* mat;
    const uint64_t* fuel;
    uint32_t M, G;
    uint64_t nc, nfuel;
    T dx_fuel, boundl, boundr;
    uint64_t base_seed, n_hist, N, max_events;
    GenState* st;
    double* tally;
    const nraps_site* bank[2];
    SiteSink sink;
    nraps_history_record* records;
};

struct BankArgs {
    GenState* st;
    SiteSink sink;
    uint64_t n_hist;
    uint32_t* offsets;        /* n_hist                                       */
    uint32_t* block_sums;     /* ceil(n_hist/4096)                            */
    nraps_site* bank[2];
    uint64_t bank_cap;
    uint32_t* hist;           /* entropy histogram, one bin per cell          */
};

struct FinalizeArgs {
    GenState* st;
    double* tally;            /* G*nc                                         */
    const double* nsf64;      /* [m + M*g] nut*sigf in FP64                   */
    const double* dx64;       /* cell widths (the mesh's delta_x)             */
    const uint8_t* mat;
    uint32_t M, G;
    uint64_t nc, N, generations, skip;
    int mode;
    double conv_const;        /* 3565e6*36.2/(200e6*1.602176634e-19*nu*L)    */
    double* flux_acc;         /* G*nc: sum of flux*conversion*fund            */
    double* fs_acc;           /* nc                                           */
    double* flux_sum;         /* G*nc: sum of per-generation tally/(N dx)     */
    double* flux_sq;          /* G*nc                                         */
    double* k64;              /* generations                                  */
    double* entropy;          /* generations                                  */
    const uint32_t* hist;
    uint32_t* hist_w;
    double* partials;         /* 2 * n_blocks                                 */
    uint32_t n_blocks;
    int bank_mode;
    uint64_t bank_cap;
};

/* Launch k<<<g, b, smem, s>>>(args...), with programmatic stream
   serialization when pdl (the kernel must call nrdev::pdl_wait() before it
   touches what the previous kernel in the stream produces or reads). */
template <typename... KArgs, typename... Args>
inline cudaError_t launch_k(bool pdl, void (*k)(KArgs...), dim3 g, dim3 b, size_t smem, cudaStream_t s,
                            Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = g;
    cfg.blockDim = b;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = pdl ? at : nullptr;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k, static_cast<KArgs>(args)...);
}

/* launchers (each returns the number of kernels it launched, <0 on error) */
template <class T>
int launch_plain(const PlainArgs<T>& a, int mode, int block, cudaStream_t s);
int launch_bank_order(const BankArgs& a, cudaStream_t s);
/* offsets[i] = sum(count[0..i)), offsets[n] = total (offsets has n+1 slots) */
/* Load the scan kernels now (lazy module loading would otherwise load them
   inside the first generation that launches them). */
void preload_bank_kernels();
int launch_exclusive_scan(const uint32_t* count, uint64_t n, uint32_t* block_sums, uint32_t* offsets,
                          unsigned long long* total, cudaStream_t s, bool pdl = false);
/* the scan works on tiles of 2^NR_SCAN_TILE_LOG2 counts; up to
   NR_SCAN_CARRY_MAX_TILES tiles it takes two launches, beyond that three */
constexpr int NR_SCAN_TILE_LOG2 = 12;
constexpr uint64_t NR_SCAN_CARRY_MAX_TILES = 4096;
/* per tile of 2^NR_SCAN_TILE_LOG2 counts: offsets relative to the tile's
   start, and tile_sums[tile] = the tile's total (one launch; the consumer
   adds the exclusive scan of tile_sums).  Returns launches (1, or 0 for
   n = 0), or -1. */
int launch_scan_local(const uint32_t* count, uint64_t n, uint32_t* tile_sums, uint32_t* offsets, cudaStream_t s,
                      bool pdl = false);
int launch_finalize(const FinalizeArgs& a, cudaStream_t s);
int launch_pcg_stream(uint64_t seed, const uint64_t* streams, uint64_t n, uint32_t per,
                      uint32_t* out, cudaStream_t s);
int launch_log_eval(const double* x, uint64_t n, double* o64, float* o32, cudaStream_t s);
uint32_t finalize_blocks_for(uint64_t nc);

#endif
