/*
 * event.cuh — event-based Woodcock (delta-tracking) transport engine.
 *
 * One engine runs one generation of every problem instance it holds in a
 * fixed sequence of launches:
 *   pass 0      every source particle is born (from its instance's ordered
 *               fission bank, or the uniform fuel source) and runs up to K
 *               real collisions; survivors are compacted into queue 0
 *               (or, sorted: R rounds of one flight kernel and one
 *               collision kernel over event-type queues);
 *   pass 1..P-1 the queued particles run K more real collisions each and
 *               the survivors are compacted into the other queue;
 *   drain       the last queue runs to completion;
 *   bank        exclusive scan of per-history site counts, then the
 *               unordered sites are scattered to (parent, sequence) order
 *               (ranged launches: each range orders its own sites);
 *   finalize    per-cell FP64 flux/fission-source accumulation, Shannon
 *               entropy, and per-instance k, bank size and generation index.
 *               One instance with a two-half tally, one pass, few cells:
 *               the last block of the bank scatter closes the generation (k,
 *               bank size, generation index), and the fold (flux, fission
 *               source, entropy) runs in extra blocks of the next transport
 *               launch, which the SMs take up as the transport's last
 *               histories leave them idle; a flush folds what is left.
 * Every particle owns a PCG32 stream (seed of its instance and generation,
 * stream = its history index within the instance), so the result does not
 * depend on K, P, the block size, or which other instances share the batch.
 */
#ifndef NRAPS_EVENT_CUH
#define NRAPS_EVENT_CUH
#include <string>
#include <vector>

#include "arena.hpp"
#include "engine.cuh"

/* Per-instance device buffers owned by the caller (a session or a batch). */
struct EvBuffers {
    GenState* st;
    double* tally;                         /* G*nc, or two halves of G*nc   */
    uint32_t tally_shift = 0;              /* bin b of a half at
                                              tally[b << tally_shift]        */
    uint64_t tally_stride = 0;             /* (G*nc) << tally_shift: generation
                                              g scores into half g & 1 (the
                                              fold of one generation can then
                                              run beside the next one's
                                              transport); 0: one tally      */
    double *flux_acc, *fs_acc, *flux_sum, *flux_sq;
    double *k64, *entropy;                 /* generations                    */
    nraps_site* bank[2];                   /* BANK mode ordered banks        */
    uint64_t bank_cap;
    uint32_t* hist;                        /* ev_hist_words(nc) (BANK mode)  */
    uint64_t generations, skip;
    uint64_t seed;
};

/* Site counters of the entropy histogram.  An instance with few cells keeps
   them 128 B apart (counter of cell c at word c << 5), so the additions to
   its hot fuel cells spread over the L2 slices; up to 2M cells one counter
   per 32 B sector (word c << 3: with eight to a sector, the additions of a
   localised source's hot cells queued on a few sectors -- a 200,000-cell
   slab's generation took 2.35 ms against 2.15 ms spread out); beyond that
   densely. */
#define EV_HIST_SPREAD_MAX_CELLS 4096u
#define EV_HIST_SECTOR_MAX_CELLS 2097152u
__host__ __device__ inline uint32_t ev_hist_shift(uint64_t nc) {
    return nc <= EV_HIST_SPREAD_MAX_CELLS ? 5u : (nc <= EV_HIST_SECTOR_MAX_CELLS ? 3u : 0u);
}
__host__ __device__ inline uint64_t ev_hist_words(uint64_t nc) { return nc << ev_hist_shift(nc); }

/* FP64 tally bins one per 32 B sector (bin b at word b << 2): with several
   bins to a sector the reductions of a launch queue on fewer L2 sectors.
   On a 2,000-cell, 4-group slab the transport's time depended on where the
   tally lay (0.093-0.118 ms across 4 KB offsets; flat at 0.092-0.093 ms
   spread out); on a 200,000-cell, 8-group slab spreading took a generation
   of 10M histories from 4.09 to 2.37 ms.  Tallies of more than 2M bins (64 MB
   spread out, half the L2) stay dense. */
#define EV_TALLY_SPREAD_MAX_BINS 2097152u
__host__ __device__ inline uint32_t ev_tally_shift(uint64_t bins) { return bins <= EV_TALLY_SPREAD_MAX_BINS ? 2u : 0u; }

struct EvParams {
    uint32_t block = 256;   /* threads per block of the transport passes       */
    uint32_t K = 4;         /* real collisions per particle per queue pass     */
    uint32_t passes = 3;    /* queue passes before the drain pass; 0 = one
                               pass that runs every particle to its end      */
    uint32_t sort = 0;      /* > 0: the sorted transport (single instance): this
                               many rounds of flight and collision kernels over
                               event-type queues, then one pass for the rest */
    uint32_t range = 0;     /* > 0 (one pass): a ranged launch, one block per
                               range of this many histories of one instance,
                               that instance's tables in shared memory     */
    uint32_t tail = 0;      /* a warp of a non-final pass whose input is used
                               up and that holds fewer live particles than
                               this re-queues them and leaves, so the next
                               pass runs the stragglers in full warps       */
};

class EventEngine {
public:
    EventEngine();
    ~EventEngine();
    EventEngine(const EventEngine&) = delete;
    EventEngine& operator=(const EventEngine&) = delete;

    /* mode (PHYSICS/BANK), exact_log, max_events; keeps the instances. */
    int configure(const nraps_opts& o, std::string& err);
    /* Build tables for one problem; returns the instance index, or -1. */
    int add_instance(const nraps_problem& p, const EvBuffers& b, std::string& err);
    void clear_instances();
    /* Allocate later instances' tables stream-ordered from `pool` on `s`
       (the request server admits and retires instances every step). */
    void set_pool(cudaMemPool_t pool, cudaStream_t s);
    /* Take every buffer of up to DeviceArena::ITEM_MAX bytes from `a` (each
       on its own 64 KB); `a` must outlive the engine. */
    void set_arena(DeviceArena* a);
    /* Drop one instance (later instances shift down by one). */
    void remove_instance(uint32_t idx);
    uint32_t n_instances() const;
    /* Upload descriptors and size the shared queues/site slabs. */
    int commit(cudaStream_t s, std::string& err);
    /* One generation of every instance; returns kernels launched, <0 on error. */
    int enqueue_generation(cudaStream_t s, bool with_finalize = true, cudaEvent_t t0 = nullptr,
                           cudaEvent_t t1 = nullptr);
    uint64_t launches_per_generation() const;
    /* Fold a generation left pending by a deferred end of generation (a
       no-op launch-wise when none can be pending); returns kernels
       launched, <0 on error.  Called before anything reads the flux,
       fission source or entropy. */
    int flush_fold(cudaStream_t s);
    /* Per-history records of instance 0 (trace), or nullptr. */
    void set_records(nraps_history_record* rec);
    /* Device scan offsets (n_total+1) of the last generation, for traces. */
    const uint32_t* offsets() const;
    uint64_t n_total() const;
    /* Batch-level counters (collisions etc.) when the engine has several
       instances; a single instance counts into its own GenState. */
    GenState* batch_stats() const;
    /* Device bytes of the shared (per-generation) buffers. */
    uint64_t shared_bytes() const;
    /* Device bytes one instance's tables need. */
    static uint64_t table_bytes(const nraps_problem& p);

    EvParams params;
    /* Size the persistent grid for the current params (after a change). */
    int size_grid();

    struct Impl;
private:
    Impl* impl_;
};
#endif
