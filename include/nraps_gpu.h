/*
 * nraps_gpu.h — C ABI of the GB300 Monte Carlo k-eigenvalue engine.
 *
 * This is the drop-in boundary for NRAPS's CPU solver
 *   pub fn monte_carlo(variables: &Variables, xsdata: &XSData, delta_x: &DeltaX,
 *                      meshid: &Vec<Mesh>, fuel_indices: &Vec<usize>,
 *                      mut k_new: f32) -> SolutionResults
 * (reference src/mc_code.rs:276-283, caller src/main.rs:337), plus its input
 * producers process_input (src/process_input.rs:85) and mesh_gen
 * (src/main.rs:85).  Plain pointers and sizes only; no C++ or torch types.
 *
 * Conventions
 *  - Every function returns an int status (NRAPS_OK == 0).  Nothing throws or
 *    aborts across this boundary; nraps_last_error() gives the message of the
 *    last failure on a context (thread-local text for calls without one).
 *  - Inputs are borrowed for the duration of the call (the reference borrows
 *    them immutably).  Result buffers are allocated by the caller with the
 *    exact SolutionResults shapes (src/main.rs:77-83).  A context owns every
 *    device allocation it makes and frees it in nraps_destroy.
 *  - One context per host thread, or serialise calls on a context.
 *  - Cross-section arrays are the reference's flat layout: value of material m
 *    in group g at [m + M*g]; scattering g->g' of material m at
 *    [G*G*m + G*g + g'] (src/main.rs:46-56, src/process_input.rs:114-150).
 */
#ifndef NRAPS_GPU_H
#define NRAPS_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NRAPS_ABI_VERSION 6u

/* ---- status codes ------------------------------------------------------- */
#define NRAPS_OK              0
#define NRAPS_ERR_INVALID     1  /* bad argument or inconsistent problem        */
#define NRAPS_ERR_CUDA        2  /* a CUDA runtime call failed                  */
#define NRAPS_ERR_NOMEM       3  /* device or host allocation failed            */
#define NRAPS_ERR_NO_DEVICE   4  /* no CUDA device / extension not usable       */
#define NRAPS_ERR_IO          5  /* input file could not be read                */
#define NRAPS_ERR_PARSE       6  /* input file value could not be parsed        */
#define NRAPS_ERR_CAPACITY    7  /* fission bank or particle queue overflowed   */
#define NRAPS_ERR_EMPTY_BANK  8  /* fission bank empty: no source for next gen  */
#define NRAPS_ERR_NOT_FOUND   9  /* unknown request / session id                */
#define NRAPS_ERR_PENDING    10  /* request admitted but not finished yet       */
#define NRAPS_ERR_CAPPED     11  /* a history hit the per-history event cap     */
#define NRAPS_ERR_REJECTED   12  /* request does not fit the memory budget      */
#define NRAPS_ERR_UNSUPPORTED 13 /* input selects a solver this library lacks   */

/* ---- solver options ----------------------------------------------------- */
/* mode: which algorithm the generation loop follows.                        */
#define NRAPS_MODE_COMPAT   0  /* the reference's algorithm, quirks included:
                                  fresh uniform fuel source every generation,
                                  stale xs index after scatter, one uniform per
                                  binary-search probe, N+T histories, Q5 fund. */
#define NRAPS_MODE_PHYSICS  1  /* same fresh source, quirks fixed.           */
#define NRAPS_MODE_BANK     2  /* fission bank + source normalisation + entropy
                                  (power iteration on the fission source).   */
/* precision: arithmetic of the transport (flights, positions, cross
   sections).  Tallies, k and entropy always accumulate in 64 bits.         */
#define NRAPS_PREC_FP64     0
#define NRAPS_PREC_FP32     1
/* tracking */
#define NRAPS_TRACK_SURFACE  0 /* plain history-per-thread, surface tracking
                                  across every tally cell, track-length tallies */
#define NRAPS_TRACK_WOODCOCK 1 /* event-based delta tracking, SoA particle queues,
                                  collision estimators (PHYSICS/BANK, FP32 only) */
/* events_per_pass value: a single transport pass, no re-queueing */
#define NRAPS_ONE_PASS 0xFFFFFFFFu

typedef struct nraps_opts {
    uint32_t abi_version;        /* must be NRAPS_ABI_VERSION                  */
    int32_t  device;             /* CUDA ordinal; -1 = the current device      */
    uint64_t seed;               /* base seed of every PCG32 stream            */
    int32_t  mode;               /* NRAPS_MODE_*                                */
    int32_t  precision;          /* NRAPS_PREC_*                                */
    int32_t  tracking;           /* NRAPS_TRACK_*                               */
    uint32_t compat_threads;     /* COMPAT: the reference's T (histories per
                                    generation = N + T); 0 = exactly N        */
    uint64_t max_events;         /* per-history event cap; 0 = 1<<24           */
    uint32_t block_size;         /* 0 = tuned default                          */
    uint32_t events_per_pass;    /* WOODCOCK: real collisions a particle runs
                                    before it is re-queued; 0 = tuned default;
                                    NRAPS_ONE_PASS = no re-queueing: one pass
                                    runs every particle to its end          */
    uint32_t passes;             /* WOODCOCK: queue passes per generation before
                                    the drain pass; 0 = tuned default         */
    uint32_t use_graphs;         /* 1 = replay each generation as a CUDA graph */
    double   bank_factor;        /* bank capacity = bank_factor*N (+slack); 0=3 */
    uint32_t entropy_bins;       /* Shannon-entropy bins: must be 0 (one per cell) */
    uint32_t exact_log;          /* WOODCOCK: 1 = flights use the shared software
                                    logarithm (bit-reproducible on a CPU);
                                    0 = the hardware log2 unit (fast)         */
    uint32_t tail_lanes;         /* WOODCOCK: when a pass's input is used up, a
                                    warp with fewer live particles re-queues
                                    them for the next pass (needs passes >= 1);
                                    0 = off                                   */
    uint32_t sort_rounds;        /* WOODCOCK, one instance: 1..16 = the sorted
                                    transport (particles in event-type queues
                                    in HBM: this many rounds of one flight
                                    kernel and one collision kernel, then one
                                    pass runs the survivors to their ends);
                                    0 = tuned                                 */
    uint32_t initial_source;     /* BANK: 0 = the reference's uniform fuel source
                                    for generation 0; 1 = N sites drawn
                                    (deterministically) from the fission source
                                    of the deterministic diffusion solution  */
    uint32_t range_len;          /* WOODCOCK, one pass: 64..32768 = a ranged
                                    launch, one block per range of this many
                                    histories of one instance, that instance's
                                    tables in shared memory (BANK: the range
                                    orders its own sites); 0 = tuned /
                                    persistent                               */
    uint32_t reserved[2];
} nraps_opts;

/* Fill *o with the defaults (FP64 surface tracking, COMPAT, seed 1). */
void nraps_opts_default(nraps_opts* o);

/* ---- problem description (mirrors the reference structs) --------------- */
/* Variables (src/main.rs:22-39).  rodpitch is the water gap, i.e. the value
   process_input stores after subtracting the rod diameter (process_input.rs:102). */
typedef struct nraps_variables {
    uint32_t analk, mattypes, energygroups;
    uint64_t generations, histories, skip;
    uint32_t numass, numrods;
    float    roddia, rodpitch;
    uint64_t mpfr, mpwr;
    float    boundl, boundr;
} nraps_variables;

/* DeltaX (src/main.rs:41-44) */
typedef struct nraps_delta_x { float fuel, water; } nraps_delta_x;

/* XSData (src/main.rs:46-56): n_xs = M*G entries each, scat_matrix M*G*G. */
typedef struct nraps_xsdata {
    const float *sigt, *sigs, *mu, *siga, *sigf, *nut, *chit;
    const float *scat_matrix;    /* [G*G*m + G*g + g']                        */
    const float *inv_sigtr;      /* 1/(sigt - mu*sigs) (process_input.rs:152-156) */
    uint64_t n_xs, n_scat;
} nraps_xsdata;

/* Vec<Mesh> (src/main.rs:68-75) as structure-of-arrays of n_cells cells. */
typedef struct nraps_mesh {
    const uint8_t* matid;
    const float *delta_x, *mesh_left, *mesh_right;
    uint64_t n_cells;
} nraps_mesh;

/* Everything one monte_carlo call borrows. */
typedef struct nraps_problem {
    nraps_variables variables;
    nraps_xsdata    xsdata;
    nraps_delta_x   delta_x;
    nraps_mesh      mesh;
    const uint64_t* fuel_indices;   /* Vec<usize> from mesh_gen                */
    uint64_t        n_fuel;
    float           k_new;          /* initial k                               */
} nraps_problem;

/* ---- results (SolutionResults, src/main.rs:77-83, plus FP64 extras) ----- */
typedef struct nraps_stats {
    double   k_mean, k_sigma;         /* over active generations, FP64        */
    uint64_t histories, collisions, virtual_collisions, crossings;
    uint64_t absorbed, leaked, capped, sites;
    double   transport_ms;            /* device time of the transport kernels  */
    double   total_ms;                /* device time of all generations        */
    uint64_t transport_launches;
    uint64_t gpu_launches;            /* kernels this library launched         */
} nraps_stats;

typedef struct nraps_result {
    /* SolutionResults: caller-allocated, f32, row-major [g*cells + c]        */
    float* flux;              /* G*cells                                      */
    float* assembly_average;  /* G*cells                                      */
    float* fission_source;    /* cells                                        */
    float* k;                 /* generations                                  */
    float* k_fund;            /* generations                                  */
    /* optional FP64 extras (NULL = not wanted)                               */
    double* k64;              /* generations: per-generation k                */
    double* entropy;          /* generations: Shannon entropy of the source   */
    double* flux_mean;        /* G*cells: mean per-generation flux (active)   */
    double* flux_sem;         /* G*cells: standard error of flux_mean         */
    nraps_stats* stats;
} nraps_result;

/* ---- per-history trace (parity) ----------------------------------------- */
#define NRAPS_FATE_ABSORBED 0
#define NRAPS_FATE_LEAKED   1
#define NRAPS_FATE_CAPPED   2
typedef struct nraps_history_record {
    uint32_t collisions;   /* interaction events                              */
    uint32_t crossings;    /* cell faces crossed                              */
    uint32_t reflections;  /* outer-boundary reflections                      */
    uint32_t segments;     /* particle_travel calls (flight resamples)        */
    int32_t  fate;         /* NRAPS_FATE_*                                    */
    uint32_t final_cell;
    uint32_t final_group;
    uint32_t n_sites;      /* fission sites banked (BANK mode)                */
    double   final_x;
    double   track;        /* sum of tallied track lengths, in history order  */
    double   nsf_track;    /* sum of nu*sigf*track (track-length k score)     */
    uint64_t draws;        /* PCG32 outputs consumed                          */
} nraps_history_record;

/* A fission site (BANK mode source point). */
typedef struct nraps_site {
    float    x;
    uint32_t cell;
    uint32_t group;
    uint32_t pad;
} nraps_site;

/* ---- context ------------------------------------------------------------ */
typedef struct nraps_ctx nraps_ctx;
typedef struct nraps_session nraps_session;

int  nraps_create(nraps_ctx** out, const nraps_opts* opts);
void nraps_destroy(nraps_ctx* ctx);
const char* nraps_last_error(const nraps_ctx* ctx);
int  nraps_set_opts(nraps_ctx* ctx, const nraps_opts* opts);
int  nraps_get_opts(const nraps_ctx* ctx, nraps_opts* out);
/* Number of kernels this context has launched since creation. */
uint64_t nraps_launch_count(const nraps_ctx* ctx);
/* The cudaStream_t (as void*) every call on this context is ordered on. */
void* nraps_ctx_stream(nraps_ctx* ctx);

/* The drop-in: replaces monte_carlo (src/mc_code.rs:276-380).  Runs
   variables->generations generations synchronously, host buffers in/out. */
int nraps_monte_carlo(nraps_ctx* ctx,
                      const nraps_variables* variables,
                      const nraps_xsdata* xsdata,
                      const nraps_delta_x* delta_x,
                      const nraps_mesh* meshid,
                      const uint64_t* fuel_indices, uint64_t n_fuel,
                      float k_new,
                      nraps_result* out);

/* Same, with the inputs bundled. */
int nraps_solve(nraps_ctx* ctx, const nraps_problem* problem, nraps_result* out);

/* Device-resident session: tables and banks stay in HBM between calls.
   run() enqueues generations on the context's stream and returns at once.
   A WOODCOCK BANK session with one pass and few cells may leave the last
   enqueued generation's fold (flux, fission source, entropy) pending: the
   next generation's transport launch runs it, and sync(), results() and
   timing() complete it first.  flush() enqueues it on the context's stream
   without waiting (nothing when none is pending). */
int  nraps_session_create(nraps_ctx* ctx, const nraps_problem* problem, nraps_session** out);
int  nraps_session_run(nraps_session* s, uint64_t n_generations);
int  nraps_session_flush(nraps_session* s);
int  nraps_session_sync(nraps_session* s);
int  nraps_session_results(nraps_session* s, nraps_result* out);
/* Time each generation with CUDA events on the context's stream (turns CUDA
   graph replay off for this session). */
int  nraps_session_set_profile(nraps_session* s, int on);
/* Sync, then report accumulated device time of the transport phases and of
   whole generations (profile mode), transport launches, real collisions and
   histories simulated so far. */
int  nraps_session_timing(nraps_session* s, double* transport_ms, double* total_ms,
                          uint64_t* transport_launches, uint64_t* collisions,
                          uint64_t* histories);
/* WOODCOCK sessions: the launch shape in use.  With block_size,
   events_per_pass and passes all 0 in the options, the first inactive
   generations each try one candidate shape (synchronously) and the one with
   the least time per real collision is kept; results do not depend on the
   shape.  The context remembers the choice per problem shape (MatTypes,
   EnergyGroups, cells, Histories, mode, exact_log): a later session of the
   same shape on the same context starts with it and tries nothing
   (n_tried = 0), so repeated nraps_monte_carlo calls tune once.  tried_ms
   receives the whole-generation time of each candidate tried (up to
   tried_cap). */
int  nraps_session_tuning(nraps_session* s, uint32_t* block, uint32_t* events_per_pass,
                          uint32_t* passes, uint32_t* tail_lanes, uint32_t* sort_rounds, uint32_t* range_len,
                          uint32_t* n_tried, float* tried_ms, uint32_t tried_cap);
/* generations completed so far (enqueued work included after sync) */
uint64_t nraps_session_generation(const nraps_session* s);
void nraps_session_destroy(nraps_session* s);

/* One generation with per-history records, for parity with a CPU model.
   generation: index mixed into the PCG seed.  k: k of the previous generation.
   sites_in/n_sites_in: BANK-mode source (NULL = the fresh uniform fuel source).
   records: n_records entries (one per history simulated).
   tally: G*cells FP64 track-length (or collision-estimator) tally, or NULL.
   sites_out/cap_sites_out/n_sites_out: ordered bank produced, or NULL.
   k_fixed_out: the generation's k score in 2^-32 fixed point (sum over all
   scores of round(score * 2^32)), or NULL.  */
int nraps_trace_generation(nraps_ctx* ctx, const nraps_problem* problem,
                           uint64_t generation, double k,
                           const nraps_site* sites_in, uint64_t n_sites_in,
                           nraps_history_record* records, uint64_t n_records,
                           double* tally,
                           nraps_site* sites_out, uint64_t cap_sites_out,
                           uint64_t* n_sites_out, uint64_t* k_fixed_out);

/* Raw PCG32 stream (rand.rs PCG32 seeded with seed/stream), for RNG parity. */
int nraps_pcg32_stream(nraps_ctx* ctx, uint64_t seed, const uint64_t* streams,
                       uint64_t n_streams, uint32_t per_stream, uint32_t* out);

/* The shared natural logarithm evaluated on the device (FP64 and FP32). */
int nraps_log_eval(nraps_ctx* ctx, const double* x, uint64_t n, double* out64,
                   float* out32);

/* ---- host front end (no GPU) --------------------------------------------
   process_input (src/process_input.rs:85-175) and mesh_gen (src/main.rs:85-143).
   Arrays inside the returned structures are owned by the library; free them
   with nraps_input_free / nraps_meshbuf_free. */
typedef struct nraps_input {
    nraps_variables variables;
    nraps_delta_x   delta_x;
    float *sigt, *sigs, *mu, *siga, *sigf, *nut, *chit, *scat_matrix, *inv_sigtr;
    uint64_t n_sigt, n_sigs, n_mu, n_siga, n_sigf, n_nut, n_chit, n_scat, n_inv_sigtr;
    uint8_t* matid;           /* MatID entries                                 */
    uint64_t n_matid;
    int32_t  solution;        /* process_input's bool: Solution != 1           */
    int32_t  solver;          /* 0 LinAlg, 1 Gaussian, 2 Jacobian, 3 SR       */
} nraps_input;

typedef struct nraps_meshbuf {
    uint8_t* matid;
    float *delta_x, *mesh_left, *mesh_right;
    uint64_t n_cells;
    uint64_t* fuel_indices;
    uint64_t n_fuel;
} nraps_meshbuf;

int  nraps_process_input(const char* path, nraps_input** out);
/* Parse an in-memory input text (same rules as nraps_process_input). */
int  nraps_process_input_text(const char* text, uint64_t len, nraps_input** out);
void nraps_input_free(nraps_input* in);
int  nraps_mesh_gen(const uint8_t* matid, uint64_t n_matid,
                    const nraps_variables* variables, const nraps_delta_x* delta_x,
                    nraps_meshbuf** out);
void nraps_meshbuf_free(nraps_meshbuf* m);
/* Fill a problem view from parsed input + mesh (pointers alias them). */
int  nraps_problem_view(const nraps_input* in, const nraps_meshbuf* mesh, nraps_problem* out);

/* ---- batched instances ----------------------------------------------------
   Build-defined (the reference solves one problem per call).  Independent
   slab problems of any size advance together: one launch sequence of the
   WOODCOCK engine per generation for all of them (CUDA-graph replayed with
   opts.use_graphs).  The context's options apply to every instance; seeds[i]
   seeds instance i (NULL: opts.seed + i).  Every instance's results are the
   ones it would get alone with the same seed. */
typedef struct nraps_batch nraps_batch;
int  nraps_batch_create(nraps_ctx* ctx, const nraps_problem* problems, uint32_t n,
                        const uint64_t* seeds, nraps_batch** out);
int  nraps_batch_run(nraps_batch* b, uint64_t n_generations);      /* async */
int  nraps_batch_sync(nraps_batch* b);
int  nraps_batch_results(nraps_batch* b, uint32_t i, nraps_result* out);
/* device ms of all generations run, histories simulated, real collisions */
int  nraps_batch_timing(nraps_batch* b, double* ms, uint64_t* histories, uint64_t* collisions);
/* The batch's launch shape (a ranged pass: threads per block, histories per
   range).  With block_size, range_len, events_per_pass and passes all 0 in
   the options, the first inactive generations (as many as the smallest Skip
   of the batch allows, at most 12) each try one of blocks of 128, 256 and
   512 threads with ranges of 1024..8192 histories, synchronously, and the
   shape with the least time per real collision is kept; every result is the
   same whatever the shape.  tried_ms receives each tried generation's time. */
int  nraps_batch_tuning(nraps_batch* b, uint32_t* block, uint32_t* range_len, uint32_t* n_tried,
                        float* tried_ms, uint32_t tried_cap);
uint32_t nraps_batch_size(const nraps_batch* b);
void nraps_batch_destroy(nraps_batch* b);

/* ---- request server (continuous batching) ---------------------------------
   Build-defined.  submit() queues a k-eigenvalue solve; each step() admits
   queued requests while device slots and the HBM budget allow, runs one
   generation of every admitted request together, and retires requests whose
   standard error of k (over their active generations, at least min_active)
   is at most sigma_k_target, or that reached their Generations cap.  Fission
   banks and tallies stay on the device from admission until release(). */
#define NRAPS_REQ_QUEUED   0
#define NRAPS_REQ_RUNNING  1
#define NRAPS_REQ_DONE     2
#define NRAPS_REQ_REJECTED 3
typedef struct nraps_server_opts {
    uint64_t hbm_budget_bytes;   /* admission limit; 0 = 120 GiB               */
    double   sigma_k_target;     /* absolute standard error of k (50 pcm = 5e-4) */
    uint32_t min_active;         /* active generations before the test         */
    uint32_t max_slots;          /* requests on the device at once, <= 4095    */
    uint32_t reserved[4];
} nraps_server_opts;
typedef struct nraps_request_info {
    uint64_t id;
    int32_t  state;              /* NRAPS_REQ_*                                */
    int32_t  status;             /* NRAPS_OK, or why it stopped                */
    uint64_t generations_run;
    uint64_t histories_per_generation;
    double   k_mean, k_sigma;    /* over the active generations                */
    double   t_submit, t_admit, t_done;  /* seconds on nraps_server_clock      */
} nraps_request_info;
typedef struct nraps_server nraps_server;
void nraps_server_opts_default(nraps_server_opts* o);
int  nraps_server_create(nraps_ctx* ctx, const nraps_server_opts* o, nraps_server** out);
/* copies the problem; NRAPS_ERR_REJECTED if it can never fit the budget */
int  nraps_server_submit(nraps_server* s, const nraps_problem* p, uint64_t seed, uint64_t* req_id);
/* One step: admit waiting requests in arrival order while a slot and the
   HBM budget allow, run every admitted request together for as many
   generations as no request could retire within (each needs
   max(2, min_active) active generations before its k can count as
   converged, and stops at its Generations), at most 4, then read back every
   request's k statistics and retire the converged (or capped) ones.
   Admitted requests' buffers come from the context's stream-ordered memory
   pool, so admissions and retirements do not synchronise the device. */
int  nraps_server_step(nraps_server* s, uint32_t* n_running, uint32_t* n_finished);
/* Ids of requests retired since the last call (oldest first), at most cap;
   *n receives how many were written. */
int  nraps_server_finished(nraps_server* s, uint64_t* ids, uint32_t cap, uint32_t* n);
/* NRAPS_ERR_PENDING while queued/running; fills out (may be NULL) when done */
int  nraps_server_poll(nraps_server* s, uint64_t req_id, nraps_result* out, nraps_request_info* info);
int  nraps_server_release(nraps_server* s, uint64_t req_id);
int  nraps_server_stats(nraps_server* s, uint64_t* histories, uint64_t* completed, uint32_t* running,
                        uint32_t* waiting, double* busy_ms, uint64_t* bytes_in_use);
double nraps_server_clock(const nraps_server* s);
void nraps_server_destroy(nraps_server* s);

/* ---- one generation without allocating ----------------------------------
   No counterpart in the reference: for callers that cannot allocate device
   memory themselves at call time (an application whose device memory is all
   handed out by its own pool, a pre-planned memory layout, a job that must
   not fail on an allocation midway).  Runs one PHYSICS-mode generation of the
   plain FP32 kernel on problem arrays that are already on the device and
   writes the FP64 track-length tally (G*n_cells, row-major [g*n_cells + c])
   and k (one double) into caller buffers on the caller's stream.  Its working
   state lives in a fixed array inside the library (about 80 KB per device,
   kept until the process exits); nothing is allocated.  Limits:
   MatTypes*EnergyGroups <= 1024, MatTypes*EnergyGroups^2 <= 16384,
   EnergyGroups <= 16; larger problems are rejected with NRAPS_ERR_INVALID.
   The first call on a device looks up the array's device address; make it
   before any stream capture.  Every call checks the device inputs and waits
   for that check (one synchronisation of `stream`), so no call can be made
   while `stream` is being captured.  Calls share the array: calls whose work
   overlaps on the GPU race, so order them; the race includes the input check
   (an overlapping call can make another call fail on its inputs, or pass
   with bad ones).  After the check the call enqueues the generation and returns;
   d_error (may be NULL) receives the generation's error bits (4 = a history
   hit max_events).  Errors are reported through nraps_last_error(NULL). */
typedef struct nraps_device_problem {
    const float *sigt, *sigs, *mu, *siga, *sigf, *nut, *chit, *scat_matrix, *inv_sigtr;
    const uint8_t* matid;
    const float *delta_x, *mesh_left, *mesh_right;
    const uint64_t* fuel_indices;
    uint32_t mattypes, energygroups;
    uint64_t n_cells, n_fuel, histories;
    float boundl, boundr;
} nraps_device_problem;

int nraps_physics_generation_noalloc(const nraps_device_problem* p, uint64_t seed,
                                     uint64_t generation, uint64_t max_events,
                                     double* d_tally, double* d_k, uint32_t* d_error,
                                     void* stream);

/* ---- output files and input-file dispatch (no GPU for the first three) ----
   Text of a float as Rust's Display writes it (plot_solution's to_string(),
   src/plot_solution.rs:14-34): shortest round-trip digits, positional, no
   exponent; "1" for 1.0, "-0", "NaN", "inf", "-inf".  Writes a NUL-terminated
   string; returns its length, or -1 if cap is too small (64 always fits f32,
   400 always fits f64). */
int nraps_format_f32(float v, char* buf, uint64_t cap);
int nraps_format_f64(double v, char* buf, uint64_t cap);
/* plot_solution (src/plot_solution.rs:7-58): writes dir/vars.csv (assembly
   length, cells, generations), dir/interface.csv (G flux rows, G
   assembly-average rows, the fission-source row) and dir/k_eff.csv (k, k_fund)
   from r's SolutionResults arrays.  dir NULL or "" = the working directory.
   plot.py is not started. */
int nraps_write_solution(const char* dir, const nraps_result* r, uint32_t energygroups,
                         uint64_t cells, uint64_t generations, double assembly_length);
/* The dispatch of src/main.rs:332-364: process_input(input_path; NULL =
   "./TestCaseC.txt"), mesh_gen, then
     Solution = 1           -> Monte Carlo with k = 1.0 on ctx;
     otherwise, solver LinAlg -> nraps_diffusion_solve (no GPU; ctx may be
                               NULL), whose results have one k, no k_fund
                               and no fission source: those CSV rows are
                               written empty;
     other solvers          -> NRAPS_ERR_UNSUPPORTED (the reference returns
                               empty results for them);
   then the three CSV files into out_dir with the last cell's right edge as
   the assembly length.  stats_out (Monte Carlo only) may be NULL. */
int nraps_run_input(nraps_ctx* ctx, const char* input_path, const char* out_dir, nraps_stats* stats_out);

/* ---- deterministic diffusion solver (no GPU) -----------------------------
   nalgebra_method (src/discrete.rs:169-356): multigroup finite-difference
   diffusion with the reference's boundary rows, group sweep, convergence
   test (delta_flux >= 1e-5 and delta_k >= 1e-6 keep it going) and power
   normalisation, in FP64 with tridiagonal solves (agrees with the reference
   to its f32 rounding).  flux / assembly_average: caller-allocated G*cells
   f32 or NULL.  max_iterations 0 = 100000; NRAPS_ERR_CAPPED if reached. */
typedef struct nraps_diffusion_info {
    double   k;
    uint64_t iterations;
    int32_t  converged;
    int32_t  pad;
    double   delta_flux, delta_k;
} nraps_diffusion_info;
int nraps_diffusion_solve(const nraps_problem* problem, uint64_t max_iterations, float* flux,
                          float* assembly_average, nraps_diffusion_info* info);
/* An initial fission source from the diffusion solution: n_sites sites,
   cell c chosen with probability proportional to sum_g nu sigf phi_g dx_c,
   x stratified within the cell, group from the cell material's chi --
   deterministic (stratified and low-discrepancy, no random numbers), sorted
   by x.  out: caller-allocated n_sites.  info may be NULL. */
int nraps_diffusion_source(const nraps_problem* problem, uint64_t n_sites, nraps_site* out,
                           nraps_diffusion_info* info);

/* Text of a status code. */
const char* nraps_status_string(int status);

#ifdef __cplusplus
}
#endif
#endif /* NRAPS_GPU_H */
