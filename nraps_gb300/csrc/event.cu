/*
 * event.cu — event-based Woodcock transport (FP32 flights, FP64 tallies).
 *
 * Particle record in the HBM queues (structure of arrays, 24 bytes):
 *   x f32 | mu f32 | PCG32 state u64 | particle id u32 | g:4 inst:12 seq:16
 * Delta tracking: each flight samples d = -ln(u)/maj[g] with the per-group
 * majorant over the instance's materials; the flight is real with probability
 * sigtr(x)/maj[g], else virtual.  Real collisions score the collision
 * estimators (flux 1/sigtr into the tally cell, k score nu*sigf/sigtr in
 * 2^-32 fixed point, both precomputed per material and group), bank
 * floor(nu*sigf/sigtr/k + u) sites (BANK mode), then absorb with probability
 * siga/sigtr or scatter (transport-corrected CDF, isotropic mu).  Outer
 * boundaries: vacuum leaks, reflective mirrors the position.
 *
 * Warps work independently: each iteration every live lane flies once (the
 * flight is virtual or ends in a real collision); lanes whose particle died
 * take the next input particle (claimed 64 at a time per warp); particles
 * that completed K real collisions and new fission sites are staged per warp
 * in shared memory and flushed 32 at a time with one atomic each.
 * Single-instance launches stage the instance's tables in shared memory;
 * batched launches read each particle's instance tables through L1; ranged
 * launches give each block a range of one instance's histories (its tables
 * staged, or read from global memory when they do not fit).
 *
 * Fission-bank order (parent, seq): persistent launches flush sites into 128
 * slabs, then the per-history site counts are scanned and every site is
 * scattered to offsets[parent] + seq; ranged launches append a range's sites
 * to chunks of a shared pool and order each range on its own (ev_rb_scan,
 * ev_rb_scatter).  Every kernel of a generation is launched with
 * programmatic stream serialization and waits (griddepcontrol) before
 * touching what the kernel before it produced.
 */
#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "dev_util.cuh"
#include "event.cuh"
#include "nr_math.h"
#include "tables.hpp"

namespace {

constexpr uint32_t NSLAB = 128;
constexpr uint32_t MAX_PASSES = 16;
/* cells of a shared-memory site histogram in the single-instance scatter */
constexpr uint32_t HIST_SMEM_MAX_CELLS = 12288;
/* the scatter keeps the scan tiles' bases in shared memory beside the cell
   histogram: up to this many tiles (33.5M histories) */
constexpr uint64_t LOCAL_SCAN_MAX_TILES = 8192;
/*
 * Unsigned division by an invariant divisor d (1 <= d < 2^63) as a 64x64
 * multiply-high, a subtraction and two shifts (Granlund & Montgomery,
 * "Division by invariant integers using multiplication", PLDI 1994, fig. 4.1):
 * with l = ceil(log2 d) and m = floor(2^64 (2^l - d) / d) + 1,
 * q = (t + ((n - t) >> min(l,1))) >> max(l-1,0) where t = mulhi(m, n).
 */
struct NDiv {
    unsigned long long m;
    uint32_t sh1, sh2;
    __host__ static NDiv make(uint64_t d) {
        NDiv r;
        uint32_t l = 0;
        while (l < 63 && (1ULL << l) < d) ++l;
        r.m = (unsigned long long)((((unsigned __int128)((1ULL << l) - d)) << 64) / d) + 1ULL;
        r.sh1 = l < 1 ? l : 1u;
        r.sh2 = l > 1 ? l - 1 : 0u;
        return r;
    }
    __device__ __forceinline__ uint64_t div(uint64_t n) const {
        const uint64_t t = __umul64hi(m, n);
        return (t + ((n - t) >> sh1)) >> sh2;
    }
};

/* the largest per-instance table a ranged launch stages in shared memory */
constexpr size_t RANGED_SMEM_MAX = 40 * 1024;

constexpr uint32_t NLOG2N_TAB = 65536;
constexpr double LOG2E = 1.4426950408889634;
constexpr int SCATTER_ONE_THREADS = 512;
constexpr uint32_t SCATTER_ONE_SPLIT = 2;   /* blocks per slab */

struct EvInst {
    const float* xs;          /* [(m*G+g)*4]: sigtr, pabs, nsf_st, inv_st      */
    const double* inv_st64;   /* [m*G+g] flux score                            */
    const unsigned long long* kq; /* [m*G+g] k score in 2^-32 fixed point      */
    const float* ocdf;        /* [(m*G+g)*G + e] outcome CDF of a collision    */
    const float* chicdf;      /* [m*G + g]                                     */
    const float* maj;         /* [g] majorant, [G+g] inverse                   */
    const float4* rdat;       /* R+1: left edge, 1/dx, first cell, cells       */
    const uint8_t* rmat;      /* R                                             */
    const uint2* bins;        /* nbins: next boundary, first region | multi<<31 */
    const uint32_t* fuel;     /* nfuel                                         */
    const float* cleft;       /* nc                                            */
    const float* cdx;         /* nc                                            */
    const uint8_t* cmat;      /* nc                                            */
    const double* nsf64;      /* [m + M*g]                                     */
    const double* inv_dx64;   /* nc                                            */
    uint32_t M, G, R, nc, nbins, nfuel;
    float L, inv_binw, boundl, boundr;
    uint64_t hist_begin, N, seed;
    NDiv ndiv;                /* division by N                                 */
    GenState* st;
    double* tally;
    uint64_t tally_stride;    /* generation g scores into tally + (g & 1) * this */
    uint32_t tally_shift;     /* bin b of a half at [b << tally_shift]          */
    double *flux_acc, *fs_acc, *flux_sum, *flux_sq, *k64, *entropy;
    nraps_site* bank[2];
    uint64_t bank_cap;
    uint32_t* hist;
    uint32_t hist_shift;      /* site counter of cell c at hist[c << hist_shift] */
    uint64_t generations, skip, cell_begin;
    double conv_const;
};

struct EvArgs {
    const EvInst* inst;
    uint32_t n_inst;
    const uint64_t* inst_begin;   /* n_inst+1 particle-id prefix              */
    const uint64_t* cell_begin;   /* n_inst+1 global-cell prefix              */
    uint64_t n_total, n_cells_total;
    float* qx[2];
    float* qmu[2];
    unsigned long long* qrng[2];
    uint32_t* qid[2];
    uint32_t* qpk[2];
    unsigned long long* qcount;   /* MAX_PASSES+2: particles queued by pass p */
    unsigned long long* claim;    /* MAX_PASSES+2: input claimed by pass p    */
    unsigned long long* blocks_done; /* finalize: blocks that finished          */
    /* deferred end of generation (one instance): blocks from fold_from on
       of a one-pass transport launch fold the generation left pending
       (0xFFFFFFFF: none); scatter_close: the last block of the bank scatter
       closes the generation; their block counters */
    uint32_t fold_from;
    int scatter_close;
    unsigned long long* scatter_done;
    unsigned long long* fold_done;
    uint4* sites;                 /* NSLAB slabs of slab_cap site records      */
    unsigned long long* slab_count;
    uint64_t slab_cap;
    uint32_t* count;
    uint32_t* offsets;            /* n_total+1                                */
    /* deferred end of generation: offsets hold each history's offset from
       its scan tile's start, tile_sums the n_tiles tiles' totals (the scatter
       adds the tiles' bases, the close takes the bank size from them);
       nullptr: offsets are the whole exclusive scan */
    uint32_t* tile_sums;
    uint32_t n_tiles;
    GenState* stats;
    uint64_t max_events;
    nraps_history_record* rec;
    int bank;
    /* single-instance launch with at most HIST_SMEM_MAX_CELLS cells: the
       scatter counts sites per cell in shared memory */
    int hist_smem;
    /* n*log2(n) for n < NLOG2N_TAB (FP64, filled once on the host with the
       shared logarithm): the entropy is log2(B) - sum_c n_c log2(n_c) / B */
    const double* nlog2n;
    /* ranged launch of a batch (one-pass, every instance's tables fit shared
       memory): block b takes range b of range_len histories of one instance,
       stages that instance's tables and claims from a block-local counter.
       range_begin[i] = ranges before instance i (n_inst+1 entries); 0 = off */
    uint32_t range_len;
    const uint32_t* range_begin;
    /* ranged bank (BANK mode, ranged launch): a block appends its range's
       sites to chunks of RB_CHUNK records taken from a shared pool
       (block-local fill counter, per-range chunk list), so the bank order is
       later made per range from a block-local scan of the range's site
       counts, with no scan over every history and no scatter across the
       whole bank.  rb = 0: the site slabs of the other launches. */
    int rb;
    uint32_t rb_pool_chunks;
    unsigned long long* rb_next;     /* chunks handed out this generation     */
    uint32_t* rb_chunk;              /* ranges * RB_MAXC chunk ids              */
    uint32_t* rb_fill;               /* ranges: sites the range appended        */
    unsigned long long* rb_base;     /* ranges: first bank position in its instance */
    unsigned long long* rb_total;    /* n_inst: sites of the generation         */
    /* sorted transport: the collision queue (structure of arrays, the
       flight queue's record plus the region of the collision) and its fill
       per round */
    float* cx;
    float* cmu;
    unsigned long long* crng;
    uint32_t* cid;
    uint32_t* cpk;
    uint32_t* creg;
    unsigned long long* ccount;      /* MAX_PASSES+2                            */
};

/* ranged bank geometry */
constexpr uint32_t RB_CHUNK = 1024;          /* site records per chunk (16 KB)   */
constexpr uint32_t RB_MAXC = 256;            /* chunks per range: 8 sites per
                                                history of the longest range   */
constexpr uint32_t RB_MAX_RANGE = 32768;     /* longest range (its scan is in
                                                shared memory)                 */
constexpr uint32_t RB_HIST_SMEM = 8192;      /* cells counted in shared memory   */
constexpr uint32_t RB_THREADS = 256;
constexpr uint32_t RB_UNSET = 0xFFFFFFFFu;   /* chunk not handed out yet         */
constexpr uint32_t RB_FULL = 0xFFFFFFFEu;    /* the pool or the range is full    */
constexpr uint32_t RB_SPIN_MAX = 1u << 20;   /* bound on waiting for a chunk id  */

/* table view: shared memory (single instance) or the instance's globals */
struct TView {
    const float4* xs;             /* [m*G+g]: sigtr, pabs, nsf_st, inv_st     */
    const double* inv_st64;
    const unsigned long long* kq;
    const float* ocdf;
    const float* chi;
    const float* maj;
    const float4* rdat;
    const uint2* bins;
    const uint8_t* rmat;
    uint32_t G, R, nbins;
    float L, inv_binw, boundl, boundr;
};

__device__ __forceinline__ float u24(uint32_t u) { return __fmul_rn(__uint2float_rn(u >> 8), 0x1p-24f); }
__device__ __forceinline__ float u24pos(uint32_t u) { return __fmul_rn(__uint2float_rn((u >> 8) + 1u), 0x1p-24f); }

template <bool EXACT> __device__ __forceinline__ float neg_log(float u) {
    if (EXACT) return -nr_logf(u);
    return -__logf(u);
}

/* region r with left[r] <= x < left[r+1] (the last region for x == L), for
   0 <= x <= L: the bin gives the first region its points can lie in and the
   next boundary; a bin with several boundaries walks on (bins are narrower
   than half the narrowest region unless their count is capped) */
__device__ __forceinline__ uint32_t region_of(const TView& t, float x) {
    int b = (int)__fmul_rn(x, t.inv_binw);
    b = b < 0 ? 0 : (b >= (int)t.nbins ? (int)t.nbins - 1 : b);
    const uint2 e = t.bins[b];
    uint32_t r = (e.y & 0x7FFFFFFFu) + (x >= __uint_as_float(e.x) ? 1u : 0u);
    if (e.y & 0x80000000u)
        while (r + 1 < t.R && x >= t.rdat[r + 1].x) ++r;
    return r;
}

/* number of CDF entries below v, clamped to G-1: the chi group of energy()
   (partition_point on a non-decreasing CDF), without data-dependent branches */
__device__ __forceinline__ uint32_t count_below(const float* cdf, uint32_t G, float v) {
    uint32_t n = 0;
    for (uint32_t e = 0; e < G; ++e) n += (cdf[e] < v) ? 1u : 0u;
    return n < G - 1 ? n : G - 1;
}
/* number of the G entries of a collision's outcome CDF that are <= v:
   0 = absorbed, n >= 1 = scattered into group n - 1 */
__device__ __forceinline__ uint32_t count_outcome(const float* cdf, uint32_t G, float v) {
    uint32_t n = 0;
    for (uint32_t e = 0; e < G; ++e) n += (cdf[e] <= v) ? 1u : 0u;
    return n;
}

struct Part {
    float x, mu;
    nr_pcg32 rng;
    uint32_t id, local, g, inst, seq;
};

struct Acc {
    unsigned long long kq;
    uint32_t coll, virt, absorbed, leaked, capped;
};

/* Per-instance values a lane needs when it takes a particle or scores a
   collision.  A single-instance launch keeps one copy per block, filled once;
   a batched launch keeps one per lane, refilled only when the lane's instance
   changes (consecutive particles of a lane nearly always share one).  This
   keeps dependent global loads (descriptor -> GenState -> generation) and the
   generation-seed hash off the per-particle path. */
struct Hot {
    double* tally;
    unsigned long long gseed;       /* PCG seed of the instance's generation   */
    unsigned long long hist_begin;
    uint32_t nc;
    float inv_k;                    /* (float)(1/k) of the previous generation */
    uint32_t inst;
    uint32_t tshift;                /* tally bin b at tally[b << tshift]       */
};

__device__ __forceinline__ void load_hot(Hot& h, const EvInst& I, uint32_t inst, bool bank) {
    const GenState* st = I.st;
    const uint64_t gen = st->gen;
    h.tally = I.tally + (gen & 1) * I.tally_stride;
    h.tshift = I.tally_shift;
    h.nc = I.nc;
    h.hist_begin = I.hist_begin;
    h.gseed = nr_generation_seed(I.seed, gen);
    h.inv_k = bank ? st->inv_kf : 0.0f;
    h.inst = inst;
}

/* Batched launches: per lane, the generation seed and first history of the
   instance whose birth records the lane last prefetched. */
struct PfHot {
    unsigned long long gseed, hist_begin;
    uint32_t inst, pad;
};

/* Bank source of a single-instance launch: the ordered bank of the previous
   generation, its size B and the divisor N (histories); particle i starts at
   site floor(i*B/N). */
struct SrcBank {
    const nraps_site* bank;
    unsigned long long nbk;
    NDiv ndiv;
};

/* floor(i*B/N) for i < N <= 2^32 and B < 2^32: the product fits 64 bits and
   the division by N is a multiply-high with N's invariant reciprocal
   (integer pipes only; FP64 and 64-bit division are slow on this part) */
__device__ __forceinline__ uint64_t bank_site(uint64_t i, uint64_t nbk, const NDiv& nd) {
    return nd.div(i * nbk);
}

__device__ __forceinline__ TView global_view(const EvInst& I) {
    TView t;
    t.xs = reinterpret_cast<const float4*>(I.xs); t.inv_st64 = I.inv_st64; t.kq = I.kq; t.ocdf = I.ocdf;
    t.chi = I.chicdf; t.maj = I.maj; t.rdat = I.rdat; t.bins = I.bins; t.rmat = I.rmat;
    t.G = I.G; t.R = I.R; t.nbins = I.nbins; t.L = I.L; t.inv_binw = I.inv_binw;
    t.boundl = I.boundl; t.boundr = I.boundr;
    return t;
}

/* shared-memory footprint of one instance's tables: 8-byte and 16-byte
   arrays first, then floats, then bytes */
__host__ __device__ __forceinline__ size_t smem_bytes_for(uint32_t M, uint32_t G, uint32_t R, uint32_t nbins) {
    const size_t MG = (size_t)M * G;
    size_t b = MG * 16 + MG * 16 + ((size_t)R + 1) * 16 + (size_t)nbins * 8;
    b += (MG * G + MG + 2 * (size_t)G) * 4 + R;
    return (b + 15) / 16 * 16;
}

/* Copies one instance's tables into shared memory at tab (block-wide; the
   caller synchronises) and points t at them. */
__device__ __forceinline__ void stage_tables(const EvInst& I, unsigned char* tab, TView& t) {
    const uint32_t M = I.M, G = I.G, R = I.R, NB = I.nbins, MG = M * G;
    double* s_inv64 = reinterpret_cast<double*>(tab);
    unsigned long long* s_kq = reinterpret_cast<unsigned long long*>(s_inv64 + MG);
    float4* s_xs = reinterpret_cast<float4*>(s_kq + MG);
    float4* s_rdat = s_xs + MG;
    uint2* s_bins = reinterpret_cast<uint2*>(s_rdat + R + 1);
    float* s_ocdf = reinterpret_cast<float*>(s_bins + NB);
    float* s_chi = s_ocdf + MG * G;
    float* s_maj = s_chi + MG;
    uint8_t* s_rmat = reinterpret_cast<uint8_t*>(s_maj + 2 * G);
    const float4* g_xs = reinterpret_cast<const float4*>(I.xs);
    for (uint32_t i = threadIdx.x; i < MG; i += blockDim.x) {
        s_inv64[i] = I.inv_st64[i]; s_kq[i] = I.kq[i]; s_xs[i] = g_xs[i];
    }
    for (uint32_t i = threadIdx.x; i <= R; i += blockDim.x) s_rdat[i] = I.rdat[i];
    for (uint32_t i = threadIdx.x; i < NB; i += blockDim.x) s_bins[i] = I.bins[i];
    for (uint32_t i = threadIdx.x; i < MG * G; i += blockDim.x) s_ocdf[i] = I.ocdf[i];
    for (uint32_t i = threadIdx.x; i < MG; i += blockDim.x) s_chi[i] = I.chicdf[i];
    for (uint32_t i = threadIdx.x; i < 2 * G; i += blockDim.x) s_maj[i] = I.maj[i];
    for (uint32_t i = threadIdx.x; i < R; i += blockDim.x) s_rmat[i] = I.rmat[i];
    t.xs = s_xs; t.inv_st64 = s_inv64; t.kq = s_kq; t.ocdf = s_ocdf; t.chi = s_chi; t.maj = s_maj;
    t.rdat = s_rdat; t.bins = s_bins; t.rmat = s_rmat;
    t.G = G; t.R = R; t.nbins = NB; t.L = I.L; t.inv_binw = I.inv_binw;
    t.boundl = I.boundl; t.boundr = I.boundr;
}

constexpr int WARPS_MAX = 8;        /* batched (ONE = 0) blocks: at most 256 threads */
struct Stage;
__host__ __device__ __forceinline__ size_t stage_bytes(uint32_t block);
constexpr uint32_t CHUNK = 64;      /* particles a warp claims per atomic     */
constexpr uint32_t STAGE = 64;      /* records a warp stages before a flush   */

struct Stage {
    float x[STAGE], mu[STAGE];
    unsigned long long rng[STAGE];
    uint32_t id[STAGE], pk[STAGE];
    uint4 site[STAGE];
    /* prefetched input records of the warp's current chunk */
    uint4 pf_a[CHUNK];
    unsigned long long pf_rng[CHUNK];
};

static_assert(sizeof(Stage) % 16 == 0, "Stage keeps the tables after it 16-byte aligned");
__host__ __device__ __forceinline__ size_t stage_bytes(uint32_t block) { return (size_t)(block / 32) * sizeof(Stage); }

/* flush the first n staged survivors of a warp to the out queue (warp-wide) */
__device__ __forceinline__ void flush_particles(const EvArgs& a, Stage& sg, uint32_t n, int pass, int qout,
                                                uint32_t lane) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(&a.qcount[pass], (unsigned long long)n);
    base = __shfl_sync(0xffffffffu, base, 0);
    for (uint32_t i = lane; i < n; i += 32) {
        uint64_t o = base + i;
        a.qx[qout][o] = sg.x[i];
        a.qmu[qout][o] = sg.mu[i];
        a.qrng[qout][o] = sg.rng[i];
        a.qid[qout][o] = sg.id[i];
        a.qpk[qout][o] = sg.pk[i];
    }
}

/* flush the first n staged sites of a warp into its slab (warp-wide);
   returns false (all lanes) if the slab is full */
template <class S>
__device__ __forceinline__ bool flush_sites(const EvArgs& a, S& sg, uint32_t n, uint32_t slab,
                                            uint32_t lane) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(&a.slab_count[slab], (unsigned long long)n);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base + n > a.slab_cap) return false;
    for (uint32_t i = lane; i < n; i += 32) a.sites[(uint64_t)slab * a.slab_cap + base + i] = sg.site[i];
    return true;
}

/* flush the first n (<= 32) staged sites of a warp into its range's chunks
   (warp-wide; ranged launches, block b = range b).  The warp whose
   reservation holds the first slot of a chunk takes that chunk from the pool
   and publishes its id in shared memory; a warp that reaches a chunk first
   waits for the id (bounded; a wait that runs out sets NR_ERR_STALLED in
   *err).  Returns false (all lanes) when the range or the pool is full or
   a wait ran out. */
template <class S>
__device__ __forceinline__ bool flush_range_sites(const EvArgs& a, S& sg, uint32_t n, uint32_t lane,
                                                  uint32_t* s_fill, volatile uint32_t* s_chunk, unsigned int* err) {
    uint32_t p0 = 0;
    if (lane == 0) {
        p0 = atomicAdd(s_fill, n);
        /* n <= 32 < RB_CHUNK: at most one chunk starts in [p0, p0 + n) */
        const uint32_t c = (p0 + RB_CHUNK - 1) / RB_CHUNK;
        if (c * RB_CHUNK < p0 + n && c < RB_MAXC) {
            const unsigned long long id = atomicAdd(a.rb_next, 1ULL);
            const uint32_t v = id < a.rb_pool_chunks ? (uint32_t)id : RB_FULL;
            a.rb_chunk[(uint64_t)blockIdx.x * RB_MAXC + c] = v;
            s_chunk[c] = v;
        }
    }
    p0 = __shfl_sync(0xffffffffu, p0, 0);
    bool ok = true;
    if (lane < n) {
        const uint32_t pos = p0 + lane, c = pos / RB_CHUNK;
        uint32_t id = RB_FULL;
        if (c < RB_MAXC) id = s_chunk[c];
        for (uint32_t spin = 0; id == RB_UNSET && spin < RB_SPIN_MAX; ++spin) {
            __nanosleep(64);
            id = s_chunk[c];
        }
        if (id == RB_UNSET) atomicOr(err, NR_ERR_STALLED);
        ok = id < RB_FULL;
        if (ok) a.sites[(uint64_t)id * RB_CHUNK + (pos & (RB_CHUNK - 1))] = sg.site[lane];
    }
    return __all_sync(0xffffffffu, ok);
}

__device__ __forceinline__ void move_down(Stage& sg, uint32_t from, uint32_t n, uint32_t lane, bool sites) {
    /* entries [from, from+n) -> [0, n), n <= 32 */
    if (sites) {
        uint4 v = make_uint4(0, 0, 0, 0);
        if (lane < n) v = sg.site[from + lane];
        __syncwarp();
        if (lane < n) sg.site[lane] = v;
    } else {
        float x = 0.f, mu = 0.f; unsigned long long r = 0; uint32_t id = 0, pk = 0;
        if (lane < n) { x = sg.x[from + lane]; mu = sg.mu[from + lane]; r = sg.rng[from + lane]; id = sg.id[from + lane]; pk = sg.pk[from + lane]; }
        __syncwarp();
        if (lane < n) { sg.x[lane] = x; sg.mu[lane] = mu; sg.rng[lane] = r; sg.id[lane] = id; sg.pk[lane] = pk; }
    }
    __syncwarp();
}

/*
 * One queue pass.  Every warp: claim input particles, give them to idle
 * lanes, fly every live lane once per iteration, process real collisions,
 * stage fission sites and particles that completed K real collisions.
 */
template <bool SOURCE, int ONE, bool EXACT, bool BANK, bool REC, bool OP>
__device__ __forceinline__ void ev_pass_body(const EvArgs& a, int pass, uint32_t K, uint32_t tail) {
    /* ONE: 0 batched (instances mixed in a warp), 1 one instance, 2 ranged
       (block b runs range b of one instance, that instance's tables staged
       in shared memory), 3 ranged with the tables read from global memory
       (instances whose tables do not fit).  OP: one pass (every particle
       runs to its end; no survivor queue, no tail hand-off) -- K and tail
       are then ignored. */
    static_assert(!OP || SOURCE, "a one-pass launch starts from the source");
    constexpr bool RANGED = ONE >= 2;
    constexpr bool SMEM_TAB = ONE == 1 || ONE == 2;
    nrdev::pdl_trigger();
    /* batched: every read below may depend on the previous kernel; one
       instance: its tables are staged (and the range found) before the wait */
    if (!ONE) nrdev::pdl_wait();
    /* dynamic shared memory: one Stage per warp, then (ONE) the tables */
    extern __shared__ __align__(16) unsigned char smem[];
    Stage* s_stage = reinterpret_cast<Stage*>(smem);
    __shared__ Hot s_hot[ONE ? 1 : WARPS_MAX * 32];
    __shared__ PfHot s_pf[ONE ? 1 : WARPS_MAX * 32];
    __shared__ SrcBank s_src;
    TView t;
    if (!ONE) {
        s_hot[threadIdx.x].inst = 0xFFFFFFFFu;
        s_pf[threadIdx.x].inst = 0xFFFFFFFFu;
    }
    /* the instance this block runs (ONE: the only one, or, in a ranged batch
       launch, the instance of the block's range) and the range it claims */
    __shared__ unsigned long long s_claim;
    __shared__ uint32_t s_inst0;
    __shared__ unsigned long long s_rend;
    /* ranged bank: the range's fill and chunk ids */
    __shared__ uint32_t s_rfill;
    __shared__ uint32_t s_rchunk[RANGED ? RB_MAXC : 1];
    if (RANGED)
        for (uint32_t c = threadIdx.x; c < RB_MAXC; c += blockDim.x) s_rchunk[c] = RB_UNSET;
    if (ONE && threadIdx.x == 0) {
        uint32_t i0 = 0;
        unsigned long long rb = 0, re = a.n_total;
        if (RANGED) {
            uint32_t lo = 0, hi = a.n_inst;
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) >> 1;
                if (a.range_begin[mid] <= blockIdx.x) lo = mid; else hi = mid;
            }
            i0 = lo;
            const EvInst& I0 = a.inst[i0];
            rb = I0.hist_begin + (unsigned long long)(blockIdx.x - a.range_begin[i0]) * a.range_len;
            const unsigned long long iend = I0.hist_begin + I0.N;
            re = rb + a.range_len < iend ? rb + a.range_len : iend;
        }
        s_inst0 = i0;
        s_claim = rb;
        s_rend = re;
        s_rfill = 0;
    }
    if (ONE) __syncthreads();
    const uint32_t inst0 = ONE ? s_inst0 : 0u;
    if (ONE) {
        const EvInst& I = a.inst[inst0];
        unsigned char* tab = smem + (size_t)(blockDim.x >> 5) * sizeof(Stage);
        if (SMEM_TAB) stage_tables(I, tab, t);
        else t = global_view(I);
        nrdev::pdl_wait();
        if (threadIdx.x == 0) {
            load_hot(s_hot[0], I, inst0, BANK);
            if (SOURCE && BANK) {
                const GenState* st = I.st;
                s_src.bank = I.bank[st->gen & 1];
                s_src.nbk = st->n_bank;
                s_src.ndiv = I.ndiv;
            }
        }
        __syncthreads();
    }
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned lt = (1u << lane) - 1u;
    const unsigned FULL = 0xffffffffu;
    Stage& sg = s_stage[w];
    const int qin = (pass - 1) & 1, qout = pass & 1;
    const bool ranged = RANGED && SOURCE;
    /* ranged BANK launches append sites to their range's chunks (a
       compile-time choice: both flush paths in one kernel cost registers) */
    constexpr bool rbk = BANK && RANGED && SOURCE;
    const uint64_t n_in = ranged ? s_rend : (SOURCE ? a.n_total : a.qcount[pass - 1]);
    unsigned long long* claim = ranged ? &s_claim : &a.claim[pass];
    const uint32_t slab = (blockIdx.x * (blockDim.x >> 5) + w) % NSLAB;   /* every slab in use */
    uint64_t pool_next = 0, pool_end = 0;   /* warp-uniform claimed range     */
    uint64_t pf_base = 0;                   /* first index of the prefetch    */
    bool exhausted = false;
    uint32_t staged = 0, staged_sites = 0;  /* warp-uniform                   */
    bool slab_full = false;
    Acc acc = {0, 0, 0, 0, 0, 0};
    bool have = false;
    Part p;
    uint32_t done = 0;
    uint32_t events = 0;
    const uint32_t max_ev = a.max_events < 0xFFFFFFFFull ? (uint32_t)a.max_events : 0xFFFFFFFFu;
    const EvInst* Ip = &a.inst[inst0];
    TView tv = t;
    uint32_t tv_inst = 0xFFFFFFFFu;          /* batched: instance tv describes  */
    float inv_k = 0.0f;
    unsigned long long kq_part = 0;          /* batched: lane's k score for kq_inst */
    uint32_t kq_inst = 0;
    uint32_t draws = 0;
    for (;;) {
        /* ---- hand input particles to idle lanes ----------------------------
           A warp claims CHUNK input particles with one atomic and prefetches
           their records (birth site + instance, or queue entry) into shared
           memory in one coalesced step; idle lanes then take them in order. */
        unsigned need = __ballot_sync(FULL, !have);
        if (need && !exhausted) {
            if (pool_next == pool_end) {
                unsigned long long base = 0;
                if (lane == 0) base = atomicAdd(claim, (unsigned long long)CHUNK);
                base = __shfl_sync(FULL, base, 0);
                if (base >= n_in) {
                    exhausted = true;
                } else {
                    pool_next = base;
                    pool_end = base + CHUNK < n_in ? base + CHUNK : n_in;
                    __syncwarp();          /* every lane is done with the last chunk */
                    for (uint32_t k = lane; k < (uint32_t)(pool_end - pool_next); k += 32) {
                        uint64_t idx = pool_next + k;
                        if (SOURCE) {
                            /* the whole birth here, two records per lane, so the
                               per-lane hand-out below is a copy */
                            uint32_t inst = inst0;
                            if (!ONE) {
                                uint32_t lo = 0, hi = a.n_inst;
                                while (hi - lo > 1) {
                                    uint32_t mid = (lo + hi) >> 1;
                                    if (a.inst_begin[mid] <= idx) lo = mid; else hi = mid;
                                }
                                inst = lo;
                            }
                            const EvInst& I = a.inst[inst];
                            /* the record's instance, not this lane's particle's:
                               a separate cache from s_hot, which describes the
                               particle the lane is flying */
                            unsigned long long gseed, hb;
                            if (ONE) {
                                gseed = s_hot[0].gseed;
                                hb = s_hot[0].hist_begin;
                            } else {
                                PfHot& ph = s_pf[threadIdx.x];
                                if (ph.inst != inst) {
                                    ph.gseed = nr_generation_seed(I.seed, I.st->gen);
                                    ph.hist_begin = I.hist_begin;
                                    ph.inst = inst;
                                }
                                gseed = ph.gseed;
                                hb = ph.hist_begin;
                            }
                            const uint32_t local = (uint32_t)(idx - hb);
                            nr_pcg32 rng = nr_pcg32_seeded(gseed, local);
                            float bx = 0.0f, bmu;
                            uint32_t bg = 0, bcell = 0;
                            bool banked = false;
                            if (BANK && ONE) {
                                if (s_src.nbk > 0) {
                                    /* one 16-byte load of the site (x, cell, -, -) */
                                    const uint4 sv = reinterpret_cast<const uint4*>(s_src.bank)[bank_site(local, s_src.nbk, s_src.ndiv)];
                                    bx = __uint_as_float(sv.x); bcell = sv.y; banked = true;
                                }
                            } else if (BANK) {
                                const GenState* st = I.st;
                                const uint64_t nbk = st->n_bank;
                                if (nbk > 0) {
                                    const nraps_site* bank = I.bank[st->gen & 1];
                                    const uint4 sv = reinterpret_cast<const uint4*>(bank)[bank_site(local, nbk, I.ndiv)];
                                    bx = __uint_as_float(sv.x); bcell = sv.y; banked = true;
                                }
                            }
                            if (banked) {
                                /* a fission neutron's group is drawn at its birth, from chi
                                   of the material it was born in */
                                bmu = __fsub_rn(__fmul_rn(2.0f, u24(nr_pcg32_next(&rng))), 1.0f);
                                const uint32_t c = bcell < I.nc ? bcell : I.nc - 1;
                                bg = count_below(I.chicdf + (uint32_t)I.cmat[c] * I.G, I.G, u24(nr_pcg32_next(&rng)));
                            } else {
                                /* fresh uniform fuel source (spawn_neutron) */
                                const uint32_t cell = I.fuel[((uint64_t)nr_pcg32_next(&rng) * I.nfuel) >> 32];
                                const float sub = u24(nr_pcg32_next(&rng));
                                bx = __fadd_rn(I.cleft[cell], __fmul_rn(sub, I.cdx[cell]));
                                bmu = __fsub_rn(__fmul_rn(2.0f, u24(nr_pcg32_next(&rng))), 1.0f);
                                bg = count_below(I.chicdf + (uint32_t)I.cmat[cell] * I.G, I.G, u24(nr_pcg32_next(&rng)));
                            }
                            if (REC && inst == 0) a.rec[local].draws += banked ? 2 : 4;
                            sg.pf_a[k] = make_uint4(__float_as_uint(bx), __float_as_uint(bmu), (uint32_t)idx,
                                                    bg | (inst << 4));
                            sg.pf_rng[k] = rng.state;
                        } else {
                            sg.pf_a[k] = make_uint4(__float_as_uint(a.qx[qin][idx]), __float_as_uint(a.qmu[qin][idx]),
                                                    a.qid[qin][idx], a.qpk[qin][idx]);
                            sg.pf_rng[k] = a.qrng[qin][idx];
                        }
                    }
                    pf_base = pool_next;
                    __syncwarp();
                }
            }
            uint64_t avail = pool_end - pool_next;
            uint32_t rank = __popc(need & lt);
            bool got = !have && rank < avail;
            uint32_t slot = (uint32_t)(pool_next - pf_base) + rank;
            uint32_t n_need = __popc(need);
            pool_next += (uint64_t)n_need < avail ? n_need : avail;
            if (got) {
                /* birth record or queue entry: same layout */
                const uint4 r4 = sg.pf_a[slot];
                p.x = __uint_as_float(r4.x);
                p.mu = __uint_as_float(r4.y);
                p.id = r4.z;
                const uint32_t pk = r4.w;
                p.rng.state = sg.pf_rng[slot];
                p.g = pk & 15u;
                p.inst = ONE ? inst0 : (pk >> 4) & 0xFFFu;
                p.seq = pk >> 16;
                Hot& h = s_hot[ONE ? 0 : threadIdx.x];
                if (!ONE && h.inst != p.inst) load_hot(h, a.inst[p.inst], p.inst, BANK);
                p.local = (uint32_t)(p.id - h.hist_begin);
                p.rng.inc = ((uint64_t)p.local << 1) | 1ULL;
                Ip = &a.inst[ONE ? inst0 : p.inst];
                if (!ONE && p.inst != tv_inst) {
                    tv = global_view(*Ip);
                    tv_inst = p.inst;
                    /* consecutive particles of a lane nearly always share an
                       instance: flush the k score only when it changes */
                    if (p.inst != kq_inst) {
                        if (kq_part) atomicAdd(&a.inst[kq_inst].st->kq, kq_part);
                        kq_part = 0;
                        kq_inst = p.inst;
                    }
                }
                inv_k = s_hot[ONE ? 0 : threadIdx.x].inv_k;
                have = true;
                done = 0;
                events = 0;
            }
        }
        if (!__any_sync(FULL, have)) break;
        /* ---- tail hand-off: input used up and few lanes still live -------
           every live particle goes to the next pass's queue (at the start of
           its next flight, so its history is unchanged) and the warp leaves */
        if (!OP && tail && exhausted) {
            const unsigned live = __ballot_sync(FULL, have);
            if ((uint32_t)__popc(live) < tail) {
                if (have) {
                    uint32_t slot = staged + __popc(live & lt);
                    sg.x[slot] = p.x; sg.mu[slot] = p.mu; sg.rng[slot] = p.rng.state;
                    sg.id[slot] = p.id; sg.pk[slot] = p.g | (p.inst << 4) | (p.seq << 16);
                    have = false;
                }
                staged += __popc(live);
                __syncwarp();
                if (staged >= 32) {
                    flush_particles(a, sg, 32, pass, qout, lane);
                    __syncwarp();
                    move_down(sg, 32, staged - 32, lane, false);
                    staged -= 32;
                }
                break;
            }
        }

        /* ---- one flight per live lane --------------------------------------- */
        const uint32_t G = tv.G;
        nraps_history_record* rec = (REC && have && p.inst == 0) ? &a.rec[p.local] : nullptr;
        if (REC) draws = 0;
        auto next = [&]() -> uint32_t { if (REC) ++draws; return nr_pcg32_next(&p.rng); };
        int fate = -1;
        bool real = false;
        uint32_t m = 0, cell = 0, pending = 0;
        if (have) {
            /* one flight per step: a virtual collision ends the lane's step,
               so the next flight runs converged with the other lanes' flights
               (looping over virtual collisions here measured 30% more
               instructions: the extra iterations run divergent) */
            if (++events > max_ev) {
                fate = NRAPS_FATE_CAPPED;
            } else {
                float d = __fmul_rn(neg_log<EXACT>(u24pos(next())), tv.maj[G + p.g]);
                p.x = __fadd_rn(p.x, __fmul_rn(p.mu, d));
                int bounce = 0;
                while (!(p.x >= 0.0f && p.x <= tv.L)) {
                    if (p.x > tv.L) {
                        if (tv.boundr > 0.0f) { p.x = __fsub_rn(tv.L, __fsub_rn(p.x, tv.L)); p.mu = -p.mu; }
                        else { fate = NRAPS_FATE_LEAKED; break; }
                    } else {
                        if (tv.boundl > 0.0f) { p.x = -p.x; p.mu = -p.mu; }
                        else { fate = NRAPS_FATE_LEAKED; break; }
                    }
                    if (++bounce > 1000) { fate = NRAPS_FATE_CAPPED; break; }
                }
                if (fate < 0) {
                    uint32_t r = region_of(tv, p.x);
                    m = tv.rmat[r];
                    const uint32_t j = m * G + p.g;
                    const float4 X = tv.xs[j];
                    if (__fmul_rn(u24(next()), tv.maj[p.g]) < X.x) {
                        real = true;
                        acc.coll++;
                        const float4 rd = tv.rdat[r];
                        float rel = __fmul_rn(__fsub_rn(p.x, rd.x), rd.y);
                        const uint32_t nr = __float_as_uint(rd.w);
                        uint32_t k = rel > 0.0f ? (uint32_t)rel : 0u;
                        if (k >= nr) k = nr - 1;
                        cell = __float_as_uint(rd.z) + k;
                        {
                            const Hot& h = s_hot[ONE ? 0 : threadIdx.x];
                            nrdev::red_add_f64(&h.tally[((uint64_t)p.g * h.nc + cell) << h.tshift], tv.inv_st64[j]);
                        }
                        unsigned long long q = tv.kq[j];
                        acc.kq += q;
                        kq_part += q;
                        if (REC && rec) {
                            rec->collisions++;
                            rec->track += tv.inv_st64[j];
                            rec->nsf_track += (double)X.z;
                            rec->final_cell = cell;
                        }
                        if (BANK) {
                            float nu = __fadd_rn(__fmul_rn(X.z, inv_k), u24(next()));
                            int n = (int)floorf(nu);
                            pending = n > 64 ? 64u : (uint32_t)n;
                        }
                    } else {
                        acc.virt++;
                        if (REC && rec) rec->crossings++;
                    }
                }
            }
        }
        /* ---- fission sites: one per pending lane per round ------------------
           a site is a position and a cell; the child draws its group at birth */
        if (BANK) {
            while (__any_sync(FULL, pending > 0)) {
                unsigned sm = __ballot_sync(FULL, pending > 0);
                if (pending > 0) {
                    uint32_t slot = staged_sites + __popc(sm & lt);
                    sg.site[slot] = make_uint4(__float_as_uint(p.x), cell, p.id,
                                               (p.seq & 0xFFFFu) | (p.inst << 16));
                    if (p.seq >= 0xFFFFu) atomicOr(&Ip->st->error, NR_ERR_CAPACITY);
                    p.seq++;
                    pending--;
                }
                staged_sites += __popc(sm);
                __syncwarp();
                if (staged_sites >= 32) {
                    const bool fl = rbk ? flush_range_sites(a, sg, 32, lane, &s_rfill, s_rchunk, &Ip->st->error)
                                        : flush_sites(a, sg, 32, slab, lane);
                    if (!fl) slab_full = true;
                    move_down(sg, 32, staged_sites - 32, lane, true);
                    staged_sites -= 32;
                }
            }
        }
        /* ---- absorb or scatter ------------------------------------------------ */
        bool push = false;
        if (have) {
            if (real) {
                /* one uniform decides absorption and the scatter group */
                const uint32_t j = m * G + p.g;
                const uint32_t o = count_outcome(tv.ocdf + j * G, G, u24(next()));
                if (o == 0) {
                    fate = NRAPS_FATE_ABSORBED;
                } else {
                    p.g = o - 1;
                    p.mu = __fsub_rn(__fmul_rn(2.0f, u24(next())), 1.0f);
                }
                if (!OP) ++done;
            }
            if (REC && rec) rec->draws += draws;
            if (fate >= 0) {
                if (fate == NRAPS_FATE_ABSORBED) acc.absorbed++;
                else if (fate == NRAPS_FATE_LEAKED) acc.leaked++;
                else { acc.capped++; atomicOr(&Ip->st->error, NR_ERR_CAPPED); }
                if (BANK) a.count[p.id] = p.seq;
                if (REC && rec) {
                    rec->fate = fate; rec->final_group = p.g; rec->final_x = (double)p.x;
                    rec->n_sites = p.seq;
                }
                have = false;
            } else if (!OP && real && done >= K) {
                push = true;
                have = false;
            }
        }
        /* ---- stage survivors; flush 32 at a time ------------------------------ */
        const unsigned pm = OP ? 0u : __ballot_sync(FULL, push);
        if (!OP && pm) {
            if (push) {
                uint32_t slot = staged + __popc(pm & lt);
                sg.x[slot] = p.x; sg.mu[slot] = p.mu; sg.rng[slot] = p.rng.state;
                sg.id[slot] = p.id; sg.pk[slot] = p.g | (p.inst << 4) | (p.seq << 16);
            }
            staged += __popc(pm);
            __syncwarp();
            if (staged >= 32) {
                flush_particles(a, sg, 32, pass, qout, lane);
                __syncwarp();
                move_down(sg, 32, staged - 32, lane, false);
                staged -= 32;
            }
        }
    }
    __syncwarp();
    if (!ONE && kq_part) atomicAdd(&a.inst[kq_inst].st->kq, kq_part);
    if (staged) flush_particles(a, sg, staged, pass, qout, lane);
    if (BANK && staged_sites) {
        const bool fl = rbk ? flush_range_sites(a, sg, staged_sites, lane, &s_rfill, s_rchunk, &Ip->st->error)
                            : flush_sites(a, sg, staged_sites, slab, lane);
        if (!fl) slab_full = true;
    }
    if (slab_full && lane == 0) atomicOr(&a.inst[inst0].st->error, NR_ERR_CAPACITY);
    if (rbk) {
        __syncthreads();
        if (threadIdx.x == 0) a.rb_fill[blockIdx.x] = s_rfill;
    }
    /* ---- counters: one atomic per warp ---------------------------------------- */
    unsigned long long kq = nrdev::warp_sum_u64(ONE ? acc.kq : 0ull);
    unsigned long long coll = nrdev::warp_sum_u64(acc.coll), virt = nrdev::warp_sum_u64(acc.virt);
    unsigned long long ab = nrdev::warp_sum_u64(acc.absorbed), lk = nrdev::warp_sum_u64(acc.leaked);
    unsigned long long cp = nrdev::warp_sum_u64(acc.capped);
    if (lane == 0) {
        GenState* s = a.stats;
        if (ONE && kq) atomicAdd(&a.inst[inst0].st->kq, kq);
        if (coll) atomicAdd(&s->collisions, coll);
        if (virt) atomicAdd(&s->virtual_collisions, virt);
        if (ab) atomicAdd(&s->absorbed, ab);
        if (lk) atomicAdd(&s->leaked, lk);
        if (cp) atomicAdd(&s->capped, cp);
    }
}

/* The transport kernels.  Registers: 72 for the persistent one-instance
   transport (no spills; 7 blocks of 128 threads per SM.  Measured on
   single_large, 128-thread blocks, one launch per generation: 0.110 ms at a
   cap of 48, 0.099 at 56, 0.095 at 64, 0.094 at 72, 0.095 at 80, 0.101 at
   88 and 96), 64 for ranged launches with the tables in shared memory, 80
   where table pointers are global (batched, ranged over large tables). */
template <bool SOURCE, int ONE, bool EXACT, bool BANK, bool REC, bool OP>
__global__ void __launch_bounds__(256, ONE == 2 ? 4 : 3) ev_pass(EvArgs a, int pass, uint32_t K, uint32_t tail) {
    ev_pass_body<SOURCE, ONE, EXACT, BANK, REC, OP>(a, pass, K, tail);
}
__device__ __noinline__ void fold_pending_blocks(const EvArgs& a, uint32_t b, uint32_t nb);
template <bool SOURCE, bool EXACT, bool BANK, bool REC, bool OP>
__global__ void __maxnreg__(72) ev_pass_one(EvArgs a, int pass, uint32_t K, uint32_t tail) {
    if (SOURCE && OP && BANK && !REC && blockIdx.x >= a.fold_from) {
        /* a fold block: the blocks above the transport's are scheduled as
           transport blocks leave their SMs */
        nrdev::pdl_trigger();
        nrdev::pdl_wait();
        fold_pending_blocks(a, blockIdx.x - a.fold_from, gridDim.x - a.fold_from);
        return;
    }
    ev_pass_body<SOURCE, 1, EXACT, BANK, REC, OP>(a, pass, K, tail);
}
/* ranged launches in 512-thread blocks (an autotuner candidate for batches:
   fewer, larger blocks stage each range's tables once for twice the warps) */
template <int ONE, bool EXACT, bool BANK>
__global__ void __launch_bounds__(512, 2) ev_pass_wide(EvArgs a, int pass, uint32_t K, uint32_t tail) {
    static_assert(ONE >= 2, "512-thread blocks run ranged launches");
    ev_pass_body<true, ONE, EXACT, BANK, false, true>(a, pass, K, tail);
}
/* the kernel of one instantiation */
template <bool SOURCE, int ONE, bool EXACT, bool BANK, bool REC, bool OP>
constexpr auto pass_kernel() {
    if constexpr (ONE == 1) return &ev_pass_one<SOURCE, EXACT, BANK, REC, OP>;
    else return &ev_pass<SOURCE, ONE, EXACT, BANK, REC, OP>;
}

/*
 * Sorted transport (one instance).  Particles wait in structure-of-arrays
 * queues in HBM, and each event type runs in its own kernel over a queue
 * that holds only that event, so the lanes of a warp run the same code:
 *   ev_sort_flight   one flight per particle of round r's flight queue (in
 *                    round 0, the births): a leak ends the history, a virtual
 *                    collision puts the particle in round r+1's flight queue,
 *                    a real collision in round r's collision queue (with the
 *                    region it happened in);
 *   ev_sort_collide  one real collision per particle of the collision queue:
 *                    tally and k scores, fission sites, then absorption (the
 *                    history ends) or scatter (round r+1's flight queue).
 * Queue appends are warp-aggregated (one atomic per warp and queue).  After
 * R rounds the surviving particles run to their ends in one pass of the warp
 * transport (pass R, reading round R-1's output queue).  A particle draws the
 * same numbers in the same order as in ev_pass, so every history -- and with
 * it k, the tallies and the ordered bank -- is the same as with any other
 * launch shape.  Tables are read through L1 (no staging: a round's kernels
 * are short).
 */
struct SiteStage {
    uint4 site[STAGE];
};
constexpr size_t SORT_STAGE_BYTES = (256 / 32) * sizeof(SiteStage);   /* 256-thread blocks */

/* sites [from, from+n) of a warp's staging -> [0, n), n <= 32 */
__device__ __forceinline__ void move_sites_down(SiteStage& sg, uint32_t from, uint32_t n, uint32_t lane) {
    uint4 v = make_uint4(0, 0, 0, 0);
    if (lane < n) v = sg.site[from + lane];
    __syncwarp();
    if (lane < n) sg.site[lane] = v;
    __syncwarp();
}

/* warp-aggregated append of the lanes in `m` to a queue: the lane's slot */
__device__ __forceinline__ uint64_t queue_slot(unsigned long long* count, unsigned m, uint32_t lane) {
    unsigned long long base = 0;
    if (lane == 0 && m) base = atomicAdd(count, (unsigned long long)__popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    return base + __popc(m & ((1u << lane) - 1u));
}

__device__ __forceinline__ void flush_counters(const EvArgs& a, const Acc& acc, uint32_t lane) {
    const unsigned long long kq = nrdev::warp_sum_u64(acc.kq);
    const unsigned long long coll = nrdev::warp_sum_u64(acc.coll), virt = nrdev::warp_sum_u64(acc.virt);
    const unsigned long long ab = nrdev::warp_sum_u64(acc.absorbed), lk = nrdev::warp_sum_u64(acc.leaked);
    const unsigned long long cp = nrdev::warp_sum_u64(acc.capped);
    if (lane == 0) {
        GenState* s = a.stats;
        if (kq) atomicAdd(&a.inst[0].st->kq, kq);
        if (coll) atomicAdd(&s->collisions, coll);
        if (virt) atomicAdd(&s->virtual_collisions, virt);
        if (ab) atomicAdd(&s->absorbed, ab);
        if (lk) atomicAdd(&s->leaked, lk);
        if (cp) atomicAdd(&s->capped, cp);
    }
}

template <bool FIRST, bool EXACT, bool BANK>
__global__ void __launch_bounds__(256) ev_sort_flight(EvArgs a, int round) {
    nrdev::pdl_trigger();
    nrdev::pdl_wait();
    const EvInst& I = a.inst[0];
    const TView t = global_view(I);
    const GenState* st = I.st;
    const uint32_t lane = threadIdx.x & 31, G = t.G;
    const unsigned FULL = 0xffffffffu;
    const uint64_t n_in = FIRST ? a.n_total : a.qcount[round - 1];
    const int qin = (round - 1) & 1, qout = round & 1;
    unsigned long long gseed = 0, nbk = 0;
    const nraps_site* bank = nullptr;
    if (FIRST) {
        gseed = nr_generation_seed(I.seed, st->gen);
        if (BANK) { nbk = st->n_bank; bank = I.bank[st->gen & 1]; }
    }
    Acc acc = {0, 0, 0, 0, 0, 0};
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); i0 < n_in; i0 += stride) {
        const uint64_t i = i0 + lane;
        const bool valid = i < n_in;
        float x = 0.0f, mu = 0.0f;
        uint32_t id = 0, g = 0, seq = 0;
        nr_pcg32 rng;
        rng.state = 0; rng.inc = 1;
        if (valid) {
            if (FIRST) {
                /* the birth of history i, as the warp transport's prefetch makes it */
                id = (uint32_t)i;
                rng = nr_pcg32_seeded(gseed, i);
                if (BANK && nbk > 0) {
                    const uint4 sv = reinterpret_cast<const uint4*>(bank)[bank_site(i, nbk, I.ndiv)];
                    x = __uint_as_float(sv.x);
                    mu = __fsub_rn(__fmul_rn(2.0f, u24(nr_pcg32_next(&rng))), 1.0f);
                    const uint32_t c = sv.y < I.nc ? sv.y : I.nc - 1;
                    g = count_below(I.chicdf + (uint32_t)I.cmat[c] * G, G, u24(nr_pcg32_next(&rng)));
                } else {
                    const uint32_t cell = I.fuel[((uint64_t)nr_pcg32_next(&rng) * I.nfuel) >> 32];
                    const float sub = u24(nr_pcg32_next(&rng));
                    x = __fadd_rn(I.cleft[cell], __fmul_rn(sub, I.cdx[cell]));
                    mu = __fsub_rn(__fmul_rn(2.0f, u24(nr_pcg32_next(&rng))), 1.0f);
                    g = count_below(I.chicdf + (uint32_t)I.cmat[cell] * G, G, u24(nr_pcg32_next(&rng)));
                }
            } else {
                x = a.qx[qin][i]; mu = a.qmu[qin][i]; rng.state = a.qrng[qin][i]; id = a.qid[qin][i];
                const uint32_t pk = a.qpk[qin][i];
                g = pk & 15u; seq = pk >> 16;
                rng.inc = ((uint64_t)id << 1) | 1ULL;
            }
        }
        int fate = -1;
        bool real = false;
        uint32_t r = 0;
        if (valid) {
            const float d = __fmul_rn(neg_log<EXACT>(u24pos(nr_pcg32_next(&rng))), t.maj[G + g]);
            x = __fadd_rn(x, __fmul_rn(mu, d));
            int bounce = 0;
            while (!(x >= 0.0f && x <= t.L)) {
                if (x > t.L) {
                    if (t.boundr > 0.0f) { x = __fsub_rn(t.L, __fsub_rn(x, t.L)); mu = -mu; }
                    else { fate = NRAPS_FATE_LEAKED; break; }
                } else {
                    if (t.boundl > 0.0f) { x = -x; mu = -mu; }
                    else { fate = NRAPS_FATE_LEAKED; break; }
                }
                if (++bounce > 1000) { fate = NRAPS_FATE_CAPPED; break; }
            }
            if (fate < 0) {
                r = region_of(t, x);
                const uint32_t m = t.rmat[r];
                real = __fmul_rn(u24(nr_pcg32_next(&rng)), t.maj[g]) < t.xs[m * G + g].x;
                if (real) acc.coll++; else acc.virt++;
            } else {
                if (fate == NRAPS_FATE_LEAKED) acc.leaked++;
                else { acc.capped++; atomicOr(&I.st->error, NR_ERR_CAPPED); }
                if (BANK) a.count[id] = seq;
            }
        }
        const unsigned vm = __ballot_sync(FULL, valid && fate < 0 && !real);
        const unsigned rm = __ballot_sync(FULL, valid && real);
        const uint64_t vo = queue_slot(&a.qcount[round], vm, lane);
        const uint64_t ro = queue_slot(&a.ccount[round], rm, lane);
        const uint32_t pk = g | (seq << 16);
        if (valid && fate < 0) {
            if (real) {
                a.cx[ro] = x; a.cmu[ro] = mu; a.crng[ro] = rng.state; a.cid[ro] = id; a.cpk[ro] = pk;
                a.creg[ro] = r;
            } else {
                a.qx[qout][vo] = x; a.qmu[qout][vo] = mu; a.qrng[qout][vo] = rng.state;
                a.qid[qout][vo] = id; a.qpk[qout][vo] = pk;
            }
        }
    }
    flush_counters(a, acc, lane);
}

template <bool BANK>
__global__ void __launch_bounds__(256) ev_sort_collide(EvArgs a, int round) {
    extern __shared__ __align__(16) unsigned char smem[];
    nrdev::pdl_trigger();
    nrdev::pdl_wait();
    const EvInst& I = a.inst[0];
    const TView t = global_view(I);
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5, G = t.G;
    const unsigned lt = (1u << lane) - 1u;
    const unsigned FULL = 0xffffffffu;
    SiteStage& sg = reinterpret_cast<SiteStage*>(smem)[w];
    const uint32_t slab = (blockIdx.x * (blockDim.x >> 5) + w) % NSLAB;
    const uint64_t n_in = a.ccount[round];
    const int qout = round & 1;
    const float inv_k = BANK ? I.st->inv_kf : 0.0f;
    double* tally = I.tally + (I.st->gen & 1) * I.tally_stride;
    const uint32_t nc = I.nc;
    uint32_t staged_sites = 0;
    bool slab_full = false;
    Acc acc = {0, 0, 0, 0, 0, 0};
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); i0 < n_in; i0 += stride) {
        const uint64_t i = i0 + lane;
        const bool valid = i < n_in;
        float x = 0.0f, mu = 0.0f;
        uint32_t id = 0, g = 0, seq = 0, r = 0;
        nr_pcg32 rng;
        rng.state = 0; rng.inc = 1;
        if (valid) {
            x = a.cx[i]; mu = a.cmu[i]; rng.state = a.crng[i]; id = a.cid[i];
            const uint32_t pk = a.cpk[i];
            g = pk & 15u; seq = pk >> 16; r = a.creg[i];
            rng.inc = ((uint64_t)id << 1) | 1ULL;
        }
        uint32_t pending = 0, cell = 0, j = 0;
        if (valid) {
            const uint32_t m = t.rmat[r];
            j = m * G + g;
            const float4 X = t.xs[j];
            const float4 rd = t.rdat[r];
            const float rel = __fmul_rn(__fsub_rn(x, rd.x), rd.y);
            const uint32_t nr = __float_as_uint(rd.w);
            uint32_t k = rel > 0.0f ? (uint32_t)rel : 0u;
            if (k >= nr) k = nr - 1;
            cell = __float_as_uint(rd.z) + k;
            nrdev::red_add_f64(&tally[((uint64_t)g * nc + cell) << I.tally_shift], t.inv_st64[j]);
            acc.kq += t.kq[j];
            if (BANK) {
                const float nu = __fadd_rn(__fmul_rn(X.z, inv_k), u24(nr_pcg32_next(&rng)));
                const int n = (int)floorf(nu);
                pending = n > 64 ? 64u : (uint32_t)n;
            }
        }
        if (BANK) {
            while (__any_sync(FULL, pending > 0)) {
                const unsigned sm = __ballot_sync(FULL, pending > 0);
                if (pending > 0) {
                    const uint32_t slot = staged_sites + __popc(sm & lt);
                    sg.site[slot] = make_uint4(__float_as_uint(x), cell, id, seq & 0xFFFFu);
                    if (seq >= 0xFFFFu) atomicOr(&I.st->error, NR_ERR_CAPACITY);
                    seq++;
                    pending--;
                }
                staged_sites += __popc(sm);
                __syncwarp();
                if (staged_sites >= 32) {
                    if (!flush_sites(a, sg, 32, slab, lane)) slab_full = true;
                    move_sites_down(sg, 32, staged_sites - 32, lane);
                    staged_sites -= 32;
                }
            }
        }
        bool scattered = false;
        if (valid) {
            const uint32_t o = count_outcome(t.ocdf + j * G, G, u24(nr_pcg32_next(&rng)));
            if (o == 0) {
                acc.absorbed++;
                if (BANK) a.count[id] = seq;
            } else {
                g = o - 1;
                mu = __fsub_rn(__fmul_rn(2.0f, u24(nr_pcg32_next(&rng))), 1.0f);
                scattered = true;
            }
        }
        const unsigned smk = __ballot_sync(FULL, scattered);
        const uint64_t so = queue_slot(&a.qcount[round], smk, lane);
        if (scattered) {
            a.qx[qout][so] = x; a.qmu[qout][so] = mu; a.qrng[qout][so] = rng.state;
            a.qid[qout][so] = id; a.qpk[qout][so] = g | (seq << 16);
        }
    }
    __syncwarp();
    if (BANK && staged_sites && !flush_sites(a, sg, staged_sites, slab, lane)) slab_full = true;
    if (slab_full && lane == 0) atomicOr(&I.st->error, NR_ERR_CAPACITY);
    flush_counters(a, acc, lane);
}

__device__ __forceinline__ uint32_t find_inst(const uint64_t* begin, uint32_t n, uint64_t i) {
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (begin[mid] <= i) lo = mid; else hi = mid;
    }
    return lo;
}

/* ordered bank: site (parent, seq) -> offsets[parent] + seq - offsets[first
   history of its instance]; blocks walk the filled part of one slab each.
   KIND: SCAT_ONE one instance (its descriptor once per thread); SCAT_TAB
   every instance's destination (bank of the next generation, capacity,
   counters, scan offset of its first history) staged once per block in
   shared memory, so a site needs two independent loads (its parent's offset
   and a shared-memory row) instead of a chain through the instance
   descriptor and its GenState; SCAT_DIRECT the chain, for batches with more
   instances than the table holds.  Each thread keeps SCAT_U sites in flight,
   and lanes of a warp that add to the same site counter are merged into one
   addition (match on the counter's address): the sites of one warp flush
   are the children of neighbouring histories and often share a cell. */
enum { SCAT_ONE = 0, SCAT_TAB = 1, SCAT_DIRECT = 2 };
constexpr int SCAT_U = 4;
constexpr uint32_t SCAT_TAB_MAX = 1536;   /* 29 B per instance: 43.5 KB */
constexpr size_t SCAT_TAB_BYTES = 29;

template <int KIND>
__global__ void __launch_bounds__(256) ev_scatter(EvArgs a) {
    extern __shared__ unsigned long long s_tab[];
    nrdev::pdl_trigger();
    nrdev::pdl_wait();
    const uint32_t slab = blockIdx.x % NSLAB;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t per = gridDim.x / NSLAB;
    uint4** t_out = reinterpret_cast<uint4**>(s_tab);
    uint32_t** t_hist = reinterpret_cast<uint32_t**>(s_tab + a.n_inst);
    uint64_t* t_cap = reinterpret_cast<uint64_t*>(s_tab + 2 * (size_t)a.n_inst);
    uint32_t* t_base = reinterpret_cast<uint32_t*>(s_tab + 3 * (size_t)a.n_inst);
    uint8_t* t_shift = reinterpret_cast<uint8_t*>(t_base + a.n_inst);
    if (KIND == SCAT_TAB) {
        for (uint32_t i = threadIdx.x; i < a.n_inst; i += blockDim.x) {
            const EvInst& I = a.inst[i];
            t_out[i] = reinterpret_cast<uint4*>(I.bank[(I.st->gen + 1) & 1]);
            t_hist[i] = I.hist;
            t_cap[i] = I.bank_cap;
            t_base[i] = a.offsets[I.hist_begin];
            t_shift[i] = (uint8_t)I.hist_shift;
        }
        __syncthreads();
    }
    uint64_t filled = a.slab_count[slab];
    if (filled > a.slab_cap) filled = a.slab_cap;
    const uint4* src = a.sites + (uint64_t)slab * a.slab_cap;
    uint4* out0 = nullptr;
    uint64_t cap0 = 0;
    uint32_t* hist0 = nullptr;
    uint32_t shift0 = 0;
    if (KIND == SCAT_ONE) {
        const EvInst& I = a.inst[0];
        out0 = reinterpret_cast<uint4*>(I.bank[(I.st->gen + 1) & 1]);
        cap0 = I.bank_cap;
        hist0 = I.hist;
        shift0 = I.hist_shift;
    }
    /* warp-uniform chunks of SCAT_U x 32 sites: every lane runs every
       iteration, so the match below always has the full warp */
    const uint64_t wpb = blockDim.x >> 5;
    const uint64_t step = per * wpb * (SCAT_U * 32);
    for (uint64_t j0 = ((uint64_t)(blockIdx.x / NSLAB) * wpb + warp) * (SCAT_U * 32); j0 < filled; j0 += step) {
        uint4 v[SCAT_U];
        bool ok[SCAT_U];
#pragma unroll
        for (int u = 0; u < SCAT_U; ++u) {
            const uint64_t j = j0 + (uint64_t)u * 32 + lane;
            ok[u] = j < filled;
            v[u] = ok[u] ? src[j] : make_uint4(0, 0, 0, 0);
            /* a slab that overflowed keeps stale records: never follow them */
            ok[u] = ok[u] && v[u].z < a.n_total && (v[u].w >> 16) < a.n_inst;
        }
        uint32_t off[SCAT_U];
#pragma unroll
        for (int u = 0; u < SCAT_U; ++u) off[u] = ok[u] ? a.offsets[v[u].z] : 0u;
#pragma unroll
        for (int u = 0; u < SCAT_U; ++u) {
            const uint32_t inst = v[u].w >> 16;
            uint4* out;
            uint32_t* hist;
            uint32_t shift;
            uint64_t cap, pos = (uint64_t)off[u] + (v[u].w & 0xFFFFu);
            if (KIND == SCAT_ONE) {
                out = out0; hist = hist0; cap = cap0; shift = shift0;
            } else if (KIND == SCAT_TAB) {
                const uint32_t i = ok[u] ? inst : 0u;
                out = t_out[i]; hist = t_hist[i]; cap = t_cap[i]; shift = t_shift[i];
                pos -= t_base[i];
            } else {
                out = nullptr; hist = nullptr; cap = 0; shift = 0;
                if (ok[u]) {
                    const EvInst& I = a.inst[inst];
                    out = reinterpret_cast<uint4*>(I.bank[(I.st->gen + 1) & 1]);
                    hist = I.hist; cap = I.bank_cap; shift = I.hist_shift;
                    pos -= a.offsets[I.hist_begin];
                }
            }
            const bool w = ok[u] && pos < cap;
            const uint32_t cell = v[u].y & 0x07FFFFFFu;
            if (w) out[pos] = make_uint4(v[u].x, cell, v[u].y >> 27, 0u);   /* nraps_site, one 16-byte store */
            uint32_t* h = w ? hist + ((uint64_t)cell << shift) : nullptr;
            const unsigned peers = __match_any_sync(0xFFFFFFFFu, (unsigned long long)h);
            if (w && lane == (uint32_t)(__ffs(peers) - 1)) nrdev::red_add_u32(h, (uint32_t)__popc(peers));
        }
    }
}

/* Single instance, few cells: one block per slab.  Sites are counted per
   cell in shared memory and the block adds its non-zero bins to the
   instance's counters -- a hot fuel cell then costs shared-memory atomics
   instead of thousands of same-address L2 atomics.  Four sites per thread are
   loaded before any is used, so each thread keeps four load chains
   (site -> parent offset) in flight. */
__device__ __noinline__ void close_deferred(const EvArgs& a);
__global__ void __launch_bounds__(SCATTER_ONE_THREADS) ev_scatter_hist(EvArgs a) {
    extern __shared__ uint32_t s_h[];
    __shared__ bool s_last;
    nrdev::pdl_trigger();
    nrdev::pdl_wait();
    const EvInst& I = a.inst[0];
    if (a.scatter_close && blockIdx.x == gridDim.x - 1) {
        /* deferred end of generation: the block after the scatter blocks
           closes the generation while they scatter */
        close_deferred(a);
    } else {
        const uint32_t b = blockIdx.x;
        const uint32_t nc = I.nc;
        for (uint32_t c = threadIdx.x; c < nc; c += blockDim.x) s_h[c] = 0;
        const uint32_t slab = b / SCATTER_ONE_SPLIT, part = b % SCATTER_ONE_SPLIT;
        uint64_t filled = a.slab_count[slab];
        if (filled > a.slab_cap) filled = a.slab_cap;
        /* this block's contiguous share of the slab */
        const uint64_t per = (filled + SCATTER_ONE_SPLIT - 1) / SCATTER_ONE_SPLIT;
        const uint64_t lo = per * part;
        const uint64_t hi = lo + per < filled ? lo + per : filled;
        const uint4* src = a.sites + (uint64_t)slab * a.slab_cap;
        nraps_site* out = I.bank[(I.st->gen + 1) & 1];
        const uint64_t cap = I.bank_cap;
        /* offsets from the tiles' starts: the tiles' bases, an exclusive
           scan of their totals, into shared memory after the histogram */
        uint32_t* s_tb = s_h + nc;
        if (a.tile_sums) {
            __shared__ uint32_t s_sw[33];
            const uint32_t T = a.n_tiles, per_t = (T + blockDim.x - 1) / blockDim.x;
            const uint32_t t0 = threadIdx.x * per_t, t1 = t0 + per_t < T ? t0 + per_t : T;
            uint32_t run = 0;
            for (uint32_t t = t0; t < t1; ++t) run += a.tile_sums[t];
            uint32_t ex;
            nrdev::block_excl_scan(run, &ex, s_sw);
            for (uint32_t t = t0; t < t1; ++t) { const uint32_t v = a.tile_sums[t]; s_tb[t] = ex; ex += v; }
        }
        __syncthreads();
        constexpr int U = 4;
        for (uint64_t j0 = lo + threadIdx.x; j0 < hi; j0 += (uint64_t)U * blockDim.x) {
            uint4 v[U];
            uint32_t off[U];
            bool ok[U];
    #pragma unroll
            for (int u = 0; u < U; ++u) {
                uint64_t j = j0 + (uint64_t)u * blockDim.x;
                ok[u] = j < hi;
                v[u] = ok[u] ? src[j] : make_uint4(0, 0, 0, 0);
                /* a slab that overflowed keeps stale records: never follow them */
                ok[u] = ok[u] && v[u].z < a.n_total && (v[u].w >> 16) == 0u;
            }
    #pragma unroll
            for (int u = 0; u < U; ++u)
                off[u] = ok[u] ? a.offsets[v[u].z] + (a.tile_sums ? s_tb[v[u].z >> NR_SCAN_TILE_LOG2] : 0u) : 0u;
    #pragma unroll
            for (int u = 0; u < U; ++u) {
                uint64_t pos = (uint64_t)off[u] + (v[u].w & 0xFFFFu);
                if (ok[u] && pos < cap) {
                    uint32_t cell = v[u].y & 0x07FFFFFFu;
                    /* one 16-byte store (nraps_site is 4-byte aligned as a type;
                       the bank itself is 256-byte aligned) */
                    reinterpret_cast<uint4*>(out)[pos] = make_uint4(v[u].x, cell, v[u].y >> 27, 0u);
                    if (cell < nc) atomicAdd(&s_h[cell], 1u);
                }
            }
        }
        __syncthreads();
        /* non-zero bins into the instance's counters: ~NSLAB additions
           per fuel cell instead of one per site */
        for (uint32_t c = threadIdx.x; c < nc; c += blockDim.x)
            if (s_h[c]) nrdev::red_add_u32(&I.hist[(uint64_t)c << I.hist_shift], s_h[c]);
    }
    if (a.scatter_close) {
        /* the last block to finish (a counter, no waiting) advances the
           generation index and clears the slab fills.  No fence: every
           block read both before its increment (its loop bound and its
           bank depend on them); the bank, the histogram and the close's
           state are read by later launches. */
        __syncthreads();
        if (threadIdx.x == 0) s_last = atomicAdd(a.scatter_done, 1ULL) == gridDim.x - 1;
        __syncthreads();
        if (s_last) {
            for (uint32_t q = threadIdx.x; q < NSLAB; q += blockDim.x) a.slab_count[q] = 0;
            if (threadIdx.x == 0) {
                GenState* st = I.st;
                const uint64_t g = st->gen;
                if (g < I.generations) st->gen = g + 1;
                *a.scatter_done = 0;
            }
        }
    }
}

/* the instance of range r of a ranged launch (ranges of instance i are
   [range_begin[i], range_begin[i+1])) */
__device__ __forceinline__ uint32_t range_inst(const EvArgs& a, uint32_t r) {
    uint32_t lo = 0, hi = a.n_inst;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (a.range_begin[mid] <= r) lo = mid; else hi = mid;
    }
    return lo;
}

/*
 * Ranged bank, step 1 (one block per instance): the first bank position of
 * each of the instance's ranges -- the exclusive scan of the ranges' fills
 * -- and the generation's site total.
 */
__global__ void __launch_bounds__(RB_THREADS) ev_rb_scan(EvArgs a) {
    constexpr uint32_t NW = RB_THREADS / 32;
    __shared__ unsigned long long s_w[NW];
    __shared__ unsigned long long s_carry;
    nrdev::pdl_trigger();
    nrdev::pdl_wait();
    const uint32_t i = blockIdx.x, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t r0 = a.range_begin[i], r1 = a.range_begin[i + 1];
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    for (uint32_t b = r0; b < r1; b += RB_THREADS) {
        const uint32_t r = b + threadIdx.x;
        const unsigned long long f = r < r1 ? a.rb_fill[r] : 0ULL;
        unsigned long long x = f;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        if (lane == 31) s_w[w] = x;
        __syncthreads();
        if (w == 0) {
            unsigned long long y = lane < NW ? s_w[lane] : 0ULL;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned long long z = __shfl_up_sync(0xffffffffu, y, o);
                if (lane >= (uint32_t)o) y += z;
            }
            if (lane < NW) s_w[lane] = y;
        }
        __syncthreads();
        const unsigned long long carry = s_carry;
        if (r < r1) a.rb_base[r] = carry + (w ? s_w[w - 1] : 0ULL) + x - f;
        __syncthreads();
        if (threadIdx.x == 0) s_carry = carry + s_w[NW - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) a.rb_total[i] = s_carry;
}

/*
 * Ranged bank, step 2 (one block per range): the range's per-history site
 * counts are scanned in shared memory, and every site the range appended
 * goes to base + (sites of the range's earlier histories) + seq -- the
 * (parent, seq) order of the whole instance, written into a window of the
 * bank that only this block touches.  Sites are counted per cell in shared
 * memory (instances of at most RB_HIST_SMEM cells; the non-zero bins are
 * added to the instance's counters at the end) or, for larger instances,
 * straight into the counters, one addition per distinct counter of a warp.
 */
constexpr int RB_U = 4;
/* shared-memory words of a range's padded count/offset array */
__host__ __device__ constexpr uint32_t rb_loc_words(uint32_t range_len) { return range_len + range_len / 32 + 1; }
__global__ void __launch_bounds__(RB_THREADS) ev_rb_scatter(EvArgs a) {
    extern __shared__ uint32_t s_rb[];           /* loc[range_len], hist[...] */
    constexpr uint32_t NW = RB_THREADS / 32;
    __shared__ uint32_t s_ck[RB_MAXC];
    __shared__ uint32_t s_w[NW];
    nrdev::pdl_trigger();
    nrdev::pdl_wait();
    const uint32_t r = blockIdx.x, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t i0 = range_inst(a, r);
    const EvInst& I = a.inst[i0];
    const uint64_t rb = I.hist_begin + (uint64_t)(r - a.range_begin[i0]) * a.range_len;
    const uint64_t iend = I.hist_begin + I.N;
    const uint32_t nh = (uint32_t)((rb + a.range_len < iend ? rb + a.range_len : iend) - rb);
    const uint32_t nc = I.nc;
    const bool hsm = nc <= RB_HIST_SMEM;
    /* loc: the range's per-history counts, then their exclusive scan, at
       padded index j + j/32 (a thread's contiguous run below then reads
       across the banks) */
    uint32_t* loc = s_rb;
    uint32_t* hs = s_rb + rb_loc_words(a.range_len);
    if (hsm)
        for (uint32_t c = threadIdx.x; c < nc; c += RB_THREADS) hs[c] = 0;
    for (uint32_t c = threadIdx.x; c < RB_MAXC; c += RB_THREADS) s_ck[c] = a.rb_chunk[(uint64_t)r * RB_MAXC + c];
    /* the counts in one coalesced pass */
    for (uint32_t j = threadIdx.x; j < nh; j += RB_THREADS) loc[j + (j >> 5)] = a.count[rb + j];
    __syncthreads();
    /* exclusive scan of the range's site counts: each thread a contiguous
       run of ipt histories, then the block's run totals */
    const uint32_t ipt = (nh + RB_THREADS - 1) / RB_THREADS;
    const uint32_t j0 = threadIdx.x * ipt, j1 = j0 + ipt < nh ? j0 + ipt : nh;
    uint32_t sum = 0;
    for (uint32_t j = j0; j < j1; ++j) sum += loc[j + (j >> 5)];
    uint32_t x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) s_w[w] = x;
    __syncthreads();
    if (w == 0) {
        uint32_t y = lane < NW ? s_w[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t z = __shfl_up_sync(0xffffffffu, y, o);
            if (lane >= (uint32_t)o) y += z;
        }
        if (lane < NW) s_w[lane] = y;
    }
    __syncthreads();
    uint32_t run = (w ? s_w[w - 1] : 0u) + x - sum;
    for (uint32_t j = j0; j < j1; ++j) {
        const uint32_t jj = j + (j >> 5);
        const uint32_t c = loc[jj];
        loc[jj] = run;
        run += c;
    }
    __syncthreads();
    uint4* out = reinterpret_cast<uint4*>(I.bank[(I.st->gen + 1) & 1]);
    const uint64_t cap = I.bank_cap, base = a.rb_base[r];
    uint32_t* gh = I.hist;
    const uint32_t sh = I.hist_shift;
    uint32_t fill = a.rb_fill[r];
    if (fill > RB_MAXC * RB_CHUNK) fill = RB_MAXC * RB_CHUNK;
    /* block-uniform trip count: the match below always has the full warp */
    for (uint32_t q0 = 0; q0 < fill; q0 += RB_THREADS * RB_U) {
        uint4 v[RB_U];
        bool ok[RB_U];
#pragma unroll
        for (int u = 0; u < RB_U; ++u) {
            const uint32_t q = q0 + (uint32_t)u * RB_THREADS + threadIdx.x;
            const uint32_t id = q < fill ? s_ck[q / RB_CHUNK] : RB_FULL;
            ok[u] = id < RB_FULL;
            v[u] = ok[u] ? a.sites[(uint64_t)id * RB_CHUNK + q % RB_CHUNK] : make_uint4(0, 0, 0, 0);
        }
#pragma unroll
        for (int u = 0; u < RB_U; ++u) {
            /* slots of a range that ran out of room hold stale records */
            const uint64_t parent = v[u].z;
            const uint32_t cell = v[u].y & 0x07FFFFFFu;
            bool w8 = ok[u] && parent >= rb && parent < rb + nh && cell < nc;
            uint64_t pos = 0;
            if (w8) {
                const uint32_t jp = (uint32_t)(parent - rb);
                pos = base + loc[jp + (jp >> 5)] + (v[u].w & 0xFFFFu);
                w8 = pos < cap;
            }
            if (w8) out[pos] = make_uint4(v[u].x, cell, v[u].y >> 27, 0u);   /* nraps_site */
            if (hsm) {
                if (w8) atomicAdd(&hs[cell], 1u);
            } else {
                uint32_t* h = w8 ? gh + ((uint64_t)cell << sh) : nullptr;
                const unsigned peers = __match_any_sync(0xffffffffu, (unsigned long long)h);
                if (w8 && lane == (uint32_t)(__ffs(peers) - 1)) nrdev::red_add_u32(h, (uint32_t)__popc(peers));
            }
        }
    }
    if (hsm) {
        __syncthreads();
        for (uint32_t c = threadIdx.x; c < nc; c += RB_THREADS)
            if (hs[c]) nrdev::red_add_u32(&gh[(uint64_t)c << sh], hs[c]);
    }
}

/* block-wide: pass counters and slab fills back to zero for the next
   generation (called by the block that closes a generation) */
__device__ __forceinline__ void reset_pass_counters(const EvArgs& a) {
    for (uint32_t p = threadIdx.x; p < 2 * (MAX_PASSES + 2); p += blockDim.x) a.qcount[p] = 0;
    for (uint32_t p = threadIdx.x; p < MAX_PASSES + 2; p += blockDim.x) a.ccount[p] = 0;
    if (threadIdx.x == 0) *a.rb_next = 0;
    for (uint32_t q = threadIdx.x; q < NSLAB; q += blockDim.x) a.slab_count[q] = 0;
}

/* n log2(n) of a cell's site count (exact table below NLOG2N_TAB) */
__device__ __forceinline__ double nlog2n(const EvArgs& a, uint32_t n) {
    return n < NLOG2N_TAB ? a.nlog2n[n] : (double)n * nr_log((double)n) * LOG2E;
}

/* the per-instance factors of a generation's fold: 1/N, 1/k, 1/(active
   generations) and the power conversion times it (FP64 division is slow on
   this part: a single-instance finalize block computes them once) */
struct FoldK {
    double inv_n, inv_k, fund, cf;
    bool active;
};
__device__ __forceinline__ FoldK fold_factors(const EvInst& I, uint64_t gen, double k) {
    FoldK f;
    f.inv_n = 1.0 / (double)I.N;
    f.inv_k = 1.0 / k;
    f.fund = 1.0 / (double)(I.generations - I.skip);
    f.cf = I.conv_const * f.fund;
    f.active = gen >= I.skip;
    return f;
}

/*
 * One cell of one instance at the end of a generation: reads and clears its
 * G tally bins and, in active generations, accumulates flux, flux moments
 * and fission source (multiplications by precomputed reciprocals: FP64
 * division is slow on this part).  Every load that does not depend on
 * another is issued before the first store: the work is a few L2 round
 * trips, not arithmetic.
 */
__device__ __forceinline__ void fold_cell(const EvInst& I, double* __restrict__ tally, uint64_t c, const FoldK& f) {
    const uint32_t G = I.G, nc = I.nc;
    double* __restrict__ flux_acc = I.flux_acc;
    double* __restrict__ flux_sum = I.flux_sum;
    double* __restrict__ flux_sq = I.flux_sq;
    const double inv_dx = I.inv_dx64[c];
    const uint32_t m = I.cmat[c];
    const bool active = f.active;
    const double fund = f.fund;
    const double phi_scale = inv_dx * f.inv_n;              /* 1/(N dx)   */
    const double flux_scale = phi_scale * f.inv_k;          /* 1/(k N dx) */
    const double acc_scale = phi_scale * f.cf;
    double fs = 0.0;
    for (uint32_t g0 = 0; g0 < G; g0 += 4) {
        double tl[4], nsf[4], fa[4], f1[4], f2[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint32_t g = g0 + u;
            const uint64_t bin = (uint64_t)g * nc + c;
            const bool ok = g < G;
            tl[u] = ok ? tally[bin << I.tally_shift] : 0.0;
            nsf[u] = ok ? I.nsf64[m + (uint64_t)I.M * g] : 0.0;
            fa[u] = (ok && active) ? flux_acc[bin] : 0.0;
            f1[u] = (ok && active) ? flux_sum[bin] : 0.0;
            f2[u] = (ok && active) ? flux_sq[bin] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint32_t g = g0 + u;
            if (g >= G) break;
            const uint64_t bin = (uint64_t)g * nc + c;
            tally[bin << I.tally_shift] = 0.0;
            fs += nsf[u] * (tl[u] * flux_scale);
            if (active) {
                const double phi = tl[u] * phi_scale;
                flux_acc[bin] = fa[u] + tl[u] * acc_scale;
                flux_sum[bin] = f1[u] + phi;
                flux_sq[bin] = f2[u] + phi * phi;
            }
        }
    }
    if (active) I.fs_acc[c] += fs * fund;
}

/* per-instance end of generation: k, entropy, bank size, counters */
__device__ void finish_instance(const EvArgs& a, uint32_t i, const double* h_given = nullptr, bool defer = false,
                                bool set_gen = true, const unsigned long long* b_given = nullptr) {
    const EvInst& I = a.inst[i];
    GenState* st = I.st;
    /* every load first: this runs on one thread at the tail of the launch
       (h_acc is added to by other blocks: read past L1) */
    const uint64_t gen = st->gen;
    const unsigned long long kq = st->kq;
    const double k_old = st->k;
    const double h = h_given ? *h_given : *reinterpret_cast<volatile double*>(&st->h_acc);
    const double ksum = st->ksum, ksum2 = st->ksum2;
    const unsigned long long nactive = st->nactive, tot_sites = st->tot_sites, tot_hist = st->tot_histories;
    const unsigned int err0 = st->error;
    unsigned long long B = 0;
    if (a.bank)
        B = b_given ? *b_given : a.rb ? a.rb_total[i] : a.offsets[I.hist_begin + I.N] - a.offsets[I.hist_begin];
    unsigned long long c[5] = {0, 0, 0, 0, 0}, t[5] = {0, 0, 0, 0, 0};
    if (a.n_inst == 1) {
        c[0] = st->collisions; c[1] = st->virtual_collisions; c[2] = st->absorbed; c[3] = st->leaked;
        c[4] = st->capped;
        t[0] = st->tot_collisions; t[1] = st->tot_virtual; t[2] = st->tot_absorbed; t[3] = st->tot_leaked;
        t[4] = st->tot_capped;
    }
    if (gen >= I.generations) return;
    const double k_new = nr_unfix(kq) / (double)I.N;
    I.k64[gen] = k_new;
    if (gen >= I.skip) { st->ksum = ksum + k_new; st->ksum2 = ksum2 + k_new * k_new; st->nactive = nactive + 1; }
    unsigned int err = err0;
    if (a.bank) {
        if (defer) {
            /* flux, fission source and entropy of this generation are
               folded later (fold_pending_blocks): keep what they need */
            st->fold_gen = gen; st->fold_k = k_old; st->fold_B = B; st->fold_pending = 1;
        } else {
            /* h holds -sum_c n_c log2(n_c) */
            I.entropy[gen] = B ? nr_log((double)B) * LOG2E + h / (double)B : 0.0;
        }
        st->tot_sites = tot_sites + B;
        if (B > I.bank_cap) { B = I.bank_cap; err |= NR_ERR_CAPACITY; }
        st->n_bank = B;
        if (B == 0) err |= NR_ERR_EMPTY;
        if (err != err0) st->error = err;
    } else {
        I.entropy[gen] = 0.0;
    }
    if (a.n_inst == 1) {
        st->tot_collisions = t[0] + c[0]; st->tot_virtual = t[1] + c[1]; st->tot_absorbed = t[2] + c[2];
        st->tot_leaked = t[3] + c[3]; st->tot_capped = t[4] + c[4];
        st->collisions = st->virtual_collisions = st->absorbed = st->leaked = st->capped = 0;
    }
    st->tot_histories = tot_hist + I.N;
    st->kq = 0;
    st->h_acc = 0.0;
    st->n_sites = 0;
    st->k = k_new;
    st->inv_kf = (float)(1.0 / k_new);
    if (set_gen) st->gen = gen + 1;
}

constexpr int FIN_THREADS = 64;

/*
 * One thread per (instance, cell): reads and clears the cell's G tally bins,
 * accumulates flux and fission source of active generations (multiplications
 * by precomputed reciprocals: FP64 division is slow on this part), and the
 * cell's entropy term.  The last block to finish (threadfence + counter, no
 * waiting) then closes the generation of every instance and resets the pass
 * counters.
 */
__global__ void __launch_bounds__(FIN_THREADS) ev_finalize(EvArgs a) {
    __shared__ bool s_last;
    __shared__ FoldK s_f;
    nrdev::pdl_trigger();
    nrdev::pdl_wait();
    if (a.n_inst == 1) {
        if (threadIdx.x == 0) {
            const GenState* st = a.inst[0].st;
            s_f = fold_factors(a.inst[0], st->gen, st->k);
        }
        __syncthreads();
    }
    for (uint64_t gc0 = (uint64_t)blockIdx.x * blockDim.x; gc0 < a.n_cells_total;
         gc0 += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t gc = gc0 + threadIdx.x;
        double h = 0.0;
        uint32_t inst = 0xFFFFFFFFu;
        if (gc < a.n_cells_total) {
            inst = a.n_inst == 1 ? 0u : find_inst(a.cell_begin, a.n_inst, gc);
            const EvInst& I = a.inst[inst];
            const GenState* st = I.st;
            const uint64_t c = gc - I.cell_begin;
            const uint64_t gen = st->gen;
            const double k = st->k;
            uint32_t cnt = 0;
            uint64_t B = 0;
            if (a.bank) {
                cnt = I.hist[c << I.hist_shift];
                B = a.rb ? a.rb_total[inst] : a.offsets[I.hist_begin + I.N] - a.offsets[I.hist_begin];
            }
            if (gen < I.generations) {
                fold_cell(I, I.tally + (gen & 1) * I.tally_stride, c, a.n_inst == 1 ? s_f : fold_factors(I, gen, k));
                if (a.bank) {
                    I.hist[c << I.hist_shift] = 0;
                    if (cnt && B) h = -nlog2n(a, cnt);
                }
            }
        }
        if (a.bank) {
            /* warps within one instance reduce first; mixed warps add per lane */
            uint32_t i0 = __shfl_sync(0xffffffffu, inst, 0);
            bool uniform = __all_sync(0xffffffffu, inst == i0);
            if (uniform) {
                for (int o = 16; o > 0; o >>= 1) h += __shfl_down_sync(0xffffffffu, h, o);
                if ((threadIdx.x & 31) == 0 && i0 != 0xFFFFFFFFu && h != 0.0) atomicAdd(&a.inst[i0].st->h_acc, h);
            } else if (inst != 0xFFFFFFFFu && h != 0.0) {
                atomicAdd(&a.inst[inst].st->h_acc, h);
            }
        }
    }
    /* last block closes the generation */
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long d = atomicAdd(a.blocks_done, 1ULL);
        s_last = (d == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    for (uint32_t i = threadIdx.x; i < a.n_inst; i += blockDim.x) finish_instance(a, i);
    reset_pass_counters(a);
    __syncthreads();
    if (threadIdx.x == 0) {
        if (a.n_inst > 1) {
            GenState* s = a.stats;
            s->tot_collisions += s->collisions; s->tot_virtual += s->virtual_collisions;
            s->tot_absorbed += s->absorbed; s->tot_leaked += s->leaked; s->tot_capped += s->capped;
            s->collisions = s->virtual_collisions = s->absorbed = s->leaked = s->capped = 0;
        }
        *a.blocks_done = 0;
    }
}

/*
 * The deferred fold of instance 0: block b of nb folds cells
 * b * blockDim + t, stepping by nb * blockDim, of the generation a deferred
 * close left pending -- that generation's half of the tally into flux,
 * flux moments and fission source (with the k in effect during it), and
 * each cell's entropy term from the site histogram, which it clears.  The
 * last block to finish writes the generation's entropy and clears the
 * pending mark.  With nothing pending every block returns at once.
 */
__device__ __noinline__ void fold_pending_blocks(const EvArgs& a, uint32_t b, uint32_t nb) {
    __shared__ FoldK s_f;
    __shared__ unsigned long long s_gen, s_B;
    __shared__ bool s_go, s_last;
    const EvInst& I = a.inst[0];
    GenState* st = I.st;
    if (threadIdx.x == 0) {
        const unsigned long long pend = st->fold_pending;
        s_go = pend != 0;
        if (pend) {
            const uint64_t g = st->fold_gen;
            s_gen = g;
            s_B = st->fold_B;
            s_f = fold_factors(I, g, st->fold_k);
        }
    }
    __syncthreads();
    if (!s_go) return;
    const uint64_t g = s_gen, B = s_B;
    double* tally = I.tally + (g & 1) * I.tally_stride;
    double h = 0.0;
    for (uint64_t c = (uint64_t)b * blockDim.x + threadIdx.x; c < I.nc; c += (uint64_t)nb * blockDim.x) {
        fold_cell(I, tally, c, s_f);
        uint32_t* hp = &I.hist[c << I.hist_shift];
        const uint32_t cnt = *hp;
        *hp = 0;
        if (cnt && B) h -= nlog2n(a, cnt);
    }
    for (int o = 16; o > 0; o >>= 1) h += __shfl_down_sync(0xffffffffu, h, o);
    if ((threadIdx.x & 31) == 0 && h != 0.0) atomicAdd(&st->fold_h, h);
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(a.fold_done, 1ULL) == nb - 1;
    __syncthreads();
    if (!s_last || threadIdx.x != 0) return;
    __threadfence();
    /* added to by every block: read past L1 */
    const double hs = *reinterpret_cast<volatile double*>(&st->fold_h);
    I.entropy[g] = B ? nr_log((double)B) * LOG2E + hs / (double)B : 0.0;
    st->fold_h = 0.0;
    st->fold_pending = 0;
    *a.fold_done = 0;
}

/* A flush of the deferred fold (before anything reads flux, fission source
   or entropy, or a generation that closes the classic way) */
__global__ void __launch_bounds__(FIN_THREADS) ev_fold_flush(EvArgs a) {
    nrdev::pdl_trigger();
    nrdev::pdl_wait();
    fold_pending_blocks(a, blockIdx.x, gridDim.x);
}

/* The deferred close of instance 0, run by an extra block of the bank
   scatter beside the scatter blocks: k, bank size, counters (what the next
   transport needs; the fold comes later) -- all but the two values the
   scatter blocks themselves read, the generation index and the slab fills,
   which the scatter's last block advances and clears */
__device__ __noinline__ void close_deferred(const EvArgs& a) {
    __shared__ unsigned long long s_b[SCATTER_ONE_THREADS / 32];
    unsigned long long B = 0;
    if (a.tile_sums) {
        /* the bank size: the sum of the scan tiles' totals */
        unsigned long long t = 0;
        for (uint32_t i = threadIdx.x; i < a.n_tiles; i += blockDim.x) t += a.tile_sums[i];
        t = nrdev::warp_sum_u64(t);
        if ((threadIdx.x & 31) == 0) s_b[threadIdx.x >> 5] = t;
        __syncthreads();
        if (threadIdx.x == 0)
            for (uint32_t w = 0; w < (blockDim.x >> 5); ++w) B += s_b[w];
    }
    if (threadIdx.x == 0) finish_instance(a, 0, nullptr, true, false, a.tile_sums ? &B : nullptr);
    for (uint32_t p = threadIdx.x; p < 2 * (MAX_PASSES + 2); p += blockDim.x) a.qcount[p] = 0;
    for (uint32_t p = threadIdx.x; p < MAX_PASSES + 2; p += blockDim.x) a.ccount[p] = 0;
    if (threadIdx.x == 0) *a.rb_next = 0;
}

template <class T> struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaStream_t fs = nullptr;       /* pooled: freed in this stream's order */
    bool pooled = false;
    DeviceArena* arena = nullptr;    /* small buffers from here (never freed one by one) */
    bool in_arena = false;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    ~DBuf() { release(); }
    void release() {
        if (p && !in_arena) { if (pooled) cudaFreeAsync(p, fs); else cudaFree(p); }
        p = nullptr;
        pooled = false;
        in_arena = false;
    }
    cudaError_t alloc(size_t count, cudaMemPool_t pool = nullptr, cudaStream_t s = nullptr) {
        release();
        n = count;
        if (!count) return cudaSuccess;
        if (arena && !pool && count * sizeof(T) <= DeviceArena::ITEM_MAX) {
            in_arena = true;
            return arena->take(count * sizeof(T), reinterpret_cast<void**>(&p));
        }
        if (pool) {
            pooled = true;
            fs = s;
            return cudaMallocFromPoolAsync(reinterpret_cast<void**>(&p), count * sizeof(T), pool, s);
        }
        return cudaMalloc(&p, count * sizeof(T));
    }
};

}  // namespace

struct EventEngine::Impl {
    struct Inst {
        EvHostTables h;
        DBuf<unsigned char> blob;
        EvInst d{};
        EvBuffers b{};
    };
    std::vector<Inst*> inst;
    int mode = NRAPS_MODE_BANK;
    bool exact = false;
    uint64_t max_events = 1ULL << 24;
    DBuf<EvInst> d_inst;
    DBuf<uint64_t> d_inst_begin, d_cell_begin;
    DBuf<float> qx[2], qmu[2];
    DBuf<unsigned long long> qrng[2];
    DBuf<uint32_t> qid[2], qpk[2];
    DBuf<unsigned long long> qcount, slab_count;
    DBuf<uint4> sites;
    DBuf<uint32_t> count, offsets, block_sums;
    DBuf<GenState> bstats;
    DBuf<double> nlog2n;
    uint64_t n_total = 0, n_cells_total = 0, slab_cap = 0, cap_total = 0, cap_inst = 0;
    nraps_history_record* rec = nullptr;
    EvArgs args{};
    bool committed = false;
    bool fold_maybe_pending = false;   /* a deferred end of generation was enqueued */
    int grid_blocks = 0;
    /* sorted transport: the collision queue and the grid of its kernels */
    DBuf<float> cx, cmu;
    DBuf<unsigned long long> crng;
    DBuf<uint32_t> cid, cpk, creg;
    int sort_grid = 0;          /* resident blocks of the sorted kernels (0: not in use) */
    /* ranged launches stage the tables in shared memory when every
       instance's fit, else read them from global memory */
    bool ranged_fit = false;
    uint32_t range_built = 0;   /* range length d_range_begin was built for */
    uint32_t ranged_blocks = 0;
    size_t ranged_smem = 0;
    DBuf<uint32_t> d_range_begin;
    /* ranged bank buffers (the site pool shares the slab buffer) */
    bool rb_ok = false;             /* ranged launches use the ranged bank      */
    uint32_t rb_pool_chunks = 0;
    uint32_t rb_hist_cells = 0;     /* largest instance counted in shared memory */
    uint64_t bank_sum = 0;
    DBuf<uint32_t> rb_chunk, rb_fill;
    DBuf<unsigned long long> rb_base, rb_total;
    size_t smem_bytes = 0;
    bool one = true;
    /* programmatic dependent launch between the generation's kernels (each
       kernel's launch and prologue overlap the previous kernel's tail);
       NRAPS_NO_PDL=1 in the environment turns it off */
    bool pdl = !(std::getenv("NRAPS_NO_PDL") && std::getenv("NRAPS_NO_PDL")[0] == '1');
    /* per-instance tables from a stream-ordered pool (set_pool), or cudaMalloc */
    cudaMemPool_t pool = nullptr;
    cudaStream_t pool_stream = nullptr;
    DeviceArena* arena = nullptr;       /* small buffers at 64 KB strides (sessions) */
    ~Impl() { for (Inst* i : inst) delete i; }
};

EventEngine::EventEngine() : impl_(new Impl()) {}
EventEngine::~EventEngine() { delete impl_; }

int EventEngine::configure(const nraps_opts& o, std::string& err) {
    if (o.mode != NRAPS_MODE_PHYSICS && o.mode != NRAPS_MODE_BANK) { err = "WOODCOCK runs PHYSICS or BANK mode"; return NRAPS_ERR_INVALID; }
    impl_->mode = o.mode;
    impl_->exact = o.exact_log != 0;
    impl_->max_events = o.max_events ? o.max_events : (1ULL << 24);
    if (o.block_size) params.block = o.block_size;
    if (o.events_per_pass) params.K = o.events_per_pass;
    if (o.passes) params.passes = o.passes;
    params.tail = o.tail_lanes;
    params.sort = o.sort_rounds;
    params.range = o.range_len;
    if (params.range && (params.range < 64 || params.range > RB_MAX_RANGE)) { err = "range_len must be in [64, 32768]"; return NRAPS_ERR_INVALID; }
    if (params.range) { params.K = NRAPS_ONE_PASS; params.passes = 0; params.tail = 0; params.sort = 0; }
    if (params.sort > MAX_PASSES) { err = "sort_rounds must be at most 16"; return NRAPS_ERR_INVALID; }
    if (params.sort) { params.K = NRAPS_ONE_PASS; params.passes = 0; params.tail = 0; }
    if (params.K == NRAPS_ONE_PASS && o.passes == 0) params.passes = 0;  /* every particle to its end in one pass */
    if (params.tail > 32) { err = "tail_lanes must be at most 32"; return NRAPS_ERR_INVALID; }
    if (params.tail && params.passes == 0) { err = "tail_lanes needs a following pass (passes >= 1)"; return NRAPS_ERR_INVALID; }
    if (params.block != 128 && params.block != 256 && !(params.block == 512 && params.range)) {
        err = "block_size must be 128 or 256 for WOODCOCK (512 with range_len)";
        return NRAPS_ERR_INVALID;
    }
    if ((params.passes < 1 && params.K != NRAPS_ONE_PASS) || params.passes > MAX_PASSES) { err = "passes must be in [1, 16]"; return NRAPS_ERR_INVALID; }
    if (params.K < 1) { err = "events_per_pass must be >= 1"; return NRAPS_ERR_INVALID; }
    impl_->committed = false;
    return NRAPS_OK;
}

uint64_t EventEngine::table_bytes(const nraps_problem& p) {
    uint64_t M = p.variables.mattypes, G = p.variables.energygroups, nc = p.mesh.n_cells;
    /* xs, outcome and chi CDFs, majorants, flux and k scores, fuel list, per
       cell (left, width, material, nu*sigf-free FP64 width and inverse), per
       region at most one per cell (16 B + material), bins (8 B each, at most
       16384), 256-byte alignment of 17 arrays */
    return (M * G * (4 + G + 1) + 2 * G) * 4 + M * G * 16 + p.n_fuel * 4 +
           nc * (4 + 4 + 1 + 8 + 8) + (nc + 1) * (16 + 1) + 16384 * 8 + 17 * 256;
}

int EventEngine::add_instance(const nraps_problem& p, const EvBuffers& b, std::string& err) {
    if (impl_->inst.size() >= 4095) { err = "at most 4095 instances per batch"; return -1; }
    Impl::Inst* in = new Impl::Inst();
    in->blob.arena = impl_->arena;
    if (build_event_tables(p, in->h, err)) { delete in; return -1; }
    const EvHostTables& h = in->h;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = (off + bytes + 255) & ~(size_t)255; return o; };
    size_t o_xs = take(h.xs.size() * 4), o_inv64 = take(h.inv_st64.size() * 8), o_kq = take(h.kq.size() * 8);
    size_t o_ocdf = take(h.ocdf.size() * 4), o_chi = take(h.chicdf.size() * 4);
    size_t o_maj = take(h.maj.size() * 4), o_rdat = take(h.rdat.size() * 4);
    size_t o_rmat = take(h.rmat.size()), o_bins = take(h.bins.size() * 4);
    size_t o_fuel = take(h.fuel.size() * 4), o_cleft = take(h.cleft.size() * 4);
    size_t o_cdx = take(h.cdx.size() * 4), o_cmat = take(h.cmat.size()), o_nsf = take(h.nsf64.size() * 8);
    size_t o_idx = take(h.inv_dx64.size() * 8);
    std::vector<unsigned char> host(off, 0);
    auto put = [&](size_t o, const void* src, size_t bytes) { if (bytes) std::memcpy(host.data() + o, src, bytes); };
    put(o_xs, h.xs.data(), h.xs.size() * 4); put(o_inv64, h.inv_st64.data(), h.inv_st64.size() * 8);
    put(o_kq, h.kq.data(), h.kq.size() * 8);
    put(o_ocdf, h.ocdf.data(), h.ocdf.size() * 4);
    put(o_chi, h.chicdf.data(), h.chicdf.size() * 4); put(o_maj, h.maj.data(), h.maj.size() * 4);
    put(o_rdat, h.rdat.data(), h.rdat.size() * 4);
    put(o_rmat, h.rmat.data(), h.rmat.size()); put(o_bins, h.bins.data(), h.bins.size() * 4);
    put(o_fuel, h.fuel.data(), h.fuel.size() * 4); put(o_cleft, h.cleft.data(), h.cleft.size() * 4);
    put(o_cdx, h.cdx.data(), h.cdx.size() * 4); put(o_cmat, h.cmat.data(), h.cmat.size());
    put(o_nsf, h.nsf64.data(), h.nsf64.size() * 8); put(o_idx, h.inv_dx64.data(), h.inv_dx64.size() * 8);
    cudaError_t e;
    if (impl_->pool) {
        /* stream-ordered: no device-wide synchronisation per instance; the
           pageable source is staged before the copy call returns */
        e = in->blob.alloc(off, impl_->pool, impl_->pool_stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(in->blob.p, host.data(), off, cudaMemcpyHostToDevice, impl_->pool_stream);
    } else {
        e = in->blob.alloc(off);
        if (e == cudaSuccess) e = cudaMemcpy(in->blob.p, host.data(), off, cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) { err = std::string("event tables: ") + cudaGetErrorString(e); delete in; return -1; }
    unsigned char* B = in->blob.p;
    EvInst& d = in->d;
    d.xs = (const float*)(B + o_xs); d.inv_st64 = (const double*)(B + o_inv64);
    d.kq = (const unsigned long long*)(B + o_kq);
    d.ocdf = (const float*)(B + o_ocdf); d.chicdf = (const float*)(B + o_chi);
    d.maj = (const float*)(B + o_maj); d.rdat = (const float4*)(B + o_rdat);
    d.rmat = B + o_rmat; d.bins = (const uint2*)(B + o_bins); d.fuel = (const uint32_t*)(B + o_fuel);
    d.cleft = (const float*)(B + o_cleft); d.cdx = (const float*)(B + o_cdx); d.cmat = B + o_cmat;
    d.nsf64 = (const double*)(B + o_nsf); d.inv_dx64 = (const double*)(B + o_idx);
    d.M = h.M; d.G = h.G; d.R = h.R; d.nc = h.nc; d.nbins = h.nbins; d.nfuel = h.nfuel;
    d.L = h.L; d.inv_binw = h.inv_binw; d.boundl = h.boundl; d.boundr = h.boundr;
    d.N = p.variables.histories; d.seed = b.seed; d.ndiv = NDiv::make(d.N);
    d.st = b.st; d.tally = b.tally; d.tally_stride = b.tally_stride; d.tally_shift = b.tally_shift;
    d.flux_acc = b.flux_acc; d.fs_acc = b.fs_acc; d.flux_sum = b.flux_sum; d.flux_sq = b.flux_sq;
    d.k64 = b.k64; d.entropy = b.entropy;
    d.bank[0] = b.bank[0]; d.bank[1] = b.bank[1]; d.bank_cap = b.bank_cap; d.hist = b.hist;
    d.hist_shift = ev_hist_shift(h.nc);
    d.generations = b.generations; d.skip = b.skip; d.conv_const = h.conv_const;
    in->b = b;
    impl_->inst.push_back(in);
    impl_->committed = false;
    return (int)impl_->inst.size() - 1;
}

void EventEngine::remove_instance(uint32_t idx) {
    if (idx >= impl_->inst.size()) return;
    delete impl_->inst[idx];
    impl_->inst.erase(impl_->inst.begin() + idx);
    impl_->committed = false;
}

void EventEngine::clear_instances() {
    for (auto* i : impl_->inst) delete i;
    impl_->inst.clear();
    impl_->committed = false;
}

uint32_t EventEngine::n_instances() const { return (uint32_t)impl_->inst.size(); }
void EventEngine::set_arena(DeviceArena* a) {
    Impl& m = *impl_;
    m.arena = a;
    for (DBuf<float>* b : {&m.qx[0], &m.qx[1], &m.qmu[0], &m.qmu[1], &m.cx, &m.cmu}) b->arena = a;
    for (DBuf<unsigned long long>* b : {&m.qrng[0], &m.qrng[1], &m.qcount, &m.slab_count, &m.crng, &m.rb_base,
                                        &m.rb_total})
        b->arena = a;
    for (DBuf<uint32_t>* b : {&m.qid[0], &m.qid[1], &m.qpk[0], &m.qpk[1], &m.count, &m.offsets, &m.block_sums,
                              &m.d_range_begin, &m.rb_chunk, &m.rb_fill, &m.cid, &m.cpk, &m.creg})
        b->arena = a;
    m.d_inst.arena = a; m.d_inst_begin.arena = a; m.d_cell_begin.arena = a;
    m.sites.arena = a; m.bstats.arena = a; m.nlog2n.arena = a;
}
void EventEngine::set_pool(cudaMemPool_t pool, cudaStream_t s) { impl_->pool = pool; impl_->pool_stream = s; }
void EventEngine::set_records(nraps_history_record* rec) { impl_->rec = rec; impl_->committed = false; }
const uint32_t* EventEngine::offsets() const { return impl_->offsets.p; }
uint64_t EventEngine::n_total() const { return impl_->n_total; }
GenState* EventEngine::batch_stats() const { return impl_->bstats.p; }

uint64_t EventEngine::shared_bytes() const {
    const Impl* m = impl_;
    return m->n_total * (24 * 2 + 8) + m->sites.n * 16 + m->rb_chunk.n * 4 + m->rb_fill.n * 4 +
           (m->rb_base.n + m->rb_total.n) * 8;
}

namespace {
template <bool SOURCE, int ONE, bool EXACT, bool BANK, bool REC, bool OP>
void set_smem_attr(size_t smem) {
    /* the default limit of dynamic shared memory is 48 KB less the kernel's
       static shared memory: raise it for any dynamic size asked for */
    static size_t granted = 0;
    if (smem > granted) {
        cudaFuncSetAttribute(pass_kernel<SOURCE, ONE, EXACT, BANK, REC, OP>(),
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        granted = smem;
    }
}

/* fold_blocks > 0 (one pass, one instance): that many blocks after the
   transport's fold the generation a deferred close left pending */
template <bool ONE, bool EXACT, bool BANK, bool REC>
int launch_passes(const EvArgs& a, const EvParams& prm, int grid, size_t smem, uint64_t n_total,
                  cudaStream_t s, bool pdl, uint32_t fold_blocks = 0) {
    int launched = 0;
    uint32_t block = prm.block;
    smem += stage_bytes(block);
    unsigned g0 = (unsigned)std::min<uint64_t>((n_total + block - 1) / block, (uint64_t)grid);
    if (g0 == 0) g0 = 1;
    uint32_t P = prm.passes;
    cudaError_t e;
    if (P == 0) {
        /* one pass: every particle runs to its end */
        set_smem_attr<true, ONE, EXACT, BANK, REC, true>(smem);
        EvArgs af = a;
        if (ONE && BANK && !REC && fold_blocks) af.fold_from = g0;
        else fold_blocks = 0;
        e = launch_k(pdl, pass_kernel<true, ONE, EXACT, BANK, REC, true>(), dim3(g0 + fold_blocks), dim3(block), smem,
                     s, af, 0, 0xFFFFFFFFu, 0u);
    } else {
        set_smem_attr<true, ONE, EXACT, BANK, REC, false>(smem);
        set_smem_attr<false, ONE, EXACT, BANK, REC, false>(smem);
        e = launch_k(pdl, pass_kernel<true, ONE, EXACT, BANK, REC, false>(), dim3(g0), dim3(block), smem, s, a, 0,
                     prm.K, prm.tail);
    }
    if (e != cudaSuccess) return -1;
    ++launched;
    for (uint32_t p = 1; p <= P; ++p) {
        const bool last = p == P;
        if (launch_k(pdl, pass_kernel<false, ONE, EXACT, BANK, REC, false>(), dim3((unsigned)grid), dim3(block), smem, s, a,
                     (int)p, last ? 0xFFFFFFFFu : prm.K, last ? 0u : prm.tail) != cudaSuccess)
            return -1;
        ++launched;
    }
    return launched;
}
}  // namespace

namespace {
/* Every kernel a generation of this engine can launch, loaded up front: with
   lazy module loading a kernel is loaded inside the first launch that uses
   it, and the autotuner times each candidate shape by one generation. */
template <bool EXACT, bool BANK>
void preload_kernels() {
    static bool done[64] = {};           /* per device (modules load per context) */
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64 || done[dev]) return;
    done[dev] = true;
    cudaFuncAttributes fa;
    auto L = [&](const void* f) { cudaFuncGetAttributes(&fa, f); };
    L((const void*)pass_kernel<true, 1, EXACT, BANK, false, true>());
    L((const void*)pass_kernel<true, 1, EXACT, BANK, false, false>());
    L((const void*)pass_kernel<false, 1, EXACT, BANK, false, false>());
    L((const void*)pass_kernel<true, 0, EXACT, BANK, false, true>());
    L((const void*)pass_kernel<true, 0, EXACT, BANK, false, false>());
    L((const void*)pass_kernel<false, 0, EXACT, BANK, false, false>());
    L((const void*)pass_kernel<true, 2, EXACT, BANK, false, true>());
    L((const void*)pass_kernel<true, 3, EXACT, BANK, false, true>());
    L((const void*)ev_pass_wide<2, EXACT, BANK>);
    L((const void*)ev_pass_wide<3, EXACT, BANK>);
    L((const void*)ev_sort_flight<true, EXACT, BANK>);
    L((const void*)ev_sort_flight<false, EXACT, BANK>);
    L((const void*)ev_sort_collide<BANK>);
    L((const void*)ev_finalize);
    L((const void*)ev_fold_flush);
    if (BANK) {
        L((const void*)ev_scatter_hist);
        L((const void*)ev_scatter<SCAT_ONE>);
        L((const void*)ev_scatter<SCAT_TAB>);
        L((const void*)ev_scatter<SCAT_DIRECT>);
        L((const void*)ev_rb_scan);
        L((const void*)ev_rb_scatter);
        preload_bank_kernels();
    }
}
}  // namespace

int EventEngine::commit(cudaStream_t s, std::string& err) {
    Impl& m = *impl_;
    if (m.inst.empty()) { err = "no instances"; return NRAPS_ERR_INVALID; }
    uint32_t n = (uint32_t)m.inst.size();
    std::vector<uint64_t> ib(n + 1, 0), cb(n + 1, 0);
    for (uint32_t i = 0; i < n; ++i) {
        ib[i + 1] = ib[i] + m.inst[i]->d.N;
        cb[i + 1] = cb[i] + m.inst[i]->d.nc;
        m.inst[i]->d.hist_begin = ib[i];
        m.inst[i]->d.cell_begin = cb[i];
    }
    if (ib[n] >= (1ULL << 32)) { err = "at most 2^32-1 particles per batch generation"; return NRAPS_ERR_INVALID; }
    bool bank = m.mode == NRAPS_MODE_BANK;
    m.n_total = ib[n];
    m.n_cells_total = cb[n];
    std::vector<EvInst> d(n);
    uint64_t bank_sum = 0;
    for (uint32_t i = 0; i < n; ++i) { d[i] = m.inst[i]->d; bank_sum += m.inst[i]->b.bank_cap; }
    m.bank_sum = bank_sum;
    cudaError_t e = cudaSuccess;
    auto A = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
    /* shared buffers grow geometrically, so a batch whose membership changes
       between generations reallocates rarely */
    if (m.cap_inst < n) {
        m.cap_inst = std::max<uint64_t>(n, m.cap_inst + m.cap_inst / 2);
        A(m.d_inst.alloc(m.cap_inst)); A(m.d_inst_begin.alloc(m.cap_inst + 1)); A(m.d_cell_begin.alloc(m.cap_inst + 1));
    }
    A(cudaMemcpyAsync(m.d_inst.p, d.data(), n * sizeof(EvInst), cudaMemcpyHostToDevice, s));
    A(cudaMemcpyAsync(m.d_inst_begin.p, ib.data(), (n + 1) * 8, cudaMemcpyHostToDevice, s));
    A(cudaMemcpyAsync(m.d_cell_begin.p, cb.data(), (n + 1) * 8, cudaMemcpyHostToDevice, s));
    if (m.n_total > m.cap_total || !m.qx[0].p) {
        m.cap_total = std::max<uint64_t>(m.n_total, m.cap_total + m.cap_total / 2);
        uint64_t c = m.cap_total;
        for (int q = 0; q < 2; ++q) {
            A(m.qx[q].alloc(c)); A(m.qmu[q].alloc(c)); A(m.qrng[q].alloc(c));
            A(m.qid[q].alloc(c)); A(m.qpk[q].alloc(c));
        }
        A(m.count.alloc(c)); A(m.offsets.alloc(c + 1));
        A(m.block_sums.alloc((c + 4095) / 4096 + 1));
    }
    /* pass fills and claims, the finalize block count, the ranged bank's
       chunk count, the sorted rounds' collision-queue fills, the deferred
       close's and fold's block counts */
    constexpr size_t NCOUNT = 3 * (MAX_PASSES + 2) + 4;
    if (!m.qcount.p) { A(m.qcount.alloc(NCOUNT)); A(m.slab_count.alloc(NSLAB)); A(m.bstats.alloc(1)); }
    /* slabs: room for every banked site plus one partial flush per warp */
    uint64_t want_slab = bank ? (bank_sum + 2 * m.n_total) / NSLAB + 8192 : 64;
    if (want_slab > m.slab_cap || !m.sites.p) {
        m.slab_cap = std::max<uint64_t>(want_slab, m.slab_cap + m.slab_cap / 2);
        A(m.sites.alloc(NSLAB * m.slab_cap));
    }
    A(cudaMemsetAsync(m.qcount.p, 0, NCOUNT * 8, s));
    A(cudaMemsetAsync(m.slab_count.p, 0, NSLAB * 8, s));
    A(cudaMemsetAsync(m.bstats.p, 0, sizeof(GenState), s));
    if (bank && m.n_total) A(cudaMemsetAsync(m.count.p, 0, m.n_total * 4, s));
    if (e != cudaSuccess) { err = std::string("event engine buffers: ") + cudaGetErrorString(e); return NRAPS_ERR_NOMEM; }
    EvArgs& a = m.args;
    a.inst = m.d_inst.p; a.n_inst = n; a.inst_begin = m.d_inst_begin.p; a.cell_begin = m.d_cell_begin.p;
    a.n_total = m.n_total; a.n_cells_total = m.n_cells_total;
    for (int q = 0; q < 2; ++q) {
        a.qx[q] = m.qx[q].p; a.qmu[q] = m.qmu[q].p; a.qrng[q] = m.qrng[q].p; a.qid[q] = m.qid[q].p; a.qpk[q] = m.qpk[q].p;
    }
    a.qcount = m.qcount.p;
    a.claim = m.qcount.p + (MAX_PASSES + 2);
    a.blocks_done = m.qcount.p + 2 * (MAX_PASSES + 2);
    a.sites = m.sites.p;
    a.slab_count = m.slab_count.p; a.slab_cap = m.slab_cap;
    a.rb = 0;
    a.rb_next = m.qcount.p + 2 * (MAX_PASSES + 2) + 1;
    a.ccount = m.qcount.p + 2 * (MAX_PASSES + 2) + 2;
    a.scatter_done = m.qcount.p + 3 * (MAX_PASSES + 2) + 2;
    a.fold_done = m.qcount.p + 3 * (MAX_PASSES + 2) + 3;
    a.fold_from = 0xFFFFFFFFu;
    a.scatter_close = 0;
    a.rb_pool_chunks = 0;
    a.rb_chunk = nullptr; a.rb_fill = nullptr; a.rb_base = nullptr; a.rb_total = nullptr;
    a.count = m.count.p; a.offsets = m.offsets.p; a.tile_sums = nullptr; a.n_tiles = 0;
    a.stats = (n == 1) ? m.inst[0]->d.st : m.bstats.p;
    a.max_events = m.max_events;
    a.rec = m.rec;
    a.bank = bank ? 1 : 0;
    /* one instance whose tables fit: stage them in shared memory */
    m.one = false;
    m.smem_bytes = 0;
    if (n == 1) {
        const EvInst& I = m.inst[0]->d;
        size_t sb = smem_bytes_for(I.M, I.G, I.R, I.nbins);
        if (sb <= 120 * 1024) { m.one = true; m.smem_bytes = sb; }
    }
    a.hist_smem = (m.one && bank && m.inst[0]->d.nc <= HIST_SMEM_MAX_CELLS) ? 1 : 0;
    /* ranged launches: do every instance's tables fit shared memory? */
    a.range_len = 0;
    a.range_begin = nullptr;
    {
        size_t tmax = 0;
        for (uint32_t i = 0; i < n; ++i) {
            const EvInst& I = m.inst[i]->d;
            tmax = std::max(tmax, smem_bytes_for(I.M, I.G, I.R, I.nbins));
        }
        m.ranged_fit = tmax <= RANGED_SMEM_MAX;
        m.ranged_smem = (tmax + 15) / 16 * 16;
        m.range_built = 0;
    }
    if (!m.nlog2n.p) {
        std::vector<double> t(NLOG2N_TAB, 0.0);
        for (uint32_t i = 2; i < NLOG2N_TAB; ++i) t[i] = (double)i * nr_log((double)i) * LOG2E;
        if (m.nlog2n.alloc(NLOG2N_TAB) != cudaSuccess ||
            cudaMemcpy(m.nlog2n.p, t.data(), NLOG2N_TAB * 8, cudaMemcpyHostToDevice) != cudaSuccess) {
            err = "event engine buffers: entropy table";
            return NRAPS_ERR_NOMEM;
        }
    }
    a.nlog2n = m.nlog2n.p;
    if (bank) { if (m.exact) preload_kernels<true, true>(); else preload_kernels<false, true>(); }
    else { if (m.exact) preload_kernels<true, false>(); else preload_kernels<false, false>(); }
    m.committed = true;
    return size_grid();
}

int EventEngine::size_grid() {
    Impl& m = *impl_;
    if (params.range && m.range_built != params.range && m.committed) {
        /* range prefix for params.range histories per block */
        const uint32_t n = (uint32_t)m.inst.size(), RL = params.range;
        std::vector<uint32_t> rb(n + 1, 0);
        for (uint32_t i = 0; i < n; ++i) rb[i + 1] = rb[i] + (uint32_t)((m.inst[i]->d.N + RL - 1) / RL);
        if (m.d_range_begin.n < n + 1 && m.d_range_begin.alloc(std::max<size_t>(n + 1, 2 * m.d_range_begin.n)) != cudaSuccess)
            return NRAPS_ERR_NOMEM;
        if (cudaMemcpy(m.d_range_begin.p, rb.data(), (n + 1) * 4, cudaMemcpyHostToDevice) != cudaSuccess)
            return NRAPS_ERR_CUDA;
        m.ranged_blocks = rb[n];
        m.range_built = RL;
        /* ranged bank: chunk lists, fills and bases per range, a pool with
           room for every banked site plus one partial chunk per range */
        m.rb_ok = false;
        if (m.mode == NRAPS_MODE_BANK) {
            const uint64_t R = m.ranged_blocks;
            const uint64_t chunks = (m.bank_sum + RB_CHUNK - 1) / RB_CHUNK + R + 1;
            if (chunks >= RB_FULL) return NRAPS_ERR_INVALID;
            cudaError_t e = cudaSuccess;
            auto A = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
            if (m.rb_chunk.n < R * RB_MAXC) A(m.rb_chunk.alloc(R * RB_MAXC));
            if (m.rb_fill.n < R) A(m.rb_fill.alloc(R));
            if (m.rb_base.n < R) A(m.rb_base.alloc(R));
            if (m.rb_total.n < n) A(m.rb_total.alloc(n));
            if (m.sites.n < chunks * RB_CHUNK) {
                A(m.sites.alloc(chunks * RB_CHUNK));
                m.args.sites = m.sites.p;
            }
            if (e != cudaSuccess) return NRAPS_ERR_NOMEM;
            uint32_t hc = 0;
            for (uint32_t i = 0; i < n; ++i)
                if (m.inst[i]->d.nc <= RB_HIST_SMEM) hc = std::max(hc, m.inst[i]->d.nc);
            m.rb_hist_cells = hc;
            m.rb_pool_chunks = (uint32_t)chunks;
            m.rb_ok = true;
        }
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    /* persistent grid: as many blocks as are resident at once */
    int per_sm = 0;
    const void* fn = m.one ? (m.exact ? (const void*)pass_kernel<true, 1, true, true, false, true>()
                                      : (const void*)pass_kernel<true, 1, false, true, false, true>())
                           : (const void*)pass_kernel<true, 0, false, true, false, true>();
    const size_t dyn = stage_bytes(params.block) + (m.one ? m.smem_bytes : 0);
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, (int)params.block, dyn) != cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    m.grid_blocks = sms * per_sm;
    /* sorted transport (one instance, no records): the collision queue, and
       a persistent grid for its kernels */
    m.sort_grid = 0;
    if (m.one && params.sort && m.rec == nullptr) {
        if (m.cx.n < m.n_total) {
            cudaError_t e = cudaSuccess;
            auto A = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
            A(m.cx.alloc(m.cap_total)); A(m.cmu.alloc(m.cap_total)); A(m.crng.alloc(m.cap_total));
            A(m.cid.alloc(m.cap_total)); A(m.cpk.alloc(m.cap_total)); A(m.creg.alloc(m.cap_total));
            if (e != cudaSuccess) return NRAPS_ERR_NOMEM;
        }
        EvArgs& a = m.args;
        a.cx = m.cx.p; a.cmu = m.cmu.p; a.crng = m.crng.p; a.cid = m.cid.p; a.cpk = m.cpk.p; a.creg = m.creg.p;
        int pb = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pb, ev_sort_collide<true>, 256, SORT_STAGE_BYTES) != cudaSuccess ||
            pb < 1)
            pb = 1;
        m.sort_grid = sms * pb;
    }
    return NRAPS_OK;
}

uint64_t EventEngine::launches_per_generation() const {
    if (impl_->sort_grid) return 2 * (uint64_t)params.sort + 1;
    return params.passes == 0 ? 1 : 1 + params.passes;
}

int EventEngine::flush_fold(cudaStream_t s) {
    Impl& m = *impl_;
    if (!m.fold_maybe_pending) return 0;
    const unsigned nb = (unsigned)std::max<uint64_t>(1, (m.inst[0]->d.nc + FIN_THREADS - 1) / FIN_THREADS);
    if (launch_k(m.pdl, ev_fold_flush, dim3(nb), dim3(FIN_THREADS), 0, s, m.args) != cudaSuccess) return -1;
    m.fold_maybe_pending = false;
    return 1;
}

int EventEngine::enqueue_generation(cudaStream_t s, bool with_finalize, cudaEvent_t t0, cudaEvent_t t1) {
    Impl& m = *impl_;
    if (!m.committed) return -1;
    const EvArgs& a = m.args;
    bool bank = m.mode == NRAPS_MODE_BANK;
    bool rec = m.rec != nullptr;
    const bool ranged_launch =
        !rec && params.range && params.passes == 0 && m.range_built == params.range && (!bank || m.rb_ok);
    /* deferred end of generation: one instance with a two-half tally, one
       pass, cells counted in shared memory.  The scatter's last block closes
       the generation and the next transport launch's extra blocks fold it. */
    const bool deferred = with_finalize && a.hist_smem && !rec && !ranged_launch && params.passes == 0 &&
                          !m.sort_grid && m.inst[0]->d.tally_stride != 0;
    const uint32_t fold_blocks =
        deferred ? (uint32_t)((m.inst[0]->d.nc + params.block - 1) / params.block) : 0u;
    int n = 0;
    if (!deferred && m.fold_maybe_pending) {
        /* a generation that closes the classic way: fold the pending one first */
        const int q = flush_fold(s);
        if (q < 0) return -1;
        n += q;
    }
    /* arguments of the kernels after the transport (the ranged bank's
       buffers when a ranged launch uses it) */
    EvArgs ar = a;
    if (t0) cudaEventRecord(t0, s);
    int r;
#define EV_LAUNCH(ONE, EXACT, BANK, REC) \
    r = launch_passes<ONE, EXACT, BANK, REC>(a, params, m.grid_blocks, ONE ? m.smem_bytes : 0, m.n_total, s, m.pdl, \
                                             fold_blocks)
    if (rec && m.one) {
        if (bank) { if (m.exact) EV_LAUNCH(true, true, true, true); else EV_LAUNCH(true, false, true, true); }
        else { if (m.exact) EV_LAUNCH(true, true, false, true); else EV_LAUNCH(true, false, false, true); }
    } else if (rec) {
        /* one instance whose tables do not fit shared memory: read them
           from global memory, as batched launches do */
        if (bank) { if (m.exact) EV_LAUNCH(false, true, true, true); else EV_LAUNCH(false, false, true, true); }
        else { if (m.exact) EV_LAUNCH(false, true, false, true); else EV_LAUNCH(false, false, false, true); }
    } else if (ranged_launch) {
        ar.range_len = params.range;
        ar.range_begin = m.d_range_begin.p;
        if (bank) {
            ar.rb = 1;
            ar.rb_pool_chunks = m.rb_pool_chunks;
            ar.rb_chunk = m.rb_chunk.p; ar.rb_fill = m.rb_fill.p;
            ar.rb_base = m.rb_base.p; ar.rb_total = m.rb_total.p;
        }
        if (m.ranged_fit) {
            const size_t rs = stage_bytes(params.block) + m.ranged_smem;
#define EV_RANGED(EXACT, BANK) \
    if (params.block == 512) { \
        cudaFuncSetAttribute(ev_pass_wide<2, EXACT, BANK>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rs); \
        launch_k(m.pdl, ev_pass_wide<2, EXACT, BANK>, dim3(m.ranged_blocks), dim3(512), rs, s, ar, 0, 0xFFFFFFFFu, 0u); \
    } else { \
        set_smem_attr<true, 2, EXACT, BANK, false, true>(rs); \
        launch_k(m.pdl, ev_pass<true, 2, EXACT, BANK, false, true>, dim3(m.ranged_blocks), dim3(params.block), rs, s, \
                 ar, 0, 0xFFFFFFFFu, 0u); \
    }
            if (bank) { if (m.exact) { EV_RANGED(true, true); } else { EV_RANGED(false, true); } }
            else { if (m.exact) { EV_RANGED(true, false); } else { EV_RANGED(false, false); } }
#undef EV_RANGED
        } else {
            const size_t rs = stage_bytes(params.block);
#define EV_RANGED(EXACT, BANK) \
    if (params.block == 512) { \
        cudaFuncSetAttribute(ev_pass_wide<3, EXACT, BANK>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rs); \
        launch_k(m.pdl, ev_pass_wide<3, EXACT, BANK>, dim3(m.ranged_blocks), dim3(512), rs, s, ar, 0, 0xFFFFFFFFu, 0u); \
    } else { \
        set_smem_attr<true, 3, EXACT, BANK, false, true>(rs); \
        launch_k(m.pdl, ev_pass<true, 3, EXACT, BANK, false, true>, dim3(m.ranged_blocks), dim3(params.block), rs, s, \
                 ar, 0, 0xFFFFFFFFu, 0u); \
    }
            if (bank) { if (m.exact) { EV_RANGED(true, true); } else { EV_RANGED(false, true); } }
            else { if (m.exact) { EV_RANGED(true, false); } else { EV_RANGED(false, false); } }
#undef EV_RANGED
        }
        r = cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
    } else if (m.one && m.sort_grid) {
        const uint32_t R = params.sort;
        const dim3 sg((unsigned)m.sort_grid), sb(256);
        for (uint32_t rd = 0; rd < R; ++rd) {
#define EV_SORT_FLIGHT(FIRST, EXACT, BANK) launch_k(m.pdl, ev_sort_flight<FIRST, EXACT, BANK>, sg, sb, 0, s, a, (int)rd)
            if (rd == 0) {
                if (bank) { if (m.exact) EV_SORT_FLIGHT(true, true, true); else EV_SORT_FLIGHT(true, false, true); }
                else { if (m.exact) EV_SORT_FLIGHT(true, true, false); else EV_SORT_FLIGHT(true, false, false); }
            } else {
                if (bank) { if (m.exact) EV_SORT_FLIGHT(false, true, true); else EV_SORT_FLIGHT(false, false, true); }
                else { if (m.exact) EV_SORT_FLIGHT(false, true, false); else EV_SORT_FLIGHT(false, false, false); }
            }
#undef EV_SORT_FLIGHT
            if (bank) launch_k(m.pdl, ev_sort_collide<true>, sg, sb, SORT_STAGE_BYTES, s, a, (int)rd);
            else launch_k(m.pdl, ev_sort_collide<false>, sg, sb, SORT_STAGE_BYTES, s, a, (int)rd);
        }
        /* the survivors of the last round run to their ends: pass R reads
           round R-1's output queue */
        const size_t smem = stage_bytes(params.block) + m.smem_bytes;
#define EV_SORT_TAIL(EXACT, BANK) \
    set_smem_attr<false, 1, EXACT, BANK, false, false>(smem); \
    launch_k(m.pdl, pass_kernel<false, 1, EXACT, BANK, false, false>(), dim3((unsigned)m.grid_blocks), \
             dim3(params.block), smem, s, a, (int)R, 0xFFFFFFFFu, 0u)
        if (bank) { if (m.exact) { EV_SORT_TAIL(true, true); } else { EV_SORT_TAIL(false, true); } }
        else { if (m.exact) { EV_SORT_TAIL(true, false); } else { EV_SORT_TAIL(false, false); } }
#undef EV_SORT_TAIL
        r = cudaPeekAtLastError() == cudaSuccess ? (int)(2 * R + 1) : -1;
    } else if (m.one) {
        if (bank) { if (m.exact) EV_LAUNCH(true, true, true, false); else EV_LAUNCH(true, false, true, false); }
        else { if (m.exact) EV_LAUNCH(true, true, false, false); else EV_LAUNCH(true, false, false, false); }
    } else {
        if (bank) { if (m.exact) EV_LAUNCH(false, true, true, false); else EV_LAUNCH(false, false, true, false); }
        else { if (m.exact) EV_LAUNCH(false, true, false, false); else EV_LAUNCH(false, false, false, false); }
    }
#undef EV_LAUNCH
    if (r < 0) return -1;
    if (t1) cudaEventRecord(t1, s);
    n += r;
    if (bank && ar.rb) {
        launch_k(m.pdl, ev_rb_scan, dim3(a.n_inst), dim3(RB_THREADS), 0, s, ar);
        const size_t hb = ((size_t)rb_loc_words(ar.range_len) + m.rb_hist_cells) * 4;
        if (hb > 40 * 1024) cudaFuncSetAttribute(ev_rb_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hb);
        launch_k(m.pdl, ev_rb_scatter, dim3(m.ranged_blocks), dim3(RB_THREADS), hb, s, ar);
        n += 2;
    } else if (bank) {
        /* deferred end of generation: one scan launch of offsets within
           tiles; the scatter adds the tiles' bases */
        const uint64_t tiles = (m.n_total + (1ull << NR_SCAN_TILE_LOG2) - 1) >> NR_SCAN_TILE_LOG2;
        const bool local = deferred && tiles <= LOCAL_SCAN_MAX_TILES;
        int q = local ? launch_scan_local(m.count.p, m.n_total, m.block_sums.p, m.offsets.p, s, m.pdl)
                      : launch_exclusive_scan(m.count.p, m.n_total, m.block_sums.p, m.offsets.p, nullptr, s, m.pdl);
        if (q < 0) return -1;
        n += q;
        if (a.hist_smem) {
            const size_t hb = ((size_t)m.inst[0]->d.nc + (local ? tiles : 0)) * 4;
            if (hb > 40 * 1024)
                cudaFuncSetAttribute(ev_scatter_hist, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hb);
            EvArgs as = a;
            as.scatter_close = deferred ? 1 : 0;
            if (local) { as.tile_sums = m.block_sums.p; as.n_tiles = (uint32_t)tiles; }
            launch_k(m.pdl, ev_scatter_hist, dim3(NSLAB * SCATTER_ONE_SPLIT + (deferred ? 1 : 0)),
                     dim3(SCATTER_ONE_THREADS), hb, s, as);
        } else if (m.one || rec) {
            launch_k(m.pdl, ev_scatter<SCAT_ONE>, dim3(NSLAB * 8), dim3(256), 0, s, a);
        } else if (a.n_inst <= SCAT_TAB_MAX) {
            launch_k(m.pdl, ev_scatter<SCAT_TAB>, dim3(NSLAB * 8), dim3(256), (size_t)a.n_inst * SCAT_TAB_BYTES, s, a);
        } else {
            launch_k(m.pdl, ev_scatter<SCAT_DIRECT>, dim3(NSLAB * 8), dim3(256), 0, s, a);
        }
        ++n;
    }
    if (deferred) m.fold_maybe_pending = true;
    if (with_finalize && !deferred) {
        unsigned gb = (unsigned)std::min<uint64_t>((m.n_cells_total + FIN_THREADS - 1) / FIN_THREADS,
                                                   (uint64_t)m.grid_blocks * 4);
        launch_k(m.pdl, ev_finalize, dim3(gb ? gb : 1), dim3(FIN_THREADS), 0, s, ar);
        n += 1;
    }
    return cudaPeekAtLastError() == cudaSuccess ? n : -1;
}
