/*
 * bank.cu — fission-bank ordering, Shannon entropy and the per-generation
 * FP64 finalize (k estimator, flux/fission-source accumulation).
 *
 * Bank order.  Transport kernels append sites in whatever order warps reach
 * them, each tagged (parent history, sequence number within that history),
 * and every history writes how many sites it banked.  An exclusive scan of
 * those counts gives each parent's first slot, so site (p, s) lands at
 * offset[p] + s: the ordered bank is a pure function of the histories, not of
 * thread scheduling.  The next generation's particle i takes ordered site
 * floor(i * B / N) (systematic resampling to N source particles).
 *
 * Finalize follows the reference's generation bookkeeping
 * (src/mc_code.rs:340-363) in FP64: flux = tally/(k*N*dx),
 * fission_source = nu*sigf*flux, conversion = 3565e6*k*36.2 /
 * (200e6*1.602176634e-19*nu[M]*L); COMPAT takes k_new = sum(k*dx*fs) over the
 * tally bins, PHYSICS/BANK take the exact fixed-point track-length score.
 * Reductions use a fixed tree, so repeated runs give identical k.
 */
#include "engine.cuh"
#include "nr_math.h"
#include "dev_util.cuh"

using nrdev::block_excl_scan;

namespace {

constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;
static_assert(SCAN_TILE == (1 << NR_SCAN_TILE_LOG2), "scan tile size");
static_assert(SCAN_ITEMS == 4, "a thread's items are one 16-byte vector");

/* a thread's SCAN_ITEMS counts from `base` (a multiple of 4): one 16-byte
   load when all lie below n and the array is 16-byte aligned (device
   allocations are), else one by one with zeros past n */
__device__ __forceinline__ uint4 load_items(const uint32_t* count, uint64_t n, uint64_t base) {
    if (base + 3 < n && (reinterpret_cast<uintptr_t>(count) & 15u) == 0)
        return reinterpret_cast<const uint4*>(count)[base >> 2];
    uint4 v;
    v.x = base < n ? count[base] : 0u;
    v.y = base + 1 < n ? count[base + 1] : 0u;
    v.z = base + 2 < n ? count[base + 2] : 0u;
    v.w = base + 3 < n ? count[base + 3] : 0u;
    return v;
}

/* the exclusive prefix of a thread's items, from `run`, to offsets[base..) */
__device__ __forceinline__ void store_items(uint32_t* offsets, uint64_t n, uint64_t base, uint32_t run, uint4 v) {
    uint4 o;
    o.x = run; o.y = o.x + v.x; o.z = o.y + v.y; o.w = o.z + v.z;
    if (base + 3 < n && (reinterpret_cast<uintptr_t>(offsets) & 15u) == 0) {
        reinterpret_cast<uint4*>(offsets)[base >> 2] = o;
        return;
    }
    if (base < n) offsets[base] = o.x;
    if (base + 1 < n) offsets[base + 1] = o.y;
    if (base + 2 < n) offsets[base + 2] = o.z;
    if (base + 3 < n) offsets[base + 3] = o.w;
}

__global__ void __launch_bounds__(SCAN_THREADS) scan_tile_sums(const uint32_t* count, uint64_t n,
                                                               uint32_t* block_sums) {
    __shared__ uint32_t sw[33];
    nrdev::pdl_trigger();
    nrdev::pdl_wait();
    uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_ITEMS;
    const uint4 v = load_items(count, n, base);
    uint32_t s = v.x + v.y + v.z + v.w;
    uint32_t ex;
    uint32_t tot = block_excl_scan(s, &ex, sw);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(SCAN_THREADS) scan_top(uint32_t* block_sums, uint64_t nb,
                                                         unsigned long long* total, uint32_t* offsets_end) {
    __shared__ uint32_t sw[33];
    nrdev::pdl_trigger();
    nrdev::pdl_wait();
    uint32_t carry = 0;
    for (uint64_t b0 = 0; b0 < nb; b0 += SCAN_THREADS) {
        uint64_t i = b0 + threadIdx.x;
        uint32_t v = i < nb ? block_sums[i] : 0u;
        uint32_t ex;
        uint32_t tot = block_excl_scan(v, &ex, sw);
        if (i < nb) block_sums[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) {
        if (total) *total = carry;
        if (offsets_end) *offsets_end = carry;
    }
}

__global__ void __launch_bounds__(SCAN_THREADS) scan_apply(const uint32_t* count, uint64_t n,
                                                           const uint32_t* block_sums, uint32_t* offsets) {
    __shared__ uint32_t sw[33];
    nrdev::pdl_trigger();
    nrdev::pdl_wait();
    uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_ITEMS;
    const uint4 v = load_items(count, n, base);
    uint32_t s = v.x + v.y + v.z + v.w;
    uint32_t ex;
    block_excl_scan(s, &ex, sw);
    store_items(offsets, n, base, block_sums[blockIdx.x] + ex, v);
}

/* scan_top folded into scan_apply: each tile sums the tile totals before it
   itself (a block reduction over at most SCAN_CARRY_MAX_TILES values), so a
   scan of up to 16.7M counts takes two launches instead of three; the last
   tile writes the grand total. */
constexpr uint64_t SCAN_CARRY_MAX_TILES = NR_SCAN_CARRY_MAX_TILES;

__global__ void __launch_bounds__(SCAN_THREADS) scan_apply_carry(const uint32_t* count, uint64_t n,
                                                                 const uint32_t* tile_sums, uint64_t nb,
                                                                 uint32_t* offsets, unsigned long long* total) {
    __shared__ uint32_t sw[33];
    nrdev::pdl_trigger();
    nrdev::pdl_wait();
    uint32_t c = 0;
    for (uint64_t i = threadIdx.x; i < blockIdx.x; i += SCAN_THREADS) c += tile_sums[i];
    uint32_t ex0;
    const uint32_t carry = block_excl_scan(c, &ex0, sw);
    __syncthreads();
    uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_ITEMS;
    const uint4 v = load_items(count, n, base);
    uint32_t s = v.x + v.y + v.z + v.w;
    uint32_t ex;
    const uint32_t tot = block_excl_scan(s, &ex, sw);
    store_items(offsets, n, base, carry + ex, v);
    if (blockIdx.x == nb - 1 && threadIdx.x == 0) {
        offsets[n] = carry + tot;
        if (total) *total = carry + tot;
    }
}

/* Per tile: the exclusive scan of its counts from the tile's start (local
   offsets) and the tile's total.  A consumer that adds the tiles' bases
   itself (an exclusive scan of the tile totals) gets the whole scan from
   this one launch. */
__global__ void __launch_bounds__(SCAN_THREADS) scan_local(const uint32_t* count, uint64_t n, uint32_t* tile_sums,
                                                           uint32_t* offsets) {
    __shared__ uint32_t sw[33];
    nrdev::pdl_trigger();
    nrdev::pdl_wait();
    const uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_ITEMS;
    const uint4 v = load_items(count, n, base);
    uint32_t ex;
    const uint32_t tot = block_excl_scan(v.x + v.y + v.z + v.w, &ex, sw);
    store_items(offsets, n, base, ex, v);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = tot;
}

__global__ void bank_scatter(BankArgs a) {
    const GenState* st = a.st;
    uint64_t n = st->n_sites;
    if (n > a.sink.cap) n = a.sink.cap;
    nraps_site* out = a.bank[(st->gen + 1) & 1];
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t pos = (uint64_t)a.offsets[a.sink.parent[i]] + a.sink.seq[i];
        if (pos < a.bank_cap) {
            nraps_site s;
            s.x = a.sink.x[i];
            s.cell = a.sink.cell[i];
            s.group = a.sink.group[i];
            s.pad = 0;
            out[pos] = s;
            atomicAdd(&a.hist[s.cell], 1u);
        }
    }
}

__device__ __forceinline__ double block_sum_d(double v, double* sm) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0) sm[w] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0) for (int i = 0; i < nw; ++i) r += sm[i];
    __syncthreads();
    return r;
}

constexpr int FIN_THREADS = 256;

/* one thread per cell: reads and clears the cell's G tally bins */
__global__ void __launch_bounds__(FIN_THREADS) finalize_bins(FinalizeArgs a) {
    __shared__ double sm[FIN_THREADS / 32];
    const GenState* st = a.st;
    const uint64_t gen = st->gen;
    const double k = st->k;
    const bool active = gen >= a.skip;
    double fund;
    if (a.mode == NRAPS_MODE_COMPAT) fund = 1.0 / (double)(uint64_t)(a.generations - (a.skip - 1));
    else fund = 1.0 / (double)(a.generations - a.skip);
    const double conversion = a.conv_const * k;
    const double N = (double)a.N;
    double kpart = 0.0, hpart = 0.0;
    const double B = (double)st->n_bank_next;
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < a.nc;
         c += (uint64_t)gridDim.x * blockDim.x) {
        double dx = a.dx64[c];
        uint32_t m = a.mat[c];
        double fs = 0.0;
        for (uint32_t g = 0; g < a.G; ++g) {
            uint64_t bin = (uint64_t)g * a.nc + c;
            double t = a.tally[bin];
            a.tally[bin] = 0.0;
            double flux = t / (k * N * dx);
            double f = a.nsf64[m + (uint64_t)a.M * g] * flux;
            kpart += k * dx * f;
            fs += f;
            double phi = t / (N * dx);
            if (active) {
                a.flux_acc[bin] += flux * conversion * fund;
                a.flux_sum[bin] += phi;
                a.flux_sq[bin] += phi * phi;
            }
        }
        if (active) a.fs_acc[c] += fs * fund;
        if (a.bank_mode) {
            uint32_t cnt = a.hist[c];
            a.hist_w[c] = 0;
            if (cnt && B > 0.0) {
                double p = (double)cnt / B;
                hpart -= p * nr_log(p) * 1.4426950408889634;   /* log2 */
            }
        }
    }
    double ks = block_sum_d(kpart, sm);
    double hs = block_sum_d(hpart, sm);
    if (threadIdx.x == 0) {
        a.partials[2 * blockIdx.x] = ks;
        a.partials[2 * blockIdx.x + 1] = hs;
    }
}

__global__ void finalize_state(FinalizeArgs a) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    GenState* st = a.st;
    double ks = 0.0, hs = 0.0;
    for (uint32_t b = 0; b < a.n_blocks; ++b) { ks += a.partials[2 * b]; hs += a.partials[2 * b + 1]; }
    double k_new = (a.mode == NRAPS_MODE_COMPAT) ? ks : nr_unfix(st->kq) / (double)a.N;
    uint64_t gen = st->gen;
    if (gen < a.generations) {
        a.k64[gen] = k_new;
        if (gen >= a.skip) { st->ksum += k_new; st->ksum2 += k_new * k_new; st->nactive++; }
        a.entropy[gen] = a.bank_mode ? hs : 0.0;
    }
    if (a.bank_mode) {
        unsigned long long b = st->n_bank_next;
        if (b > a.bank_cap) { b = a.bank_cap; st->error |= NR_ERR_CAPACITY; }
        st->n_bank = b;
        if (b == 0) st->error |= NR_ERR_EMPTY;
        st->tot_sites += st->n_sites;
    }
    st->tot_collisions += st->collisions;
    st->tot_virtual += st->virtual_collisions;
    st->tot_crossings += st->crossings;
    st->tot_absorbed += st->absorbed;
    st->tot_leaked += st->leaked;
    st->tot_capped += st->capped;
    st->collisions = st->virtual_collisions = st->crossings = 0;
    st->absorbed = st->leaked = st->capped = 0;
    st->n_sites = 0;
    st->n_bank_next = 0;
    st->kq = 0;
    st->k = k_new;
    st->inv_kf = (float)(1.0 / k_new);
    st->gen = gen + 1;
}

}  // namespace

void preload_bank_kernels() {
    cudaFuncAttributes fa;
    cudaFuncGetAttributes(&fa, scan_tile_sums);
    cudaFuncGetAttributes(&fa, scan_top);
    cudaFuncGetAttributes(&fa, scan_apply);
    cudaFuncGetAttributes(&fa, scan_apply_carry);
    cudaFuncGetAttributes(&fa, scan_local);
}

int launch_exclusive_scan(const uint32_t* count, uint64_t n, uint32_t* block_sums, uint32_t* offsets,
                          unsigned long long* total, cudaStream_t s, bool pdl) {
    uint64_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (nb == 0) return 0;
    if (launch_k(pdl, scan_tile_sums, dim3((unsigned)nb), dim3(SCAN_THREADS), 0, s, count, n, block_sums) != cudaSuccess)
        return -1;
    if (nb <= SCAN_CARRY_MAX_TILES) {
        if (launch_k(pdl, scan_apply_carry, dim3((unsigned)nb), dim3(SCAN_THREADS), 0, s, count, n, block_sums, nb,
                     offsets, total) != cudaSuccess)
            return -1;
        return 2;
    }
    if (launch_k(pdl, scan_top, dim3(1), dim3(SCAN_THREADS), 0, s, block_sums, nb, total, offsets + n) != cudaSuccess ||
        launch_k(pdl, scan_apply, dim3((unsigned)nb), dim3(SCAN_THREADS), 0, s, count, n, block_sums, offsets) !=
            cudaSuccess)
        return -1;
    return 3;
}

int launch_scan_local(const uint32_t* count, uint64_t n, uint32_t* tile_sums, uint32_t* offsets, cudaStream_t s,
                      bool pdl) {
    const uint64_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (nb == 0) return 0;
    if (launch_k(pdl, scan_local, dim3((unsigned)nb), dim3(SCAN_THREADS), 0, s, count, n, tile_sums, offsets) !=
        cudaSuccess)
        return -1;
    return 1;
}

int launch_bank_order(const BankArgs& a, cudaStream_t s) {
    int q = launch_exclusive_scan(a.sink.count, a.n_hist, a.block_sums, a.offsets, &a.st->n_bank_next, s);
    if (q < 0) return -1;
    uint64_t grid = (a.sink.cap + 255) / 256;
    if (grid > 152 * 16) grid = 152 * 16;
    if (grid == 0) grid = 1;
    bank_scatter<<<(unsigned)grid, 256, 0, s>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? q + 1 : -1;
}

int launch_finalize(const FinalizeArgs& a, cudaStream_t s) {
    finalize_bins<<<a.n_blocks, FIN_THREADS, 0, s>>>(a);
    finalize_state<<<1, 32, 0, s>>>(a);
    return cudaPeekAtLastError() == cudaSuccess ? 2 : -1;
}

uint32_t finalize_blocks_for(uint64_t nc) {
    uint64_t b = (nc + FIN_THREADS - 1) / FIN_THREADS;
    if (b > 152 * 4) b = 152 * 4;
    if (b == 0) b = 1;
    return (uint32_t)b;
}
