/*
 * plain.cu — the plain drop-in: one thread per history, surface tracking
 * across every tally cell, track-length tallies accumulated in FP64.
 *
 * COMPAT follows NRAPS's particle_lifetime/particle_travel
 * (src/mc_code.rs:134-257) expression for expression, quirks included:
 *   spawn_neutron draw order (mc_code.rs:46-51), delta_s = mu*(-ln r)*inv_sigtr
 *   (:148), boundary/crossing/collision tests (:159-184), hit_boundary and
 *   cross_mesh arithmetic (:55-79), scat_mat_calc normalised by 1/sigs of the
 *   stale xs index (:186-192), interaction's draw order with one fresh uniform
 *   per binary-search probe (:113-132), and the stale xs index for the next
 *   flight after a scatter (:209).
 * PHYSICS/BANK carry the track length explicitly (no 0/0 at mu == 0), refresh
 * the xs index after every scatter, sample the scatter group with one draw,
 * and (BANK) bank floor(nu*sigf/sigtr/k + r) sites per collision.  Their
 * distance to a face is (face - x) * (1/mu), 1/mu set with mu, and a
 * history's k score is summed by fused multiply-adds in FP64 and fixed to
 * 2^-32 once at the history's end (the crossing loop is bound by the FP64
 * pipe: these remove a division and a conversion per crossing).
 *
 * This translation unit is compiled with --fmad=false and -prec-div=true: the
 * results must match a CPU restatement bit for bit, so no multiply-add may be
 * fused.  FP64 throughput on GB300 is a small fraction of FP32; this kernel is
 * the faithful baseline, the event-based Woodcock kernel is the fast form.
 */
#include "engine.cuh"
#include "nr_math.h"
#include "dev_util.cuh"

namespace {

template <class T> __device__ __forceinline__ T u01(uint32_t u);
template <> __device__ __forceinline__ float u01<float>(uint32_t u) { return nr_u01f(u); }
template <> __device__ __forceinline__ double u01<double>(uint32_t u) { return nr_u01d(u); }
template <class T> __device__ __forceinline__ T upos(uint32_t u);
template <> __device__ __forceinline__ float upos<float>(uint32_t u) { return nr_upos_f(u); }
template <> __device__ __forceinline__ double upos<double>(uint32_t u) { return nr_upos_d(u); }
__device__ __forceinline__ float lg(float x) { return nr_logf(x); }
__device__ __forceinline__ double lg(double x) { return nr_log(x); }
template <class T> __device__ __forceinline__ T tinf();
template <> __device__ __forceinline__ float tinf<float>() { return __int_as_float(0x7f800000); }
template <> __device__ __forceinline__ double tinf<double>() { return __longlong_as_double(0x7ff0000000000000LL); }

struct Rng {
    nr_pcg32 s;
    uint64_t draws;
    __device__ uint32_t next() { ++draws; return nr_pcg32_next(&s); }
};

struct Counters {
    uint64_t kq;
    uint32_t coll, cross, absorbed, leaked, capped;
};

using nrdev::agg_inc;

/* Rust partition_point, fixed-iteration form, deterministic predicate x < v */
template <class T>
__device__ __forceinline__ uint32_t energy_pp(const T* cdf, uint32_t G, T chi) {
    uint32_t base = 0, size = G;
    while (size > 1) {
        uint32_t half = size / 2, mid = base + half;
        if (cdf[mid] < chi) base = mid;
        size -= half;
    }
    uint32_t r = base + ((cdf[base] < chi) ? 1u : 0u);
    return r < G - 1 ? r : G - 1;
}

template <class T>
__device__ void emit_site(const PlainArgs<T>& a, T x, uint64_t cell, uint32_t g,
                          uint64_t h, uint32_t seq) {
    unsigned long long i = agg_inc(&a.st->n_sites);
    if (i < a.sink.cap) {
        a.sink.x[i] = (float)x;
        a.sink.cell[i] = (uint32_t)cell;
        a.sink.group[i] = g;
        a.sink.parent[i] = (uint32_t)h;
        a.sink.seq[i] = seq;
    } else {
        atomicOr(&a.st->error, NR_ERR_CAPACITY);
    }
}

template <class T>
__device__ void compat_history(const PlainArgs<T>& a, uint64_t h, uint64_t seed,
                               Counters& c, nraps_history_record* out) {
    Rng rng{nr_pcg32_seeded(seed, h), 0};
    const uint64_t last = a.nc - 1;
    const uint32_t G = a.G, M = a.M;
    uint64_t cell = __ldg(&a.fuel[((uint64_t)rng.next() * a.nfuel) >> 32]);
    T sub = u01<T>(rng.next());
    T mu = T(2) * u01<T>(rng.next()) - T(1);
    uint32_t g = energy_pp<T>(a.chi_cdf + (uint64_t)__ldg(&a.mat[cell]) * G, G, u01<T>(rng.next()));
    T x = __ldg(&a.left[cell]) + sub * a.dx_fuel;
    uint64_t events = 0;
    nraps_history_record rec = {};
    int fate = NRAPS_FATE_ABSORBED;
    for (;;) {
        rec.segments++;
        uint64_t xs = __ldg(&a.mat[cell]) + (uint64_t)M * g;
        T ds = mu * -lg(u01<T>(rng.next())) * __ldg(&a.inv_sigtr[xs]);
        bool stop = false, same = true;
        while (same) {
            if (++events > a.max_events) { fate = NRAPS_FATE_CAPPED; stop = true; break; }
            T end_x = x + ds;
            T mesh_end = (mu >= T(0)) ? __ldg(&a.right[cell]) : __ldg(&a.left[cell]);
            uint8_t m = __ldg(&a.mat[cell]);
            if ((mu < T(0) && mesh_end > end_x && cell == 0) ||
                (mu >= T(0) && end_x > mesh_end && cell == last)) {
                T piece = fabs((x - mesh_end) / mu);
                atomicAdd(&a.tally[(uint64_t)g * a.nc + cell], (double)piece);
                rec.track += (double)piece;
                rec.nsf_track += (double)(__ldg(&a.nsf[m + (uint64_t)M * g]) * piece);
                T bound = (mu >= T(0)) ? a.boundr : a.boundl;
                if (bound > T(0)) {
                    T nmu = mu * (-bound);
                    ds = (ds + (x - mesh_end)) * (-bound);
                    x = mesh_end; mu = nmu; rec.reflections++;
                } else { fate = NRAPS_FATE_LEAKED; stop = true; break; }
            } else if (fabs(end_x - x) > fabs(mesh_end - x)) {
                T piece = fabs((x - mesh_end) / mu);
                atomicAdd(&a.tally[(uint64_t)g * a.nc + cell], (double)piece);
                rec.track += (double)piece;
                rec.nsf_track += (double)(__ldg(&a.nsf[m + (uint64_t)M * g]) * piece);
                ds = ds + (x - mesh_end); x = mesh_end;
                cell = (mu >= T(0)) ? cell + 1 : cell - 1;
                rec.crossings++;
                if (m != __ldg(&a.mat[cell])) same = false;
            } else {
                T piece = fabs((x - end_x) / mu);
                atomicAdd(&a.tally[(uint64_t)g * a.nc + cell], (double)piece);
                rec.track += (double)piece;
                rec.nsf_track += (double)(__ldg(&a.nsf[m + (uint64_t)M * g]) * piece);
                rec.collisions++;
                T inv_sigs = T(1) / __ldg(&a.sigs[xs]);
                T cdf[NR_MAXG];
                T cum = T(0);
                const T* row = a.scat + (uint64_t)G * G * m + (uint64_t)G * g;
                for (uint32_t e = 0; e < G; ++e) { cum = cum + __ldg(&row[e]); cdf[e] = cum * inv_sigs; }
                T r_int = u01<T>(rng.next());
                T absorption = __ldg(&a.siga[xs]) / __ldg(&a.sigt[xs]);
                T nmu = T(2) * u01<T>(rng.next()) - T(1);
                uint32_t base = 0, size = G;
                while (size > 1) {
                    uint32_t half = size / 2, mid = base + half;
                    if (cdf[mid] < u01<T>(rng.next())) base = mid;
                    size -= half;
                }
                uint32_t ng = base + ((cdf[base] < u01<T>(rng.next())) ? 1u : 0u);
                if (ng > G - 1) ng = G - 1;
                if (r_int < absorption) { fate = NRAPS_FATE_ABSORBED; stop = true; break; }
                x = end_x; g = ng; mu = nmu;
                ds = mu * -lg(u01<T>(rng.next())) * __ldg(&a.inv_sigtr[xs]);
            }
        }
        if (stop) break;
    }
    c.coll += rec.collisions;
    c.cross += rec.crossings;
    if (fate == NRAPS_FATE_ABSORBED) c.absorbed++;
    else if (fate == NRAPS_FATE_LEAKED) c.leaked++;
    else c.capped++;
    if (out) {
        rec.fate = fate; rec.final_cell = (uint32_t)cell; rec.final_group = g;
        rec.final_x = (double)x; rec.draws = rng.draws;
        out[h] = rec;
    }
}

template <class T, bool BANK, bool REC>
__device__ void physics_history(const PlainArgs<T>& a, uint64_t h, uint64_t seed, T inv_k,
                                const nraps_site* src, uint64_t n_src,
                                Counters& c, nraps_history_record* out) {
    Rng rng{nr_pcg32_seeded(seed, h), 0};
    const uint64_t last = a.nc - 1;
    const uint32_t G = a.G, M = a.M;
    uint64_t cell; T x, mu; uint32_t g;
    if (n_src == 0) {
        cell = __ldg(&a.fuel[((uint64_t)rng.next() * a.nfuel) >> 32]);
        T sub = u01<T>(rng.next());
        mu = T(2) * u01<T>(rng.next()) - T(1);
        g = energy_pp<T>(a.chi_cdf + (uint64_t)__ldg(&a.mat[cell]) * G, G, u01<T>(rng.next()));
        x = __ldg(&a.left[cell]) + sub * __ldg(&a.dx[cell]);
    } else {
        uint64_t j = (h * n_src) / a.N;
        nraps_site s = src[j];
        cell = s.cell; x = (T)s.x; g = s.group;
        mu = T(2) * u01<T>(rng.next()) - T(1);
    }
    uint64_t events = 0;
    uint32_t seq = 0;
    nraps_history_record rec = {};
    int fate = NRAPS_FATE_ABSORBED;
    const T inf = tinf<T>();
    /* FP64 is ~1/64 of the FP32 rate on this part and the crossing loop is
       FP64-bound: a flight multiplies by 1/mu (set with mu) instead of
       dividing per crossing, and the history's k score is one fused
       multiply-add per track piece, fixed to 2^-32 once per history */
    T inv_mu = mu != T(0) ? T(1) / mu : inf;
    bool fwd = mu >= T(0), flat = mu == T(0);     /* set with mu */
    double ks = 0.0;
    for (;;) {
        rec.segments++;
        const uint8_t m = __ldg(&a.mat[cell]);      /* fixed within the segment */
        uint64_t xs = m + (uint64_t)M * g;
        double nsf = (double)__ldg(&a.nsf[xs]);
        T l = -lg(upos<T>(rng.next())) * __ldg(&a.inv_sigtr[xs]);
        bool stop = false, same = true;
        while (same) {
            if (++events > a.max_events) { fate = NRAPS_FATE_CAPPED; stop = true; break; }
            T face = fwd ? __ldg(&a.right[cell]) : __ldg(&a.left[cell]);
            T lf = flat ? inf : (face - x) * inv_mu;
            if (lf < l) {
                atomicAdd(&a.tally[(uint64_t)g * a.nc + cell], (double)lf);
                ks = __fma_rn(nsf, (double)lf, ks);
                if (REC) rec.track += (double)lf;
                l = l - lf; x = face;
                if (fwd ? (cell == last) : (cell == 0)) {
                    T bound = fwd ? a.boundr : a.boundl;
                    if (bound > T(0)) { mu = -mu; inv_mu = -inv_mu; fwd = !fwd; rec.reflections++; }
                    else { fate = NRAPS_FATE_LEAKED; stop = true; break; }
                } else {
                    cell = fwd ? cell + 1 : cell - 1;
                    rec.crossings++;
                    if (__ldg(&a.mat[cell]) != m) same = false;
                }
            } else {
                atomicAdd(&a.tally[(uint64_t)g * a.nc + cell], (double)l);
                ks = __fma_rn(nsf, (double)l, ks);
                if (REC) rec.track += (double)l;
                x = x + mu * l;
                rec.collisions++;
                if (BANK) {
                    T nu = __ldg(&a.nsf_sigtr[xs]) * inv_k + u01<T>(rng.next());
                    int n = (int)floor(nu);
                    if (n > 64) n = 64;
                    for (int i = 0; i < n; ++i) {
                        uint32_t sg = energy_pp<T>(a.chi_cdf + (uint64_t)m * G, G, u01<T>(rng.next()));
                        emit_site(a, x, cell, sg, h, seq);
                        ++seq;
                    }
                }
                if (u01<T>(rng.next()) < __ldg(&a.pabs[xs])) { fate = NRAPS_FATE_ABSORBED; stop = true; break; }
                T xi = u01<T>(rng.next());
                const T* cdf = a.phys_cdf + ((uint64_t)m * G + g) * G;
                uint32_t ng = G - 1;
                for (uint32_t e = 0; e + 1 < G; ++e) if (xi < __ldg(&cdf[e])) { ng = e; break; }
                g = ng;
                mu = T(2) * u01<T>(rng.next()) - T(1);
                inv_mu = mu != T(0) ? T(1) / mu : inf;
                fwd = mu >= T(0);
                flat = mu == T(0);
                xs = m + (uint64_t)M * g;
                nsf = (double)__ldg(&a.nsf[xs]);
                l = -lg(upos<T>(rng.next())) * __ldg(&a.inv_sigtr[xs]);
            }
        }
        if (stop) break;
    }
    c.kq += nr_fix(ks);
    if (REC) rec.nsf_track = ks;
    c.coll += rec.collisions;
    c.cross += rec.crossings;
    if (fate == NRAPS_FATE_ABSORBED) c.absorbed++;
    else if (fate == NRAPS_FATE_LEAKED) c.leaked++;
    else c.capped++;
    if (BANK) a.sink.count[h] = seq;
    if (REC) {
        rec.fate = fate; rec.final_cell = (uint32_t)cell; rec.final_group = g;
        rec.final_x = (double)x; rec.draws = rng.draws; rec.n_sites = seq;
        out[h] = rec;
    }
}

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

template <class T, int MODE, bool REC>
__global__ void __launch_bounds__(256) plain_kernel(PlainArgs<T> a) {
    const GenState* st = a.st;
    uint64_t gen = st->gen;
    uint64_t seed = nr_generation_seed(a.base_seed, gen);
    Counters c = {0, 0, 0, 0, 0, 0};
    uint64_t h = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (h < a.n_hist) {
        if (MODE == NRAPS_MODE_COMPAT) {
            compat_history<T>(a, h, seed, c, a.records);
        } else {
            T inv_k = (T)(1.0 / st->k);
            const nraps_site* src = nullptr;
            uint64_t n_src = 0;
            if (MODE == NRAPS_MODE_BANK && st->n_bank > 0) { src = a.bank[gen & 1]; n_src = st->n_bank; }
            physics_history<T, MODE == NRAPS_MODE_BANK, REC>(a, h, seed, inv_k, src, n_src, c, a.records);
        }
    }
    unsigned long long kq = warp_sum(c.kq);
    unsigned long long coll = warp_sum(c.coll), cross = warp_sum(c.cross);
    unsigned long long ab = warp_sum(c.absorbed), lk = warp_sum(c.leaked), cp = warp_sum(c.capped);
    if ((threadIdx.x & 31) == 0) {
        GenState* sw = a.st;
        if (kq) atomicAdd(&sw->kq, kq);
        if (coll) atomicAdd(&sw->collisions, coll);
        if (cross) atomicAdd(&sw->crossings, cross);
        if (ab) atomicAdd(&sw->absorbed, ab);
        if (lk) atomicAdd(&sw->leaked, lk);
        if (cp) { atomicAdd(&sw->capped, cp); atomicOr(&sw->error, NR_ERR_CAPPED); }
    }
}

__global__ void pcg_stream_kernel(uint64_t seed, const uint64_t* streams, uint64_t n, uint32_t per,
                                  uint32_t* out) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    nr_pcg32 r = nr_pcg32_seeded(seed, streams[i]);
    for (uint32_t j = 0; j < per; ++j) out[i * per + j] = nr_pcg32_next(&r);
}

__global__ void log_eval_kernel(const double* x, uint64_t n, double* o64, float* o32) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    o64[i] = nr_log(x[i]);
    o32[i] = nr_logf((float)x[i]);
}

}  // namespace

template <class T>
int launch_plain(const PlainArgs<T>& a, int mode, int block, cudaStream_t s) {
    if (block <= 0 || block > 256) block = 256;
    uint64_t grid = (a.n_hist + block - 1) / block;
    if (grid == 0) return 0;
    /* per-history records only in trace sessions (the record sums cost FP64
       adds on every crossing) */
    if (mode == NRAPS_MODE_COMPAT) plain_kernel<T, NRAPS_MODE_COMPAT, true><<<(unsigned)grid, block, 0, s>>>(a);
    else if (a.records) {
        if (mode == NRAPS_MODE_PHYSICS) plain_kernel<T, NRAPS_MODE_PHYSICS, true><<<(unsigned)grid, block, 0, s>>>(a);
        else plain_kernel<T, NRAPS_MODE_BANK, true><<<(unsigned)grid, block, 0, s>>>(a);
    } else {
        if (mode == NRAPS_MODE_PHYSICS) plain_kernel<T, NRAPS_MODE_PHYSICS, false><<<(unsigned)grid, block, 0, s>>>(a);
        else plain_kernel<T, NRAPS_MODE_BANK, false><<<(unsigned)grid, block, 0, s>>>(a);
    }
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}
template int launch_plain<float>(const PlainArgs<float>&, int, int, cudaStream_t);
template int launch_plain<double>(const PlainArgs<double>&, int, int, cudaStream_t);

int launch_pcg_stream(uint64_t seed, const uint64_t* streams, uint64_t n, uint32_t per,
                      uint32_t* out, cudaStream_t s) {
    if (n == 0) return 0;
    pcg_stream_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(seed, streams, n, per, out);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_log_eval(const double* x, uint64_t n, double* o64, float* o32, cudaStream_t s) {
    if (n == 0) return 0;
    log_eval_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(x, n, o64, o32);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}
