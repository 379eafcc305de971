/*
 * nraps_oracle.cpp — CPU restatement of NRAPS's Monte Carlo path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline / reference arm may load this library; the product
 * (nraps_gb300) never does.  It is what the CUDA path is checked against and
 * the timed stand-in for the reference CPU solver, which is Rust and cannot
 * be built without rustc/cargo and its crates.
 *
 * Pinned by: the reference's own unit tests (src/mc_code.rs:392-556, restated
 * in tests/test_oracle_golden.py) and the pcg-c-basic known-answer stream,
 * which the rand.rs seeding reproduces.  The reference draws its uniforms
 * from the rand 0.8.5 crate (ChaCha12 thread_rng, OS-entropy seeded), so no
 * reference run can pin monte_carlo itself: parity of whole generations is
 * against this restatement with the PCG32 streams of src/rand.rs.
 *
 * Restated items (reference file:line):
 *   Pcg32                 src/rand.rs:36-107 (explicit seed)
 *   partition_point       Rust core slice::binary_search_by, fixed-iteration
 *                         form (std since 2024), used by mc_code.rs:31,124-126
 *   energy                src/mc_code.rs:6-32
 *   direction             src/mc_code.rs:34-37
 *   spawn_neutron         src/mc_code.rs:40-53 (+ start_x, :230)
 *   hit_boundary          src/mc_code.rs:55-62
 *   cross_mesh            src/mc_code.rs:64-79
 *   scat_mat_calc         src/mc_code.rs:81-111
 *   interaction           src/mc_code.rs:113-132
 *   particle_travel       src/mc_code.rs:134-213
 *   particle_lifetime     src/mc_code.rs:215-257 (thread split :300-307)
 *   average_assembly      src/mc_code.rs:259-274
 *   monte_carlo           src/mc_code.rs:276-380
 * Build-defined algorithms with no reference counterpart (PHYSICS and BANK
 * modes: quirks fixed, explicit track length, collision-time fission bank
 * ordered by (parent, sequence), systematic source resampling, fixed-point k)
 * follow the same rules as the CUDA path, restated independently here.
 *
 * Compile with -ffp-contract=off: every expression below must round exactly
 * as written.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

#include "../include/nraps_gpu.h"
#include "../nraps_gb300/csrc/nr_math.h"   /* the shared logarithm only */

namespace orc {

/* ---- src/rand.rs:36-107 ---------------------------------------------------- */
struct Pcg32 {
    uint64_t state, inc, draws = 0;
    Pcg32(uint64_t seed, uint64_t stream) : state(0), inc((stream << 1) | 1) {
        next_u32();              /* "Move away from 0"                         */
        state = seed + inc;      /* rng.state = seed.wrapping_add(rng.inc)      */
        next_u32();
        draws = 0;
    }
    uint32_t next_u32() {
        uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        uint32_t xorshifted = (uint32_t)(((old >> 18) ^ old) >> 27);
        uint32_t rot = (uint32_t)(old >> 59);
        ++draws;
        return (xorshifted >> rot) | (xorshifted << ((32u - rot) & 31u));
    }
};

static uint64_t splitmix(uint64_t x) {
    uint64_t z = x + 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
static uint64_t gen_seed(uint64_t base, uint64_t gen) { return splitmix(base ^ splitmix(gen)); }

template <class T> T uni(Pcg32& r);
template <> float uni<float>(Pcg32& r) { return (float)r.next_u32() * 2.3283064E-10f; }
template <> double uni<double>(Pcg32& r) { return (double)r.next_u32() * 0x1p-32; }
template <class T> T upos(Pcg32& r);
template <> float upos<float>(Pcg32& r) { return (float)((r.next_u32() >> 8) + 1u) * 0x1p-24f; }
template <> double upos<double>(Pcg32& r) { return ((double)r.next_u32() + 1.0) * 0x1p-32; }
static float lg(float x) { return nr_logf(x); }
static double lg(double x) { return nr_log(x); }

/* Rust's partition_point: binary_search_by with pred -> Less / Greater, the
   fixed-iteration loop (no early exit) plus one final probe at `base`. */
template <class P> size_t partition_point(size_t n, P pred) {
    if (n == 0) return 0;
    size_t base = 0, size = n;
    while (size > 1) {
        size_t half = size / 2, mid = base + half;
        if (pred(mid)) base = mid;       /* cmp != Greater */
        size -= half;
    }
    return base + (pred(base) ? 1 : 0);
}

template <class T> T direction(T r) { return T(2) * r - T(1); }

template <class T> struct Tab {
    uint32_t M, G;
    uint64_t nc, nfuel;
    std::vector<T> sigt, sigs, siga, mu, inv_sigtr, nsf, nsf_sigtr, pabs, scat, chit;
    std::vector<T> chi_cdf;      /* [m*G + g] cumulative chi of material m   */
    std::vector<T> phys_cdf;     /* [(m*G + g)*G + g'] transport-corrected     */
    std::vector<T> left, right, dx;
    std::vector<uint8_t> mat;
    std::vector<uint64_t> fuel;
    T dx_fuel, boundl, boundr;
};

template <class T> static Tab<T> make_tab(const nraps_problem& p) {
    Tab<T> t;
    const nraps_variables& v = p.variables;
    t.M = v.mattypes; t.G = v.energygroups; t.nc = p.mesh.n_cells; t.nfuel = p.n_fuel;
    uint64_t nx = (uint64_t)t.M * t.G;
    auto cp = [&](const float* s, uint64_t n) { std::vector<T> o(n); for (uint64_t i = 0; i < n; ++i) o[i] = (T)s[i]; return o; };
    t.sigt = cp(p.xsdata.sigt, nx); t.sigs = cp(p.xsdata.sigs, nx); t.siga = cp(p.xsdata.siga, nx);
    t.mu = cp(p.xsdata.mu, nx); t.chit = cp(p.xsdata.chit, nx);
    t.scat = cp(p.xsdata.scat_matrix, nx * t.G);
    t.inv_sigtr.resize(nx); t.nsf.resize(nx); t.nsf_sigtr.resize(nx); t.pabs.resize(nx);
    for (uint64_t i = 0; i < nx; ++i) {
        /* compat reads the caller's inv_sigtr; FP64 recomputes it in FP64.  */
        if (sizeof(T) == 4) t.inv_sigtr[i] = (T)p.xsdata.inv_sigtr[i];
        else t.inv_sigtr[i] = T(1) / (t.sigt[i] - t.mu[i] * t.sigs[i]);
        t.nsf[i] = (T)p.xsdata.nut[i] * (T)p.xsdata.sigf[i];
        t.nsf_sigtr[i] = t.nsf[i] * t.inv_sigtr[i];
        t.pabs[i] = t.siga[i] * t.inv_sigtr[i];
    }
    t.chi_cdf.resize(nx);
    for (uint32_t m = 0; m < t.M; ++m) {
        T c = 0;
        for (uint32_t g = 0; g < t.G; ++g) { c += t.chit[m + t.M * g]; t.chi_cdf[m * t.G + g] = c; }
    }
    t.phys_cdf.resize(nx * t.G);
    for (uint32_t m = 0; m < t.M; ++m)
        for (uint32_t g = 0; g < t.G; ++g) {
            uint64_t xs = m + (uint64_t)t.M * g;
            T cum[64]; T c = 0;
            for (uint32_t e = 0; e < t.G; ++e) {
                T s = t.scat[(uint64_t)t.G * t.G * m + (uint64_t)t.G * g + e];
                if (e == g) s = s - t.mu[xs] * t.sigs[xs];
                if (s < T(0)) s = T(0);
                c = c + s; cum[e] = c;
            }
            for (uint32_t e = 0; e < t.G; ++e)
                t.phys_cdf[(m * t.G + g) * t.G + e] = (c > T(0)) ? cum[e] / c : T(1);
        }
    t.left.resize(t.nc); t.right.resize(t.nc); t.dx.resize(t.nc); t.mat.resize(t.nc);
    for (uint64_t c = 0; c < t.nc; ++c) {
        t.left[c] = (T)p.mesh.mesh_left[c]; t.right[c] = (T)p.mesh.mesh_right[c];
        t.dx[c] = (T)p.mesh.delta_x[c]; t.mat[c] = p.mesh.matid[c];
    }
    t.fuel.assign(p.fuel_indices, p.fuel_indices + p.n_fuel);
    t.dx_fuel = (T)p.delta_x.fuel; t.boundl = (T)v.boundl; t.boundr = (T)v.boundr;
    return t;
}

/* energy(): cumulative chi of the cell's material, partition_point(x < chi),
   clamped to G-1 (src/mc_code.rs:6-32). */
template <class T> static uint32_t energy(const Tab<T>& t, T chi, uint8_t m) {
    const T* cdf = &t.chi_cdf[(uint64_t)m * t.G];
    size_t i = partition_point(t.G, [&](size_t j) { return cdf[j] < chi; });
    return (uint32_t)std::min<size_t>(i, t.G - 1);
}

struct SiteU { float x; uint32_t cell, group; uint32_t parent, seq; };
template <class T> struct Site { T x; uint64_t cell; uint32_t group; };

template <class A> struct Sink {
    A* tally;                 /* G*nc                                       */
    uint64_t kq = 0;          /* fixed-point track-length k score           */
    std::vector<SiteU>* sites = nullptr;
};

/* One COMPAT history: particle_lifetime's body + particle_travel. */
template <class T, class A>
static void compat_history(const Tab<T>& t, Pcg32& rng, Sink<A>& sk,
                           nraps_history_record& rec, uint64_t max_events) {
    const uint64_t last = t.nc - 1;
    /* spawn_neutron: fields evaluated left to right (src/mc_code.rs:46-51)   */
    uint64_t cell = t.fuel[((uint64_t)rng.next_u32() * t.nfuel) >> 32];
    T sub = uni<T>(rng);
    T mu = direction(uni<T>(rng));
    uint32_t g = energy(t, uni<T>(rng), t.mat[cell]);
    T x = t.left[cell] + sub * t.dx_fuel;                    /* mc_code.rs:230 */
    uint64_t events = 0;
    auto score = [&](T piece) {
        sk.tally[(uint64_t)g * t.nc + cell] += (A)piece;
        rec.track += (double)piece;
        rec.nsf_track += (double)(t.nsf[t.mat[cell] + (uint64_t)t.M * g] * piece);
    };
    auto finish = [&](int fate) {
        rec.fate = fate; rec.final_cell = (uint32_t)cell; rec.final_group = g;
        rec.final_x = (double)x; rec.draws = rng.draws;
    };
    for (;;) {                                   /* while particle_exists     */
        rec.segments++;
        uint64_t xs = t.mat[cell] + (uint64_t)t.M * g;          /* :147       */
        T ds = mu * -lg(uni<T>(rng)) * t.inv_sigtr[xs];         /* :148       */
        for (;;) {                               /* while same_material       */
            if (++events > max_events) { finish(NRAPS_FATE_CAPPED); return; }
            T end_x = x + ds;
            T mesh_end = (mu >= T(0)) ? t.right[cell] : t.left[cell];
            if ((mu < T(0) && mesh_end > end_x && cell == 0) ||
                (mu >= T(0) && end_x > mesh_end && cell == last)) {
                score(std::fabs((x - mesh_end) / mu));          /* :163       */
                T bound = (mu >= T(0)) ? t.boundr : t.boundl;
                if (bound > T(0)) {                             /* hit_boundary */
                    T nmu = mu * (-bound);
                    ds = (ds + (x - mesh_end)) * (-bound);
                    x = mesh_end; mu = nmu; rec.reflections++;
                } else { finish(NRAPS_FATE_LEAKED); return; }
            } else if (std::fabs(end_x - x) > std::fabs(mesh_end - x)) {
                score(std::fabs((x - mesh_end) / mu));          /* :173       */
                uint8_t prev = t.mat[cell];
                ds = ds + (x - mesh_end); x = mesh_end;         /* cross_mesh */
                cell = (mu >= T(0)) ? cell + 1 : cell - 1;
                rec.crossings++;
                if (prev != t.mat[cell]) break;                 /* :179-181   */
            } else {
                score(std::fabs((x - end_x) / mu));             /* :184       */
                rec.collisions++;
                /* scat_mat_calc with 1/sigs[stale xs] (:186-192)            */
                T inv_sigs = T(1) / t.sigs[xs];
                T cdf[64]; T cum = 0;
                uint64_t base = (uint64_t)t.G * t.G * t.mat[cell] + (uint64_t)t.G * g;
                for (uint32_t e = 0; e < t.G; ++e) { cum += t.scat[base + e]; cdf[e] = cum * inv_sigs; }
                /* interaction(random, ...) (:195, :113-132)                  */
                T r_int = uni<T>(rng);
                T absorption = t.siga[xs] / t.sigt[xs];
                T nmu = T(2) * (uni<T>(rng)) - T(1);
                size_t pp = partition_point(t.G, [&](size_t j) { return cdf[j] < uni<T>(rng); });
                uint32_t ng = (uint32_t)std::min<size_t>(pp, t.G - 1);
                if (r_int < absorption) { finish(NRAPS_FATE_ABSORBED); return; }
                x = end_x; g = ng; mu = nmu;
                ds = mu * -lg(uni<T>(rng)) * t.inv_sigtr[xs];   /* :209 stale */
            }
        }
    }
}

/* One PHYSICS/BANK history (build-defined; quirks fixed). */
template <class T, class A>
static void physics_history(const Tab<T>& t, Pcg32& rng, Sink<A>& sk,
                            nraps_history_record& rec, uint64_t max_events,
                            bool bank, T inv_k, const Site<T>* src, uint32_t hid) {
    const uint64_t last = t.nc - 1;
    uint64_t cell; T x, mu; uint32_t g;
    if (!src) {
        cell = t.fuel[((uint64_t)rng.next_u32() * t.nfuel) >> 32];
        T sub = uni<T>(rng);
        mu = direction(uni<T>(rng));
        g = energy(t, uni<T>(rng), t.mat[cell]);
        x = t.left[cell] + sub * t.dx[cell];
    } else {
        cell = src->cell; x = src->x; g = src->group;
        mu = direction(uni<T>(rng));
    }
    uint64_t events = 0; uint32_t seq = 0;
    /* the history's k score: one fused multiply-add per track piece in FP64,
       fixed to 2^-32 once when the history ends */
    double ks = 0.0;
    auto score = [&](T piece) {
        sk.tally[(uint64_t)g * t.nc + cell] += (A)piece;
        rec.track += (double)piece;
        ks = std::fma((double)t.nsf[t.mat[cell] + (uint64_t)t.M * g], (double)piece, ks);
    };
    auto finish = [&](int fate) {
        rec.fate = fate; rec.final_cell = (uint32_t)cell; rec.final_group = g;
        rec.final_x = (double)x; rec.draws = rng.draws; rec.n_sites = seq;
        rec.nsf_track = ks;
        sk.kq += nr_fix(ks);
    };
    const T inf = std::numeric_limits<T>::infinity();
    /* distances to faces multiply by 1/mu, set whenever mu is */
    T inv_mu = mu != T(0) ? T(1) / mu : inf;
    for (;;) {
        rec.segments++;
        uint64_t xs = t.mat[cell] + (uint64_t)t.M * g;
        T l = -lg(upos<T>(rng)) * t.inv_sigtr[xs];
        for (;;) {
            if (++events > max_events) { finish(NRAPS_FATE_CAPPED); return; }
            T face = (mu >= T(0)) ? t.right[cell] : t.left[cell];
            T lf = (mu != T(0)) ? (face - x) * inv_mu : inf;
            if (lf < l) {
                score(lf);
                l = l - lf; x = face;
                if ((mu < T(0)) ? (cell == 0) : (cell == last)) {
                    T bound = (mu >= T(0)) ? t.boundr : t.boundl;
                    if (bound > T(0)) { mu = -mu; inv_mu = -inv_mu; rec.reflections++; }
                    else { finish(NRAPS_FATE_LEAKED); return; }
                } else {
                    uint8_t prev = t.mat[cell];
                    cell = (mu >= T(0)) ? cell + 1 : cell - 1;
                    rec.crossings++;
                    if (t.mat[cell] != prev) break;
                }
            } else {
                score(l);
                x = x + mu * l;
                rec.collisions++;
                uint8_t m = t.mat[cell];
                if (bank) {
                    T nu = t.nsf_sigtr[xs] * inv_k + uni<T>(rng);
                    int n = (int)std::floor(nu);
                    if (n > 64) n = 64;
                    for (int i = 0; i < n; ++i) {
                        uint32_t sg = energy(t, uni<T>(rng), m);
                        if (sk.sites) sk.sites->push_back(SiteU{(float)x, (uint32_t)cell, sg, hid, seq});
                        ++seq;
                    }
                }
                if (uni<T>(rng) < t.pabs[xs]) { finish(NRAPS_FATE_ABSORBED); return; }
                T xi = uni<T>(rng);
                const T* cdf = &t.phys_cdf[((uint64_t)m * t.G + g) * t.G];
                uint32_t ng = t.G - 1;
                for (uint32_t e = 0; e + 1 < t.G; ++e) if (xi < cdf[e]) { ng = e; break; }
                g = ng;
                mu = direction(uni<T>(rng));
                inv_mu = mu != T(0) ? T(1) / mu : inf;
                xs = m + (uint64_t)t.M * g;
                l = -lg(upos<T>(rng)) * t.inv_sigtr[xs];
            }
        }
    }
}

struct GenOut {
    std::vector<nraps_history_record> rec;
    uint64_t kq = 0;
    std::vector<SiteU> sites;
};

/* One generation, histories in id order.  accumulate into tally (A). */
template <class T, class A>
static void run_generation(const Tab<T>& t, const nraps_opts& o, uint64_t gen, double k,
                           const std::vector<Site<T>>* src, uint64_t n_hist,
                           uint64_t first, uint64_t last_excl, A* tally, GenOut& out,
                           bool keep_records) {
    uint64_t seed = gen_seed(o.seed, gen);
    uint64_t maxev = o.max_events ? o.max_events : (1ULL << 24);
    bool bank = o.mode == NRAPS_MODE_BANK;
    T inv_k = (T)(1.0 / k);
    Sink<A> sk; sk.tally = tally; sk.sites = bank ? &out.sites : nullptr;
    for (uint64_t h = first; h < last_excl; ++h) {
        Pcg32 rng(seed, h);
        nraps_history_record r; std::memset(&r, 0, sizeof r);
        if (o.mode == NRAPS_MODE_COMPAT) compat_history<T, A>(t, rng, sk, r, maxev);
        else {
            const Site<T>* s = nullptr;
            Site<T> tmp;
            if (src && !src->empty()) {
                uint64_t j = (uint64_t)((unsigned __int128)h * src->size() / n_hist);
                tmp = (*src)[j]; s = &tmp;
            }
            physics_history<T, A>(t, rng, sk, r, maxev, bank, inv_k, s, (uint32_t)h);
        }
        if (keep_records) out.rec[h - first] = r;
    }
    out.kq += sk.kq;
}


/* ---- event-based Woodcock form (build-defined; no reference counterpart) --
   Restates the FP32 delta-tracking history of the CUDA event kernel with the
   shared software logarithm (the kernel's exact_log mode): tables, region
   lookup, draw order and every rounding step are defined here independently
   of the kernel source, from the same rules.                                */
struct WTab {
    uint32_t M, G, R, nc, nfuel;
    float L, boundl, boundr;
    std::vector<float> sigtr, pabs, nsf_st, inv_st, scdf, ocdf, chicdf, maj, inv_maj;
    std::vector<float> rleft, rinvdx, cleft, cdx;
    std::vector<uint8_t> rmat, cmat;
    std::vector<uint32_t> rfirst, rncell, fuel;
};

static WTab make_wtab(const nraps_problem& p) {
    WTab t;
    const nraps_xsdata& x = p.xsdata;
    t.M = p.variables.mattypes; t.G = p.variables.energygroups; t.nc = (uint32_t)p.mesh.n_cells;
    t.nfuel = (uint32_t)p.n_fuel; t.boundl = p.variables.boundl; t.boundr = p.variables.boundr;
    uint32_t M = t.M, G = t.G;
    t.sigtr.resize(M * G); t.pabs.resize(M * G); t.nsf_st.resize(M * G); t.inv_st.resize(M * G);
    for (uint32_t m = 0; m < M; ++m)
        for (uint32_t g = 0; g < G; ++g) {
            uint32_t i = m + M * g, j = m * G + g;
            float st = (float)((double)x.sigt[i] - (double)x.mu[i] * (double)x.sigs[i]);
            t.sigtr[j] = st;
            t.pabs[j] = x.siga[i] / st;
            t.nsf_st[j] = (x.nut[i] * x.sigf[i]) / st;
            t.inv_st[j] = 1.0f / st;
        }
    t.scdf.assign(M * G * G, 1.0f);
    for (uint32_t m = 0; m < M; ++m)
        for (uint32_t g = 0; g < G; ++g) {
            uint32_t i = m + M * g;
            float cum[64]; float c = 0.0f;
            for (uint32_t e = 0; e < G; ++e) {
                float s = x.scat_matrix[(uint64_t)G * G * m + (uint64_t)G * g + e];
                if (e == g) s = s - x.mu[i] * x.sigs[i];
                if (s < 0.0f) s = 0.0f;
                c = c + s; cum[e] = c;
            }
            for (uint32_t e = 0; e < G; ++e) t.scdf[(m * G + g) * G + e] = c > 0.0f ? cum[e] / c : 1.0f;
        }
    /* outcome CDF of a real collision: absorbed below pabs, else scattered
       into the group whose share of the remaining 1 - pabs the uniform hits */
    t.ocdf.assign(M * G * G, 1.0f);
    for (uint32_t j = 0; j < M * G; ++j) {
        const float q = 1.0f - t.pabs[j];
        t.ocdf[j * G] = t.pabs[j];
        for (uint32_t e = 1; e < G; ++e) t.ocdf[j * G + e] = t.pabs[j] + q * t.scdf[j * G + e - 1];
    }
    t.chicdf.resize(M * G);
    for (uint32_t m = 0; m < M; ++m) {
        float c = 0.0f;
        for (uint32_t g = 0; g < G; ++g) { c += x.chit[m + M * g]; t.chicdf[m * G + g] = c; }
    }
    std::vector<bool> present(M, false);
    for (uint32_t c = 0; c < t.nc; ++c) {
        uint8_t m = p.mesh.matid[c];
        present[m] = true;
        bool start = c == 0 || m != p.mesh.matid[c - 1] ||
                     std::memcmp(&p.mesh.delta_x[c], &p.mesh.delta_x[c - 1], 4) != 0;
        if (start) {
            t.rleft.push_back(p.mesh.mesh_left[c]); t.rmat.push_back(m); t.rfirst.push_back(c);
            t.rncell.push_back(1); t.rinvdx.push_back((float)(1.0 / (double)p.mesh.delta_x[c]));
        } else {
            t.rncell.back()++;
        }
    }
    t.R = (uint32_t)t.rmat.size();
    t.rleft.push_back(p.mesh.mesh_right[t.nc - 1]);
    t.L = t.rleft[t.R];
    t.maj.assign(G, 0.0f); t.inv_maj.assign(G, 0.0f);
    for (uint32_t g = 0; g < G; ++g) {
        float mj = 0.0f;
        for (uint32_t m = 0; m < M; ++m) if (present[m]) mj = std::max(mj, t.sigtr[m * G + g]);
        t.maj[g] = mj; t.inv_maj[g] = 1.0f / mj;
    }
    t.cleft.assign(p.mesh.mesh_left, p.mesh.mesh_left + t.nc);
    t.cdx.assign(p.mesh.delta_x, p.mesh.delta_x + t.nc);
    t.cmat.assign(p.mesh.matid, p.mesh.matid + t.nc);
    for (uint64_t i = 0; i < p.n_fuel; ++i) t.fuel.push_back((uint32_t)p.fuel_indices[i]);
    return t;
}

static float w_u24(Pcg32& r) { return (float)(r.next_u32() >> 8) * 0x1p-24f; }
static float w_u24pos(Pcg32& r) { return (float)((r.next_u32() >> 8) + 1u) * 0x1p-24f; }
static uint32_t w_chi(const float* cdf, uint32_t G, float v) {
    size_t i = partition_point(G, [&](size_t j) { return cdf[j] < v; });
    return (uint32_t)std::min<size_t>(i, G - 1);
}
/* region r with rleft[r] <= x < rleft[r+1] (the last region for x == L) */
static uint32_t w_region(const WTab& t, float x) {
    size_t r = std::upper_bound(t.rleft.begin(), t.rleft.begin() + t.R, x) - t.rleft.begin();
    return r == 0 ? 0 : (uint32_t)(r - 1);
}

static void woodcock_history(const WTab& t, Pcg32& rng, double* tally, uint64_t& kq,
                             nraps_history_record& rec, uint64_t max_events, bool bank, float inv_k,
                             const nraps_site* src, uint32_t hid, std::vector<SiteU>* sites) {
    const uint32_t G = t.G;
    float x, mu; uint32_t g;
    if (!src) {
        uint32_t cell = t.fuel[((uint64_t)rng.next_u32() * t.nfuel) >> 32];
        float sub = w_u24(rng);
        x = t.cleft[cell] + sub * t.cdx[cell];
        mu = 2.0f * w_u24(rng) - 1.0f;
        g = w_chi(&t.chicdf[t.cmat[cell] * G], G, w_u24(rng));
    } else {
        /* a fission neutron draws its group at birth from chi of the material
           of the cell it was born in (the site carries no group) */
        x = src->x;
        mu = 2.0f * w_u24(rng) - 1.0f;
        const uint32_t c = src->cell < t.nc ? src->cell : t.nc - 1;
        g = w_chi(&t.chicdf[t.cmat[c] * G], G, w_u24(rng));
    }
    uint64_t events = 0;
    uint32_t seq = 0, last_cell = 0;
    int fate = -1;
    while (fate < 0) {
        uint32_t r = 0, m = 0;
        for (;;) {
            if (++events > max_events) { fate = NRAPS_FATE_CAPPED; break; }
            float d = -nr_logf(w_u24pos(rng)) * t.inv_maj[g];
            x = x + mu * d;
            int bounce = 0;
            while (!(x >= 0.0f && x <= t.L)) {
                if (x > t.L) {
                    if (t.boundr > 0.0f) { x = t.L - (x - t.L); mu = -mu; }
                    else { fate = NRAPS_FATE_LEAKED; break; }
                } else {
                    if (t.boundl > 0.0f) { x = -x; mu = -mu; }
                    else { fate = NRAPS_FATE_LEAKED; break; }
                }
                if (++bounce > 1000) { fate = NRAPS_FATE_CAPPED; break; }
            }
            if (fate >= 0) break;
            r = w_region(t, x);
            m = t.rmat[r];
            if (w_u24(rng) * t.maj[g] < t.sigtr[m * G + g]) break;
            rec.crossings++;
        }
        if (fate >= 0) break;
        uint32_t j = m * G + g;
        float rel = (x - t.rleft[r]) * t.rinvdx[r];
        uint32_t k = rel > 0.0f ? (uint32_t)rel : 0u;
        if (k >= t.rncell[r]) k = t.rncell[r] - 1;
        uint32_t cell = t.rfirst[r] + k;
        last_cell = cell;
        tally[(uint64_t)g * t.nc + cell] += (double)t.inv_st[j];
        kq += nr_fix((double)t.nsf_st[j]);
        rec.collisions++;
        rec.track += (double)t.inv_st[j];
        rec.nsf_track += (double)t.nsf_st[j];
        if (bank) {
            float nu = t.nsf_st[j] * inv_k + w_u24(rng);
            int n = (int)std::floor(nu);
            if (n > 64) n = 64;
            for (int i = 0; i < n; ++i) {
                if (sites) sites->push_back(SiteU{x, cell, 0u, hid, seq});
                ++seq;
            }
        }
        /* one uniform: absorbed if below ocdf[0], else the scatter group is
           the number of outcome-CDF entries at or below it, minus one */
        const float u = w_u24(rng);
        uint32_t o = 0;
        for (uint32_t e = 0; e < G; ++e) o += (t.ocdf[j * G + e] <= u) ? 1u : 0u;
        if (o == 0) { fate = NRAPS_FATE_ABSORBED; break; }
        g = o - 1;
        mu = 2.0f * w_u24(rng) - 1.0f;
    }
    rec.fate = fate; rec.final_group = g; rec.final_x = (double)x; rec.final_cell = last_cell;
    rec.n_sites = seq; rec.draws = rng.draws;
}

} // namespace orc

using namespace orc;

extern "C" {

/* ---- unit pieces, for the restated reference unit tests ----------------- */
void oracle_hit_boundary(float mu, float start_x, float delta_s, float bound, float mesh_end, float* out3) {
    out3[0] = mu * (-bound);
    out3[1] = (delta_s + (start_x - mesh_end)) * (-bound);
    out3[2] = mesh_end;
}
void oracle_cross_mesh(uint64_t mesh_index, float mu, float start_x, float mesh_end, float delta_s,
                       float* out2, uint64_t* out_index) {
    *out_index = (mu >= 0.0f) ? mesh_index + 1 : mesh_index - 1;
    out2[0] = delta_s + (start_x - mesh_end);
    out2[1] = mesh_end;
}
float oracle_direction(float r) { return direction(r); }
void oracle_scat_mat_calc(uint32_t G, uint32_t matid, uint32_t g, float inv_sigs,
                          const float* scat_matrix, float* out) {
    /* the reference does this index arithmetic in u8 (mc_code.rs:89-90) */
    uint64_t base = (uint64_t)G * G * matid + (uint64_t)G * g;
    float cum = 0.0f;
    for (uint32_t e = 0; e < G; ++e) { cum += scat_matrix[base + e]; out[e] = cum * inv_sigs; }
}
/* energy() on an explicit cumulative list */
uint32_t oracle_energy_cdf(const float* cdf, uint32_t n, float chi) {
    size_t i = partition_point(n, [&](size_t j) { return cdf[j] < chi; });
    return (uint32_t)std::min<size_t>(i, n - 1);
}
/* partition_point with one fresh uniform per probe, from a PCG32 stream;
   returns the index and the number of draws consumed. */
uint32_t oracle_partition_fresh(const float* cdf, uint32_t n, uint64_t seed, uint64_t stream,
                                uint32_t* draws) {
    Pcg32 r(seed, stream);
    size_t i = partition_point(n, [&](size_t j) { return cdf[j] < uni<float>(r); });
    *draws = (uint32_t)r.draws;
    return (uint32_t)std::min<size_t>(i, n - 1);
}
void oracle_pcg32(uint64_t seed, uint64_t stream, uint32_t n, uint32_t* out) {
    Pcg32 r(seed, stream);
    for (uint32_t i = 0; i < n; ++i) out[i] = r.next_u32();
}
uint64_t oracle_generation_seed(uint64_t base, uint64_t gen) { return gen_seed(base, gen); }
double oracle_log(double x) { return nr_log(x); }
float oracle_logf(float x) { return nr_logf(x); }

/* ---- one generation with records (parity with nraps_trace_generation) --- */
int oracle_trace_generation(const nraps_problem* p, const nraps_opts* o, uint64_t gen, double k,
                            const nraps_site* sites_in, uint64_t n_in,
                            nraps_history_record* records, uint64_t n_records,
                            double* tally, nraps_site* sites_out, uint64_t cap_out,
                            uint64_t* n_out, uint64_t* kq_out) {
    uint64_t N = p->variables.histories;
    uint64_t n_hist = N + (o->mode == NRAPS_MODE_COMPAT ? o->compat_threads : 0);
    if (n_records != n_hist) return NRAPS_ERR_INVALID;
    uint64_t nbins = (uint64_t)p->variables.energygroups * p->mesh.n_cells;
    std::vector<double> tl(nbins, 0.0);
    GenOut out; out.rec.resize(n_hist);
    auto go = [&](auto tag) {
        using T = decltype(tag);
        Tab<T> t = make_tab<T>(*p);
        std::vector<Site<T>> src;
        if (sites_in && n_in) {
            src.resize(n_in);
            for (uint64_t i = 0; i < n_in; ++i) src[i] = Site<T>{(T)sites_in[i].x, sites_in[i].cell, sites_in[i].group};
        }
        run_generation<T, double>(t, *o, gen, k, src.empty() ? nullptr : &src, N, 0, n_hist,
                                  tl.data(), out, true);
    };
    if (o->precision == NRAPS_PREC_FP32) go(float{}); else go(double{});
    std::memcpy(records, out.rec.data(), n_hist * sizeof(nraps_history_record));
    if (tally) std::memcpy(tally, tl.data(), nbins * sizeof(double));
    if (kq_out) *kq_out = out.kq;
    if (n_out) *n_out = out.sites.size();
    if (sites_out) {
        /* sites are already in (parent, seq) order: histories ran in id order */
        uint64_t n = std::min<uint64_t>(cap_out, out.sites.size());
        for (uint64_t i = 0; i < n; ++i)
            sites_out[i] = nraps_site{out.sites[i].x, out.sites[i].cell, out.sites[i].group, 0};
        if (out.sites.size() > cap_out) return NRAPS_ERR_CAPACITY;
    }
    return NRAPS_OK;
}

/* ---- the whole monte_carlo (src/mc_code.rs:276-380) --------------------
   threads: the reference's T (available_parallelism - 1); the histories are
   split exactly as mc_code.rs:302-307 and run on T std::threads, each with a
   private tally of type A, summed serially after join (mc_code.rs:331-338).
   acc64 = 0 reproduces the reference's f32 tallies; 1 accumulates in double.
   max_generations < generations runs a prefix (timing samples). */
} /* extern "C" */
template <class T, class A>
static int mc_impl(const nraps_problem* p, const nraps_opts* o, uint32_t threads,
                   uint64_t max_generations, nraps_result* res) {
    const nraps_variables& v = p->variables;
    if (threads == 0) threads = 1;
    Tab<T> t = make_tab<T>(*p);
    uint64_t N = v.histories, nc = t.nc, G = t.G;
    uint64_t gens = std::min<uint64_t>(v.generations, max_generations ? max_generations : v.generations);
    bool compat = o->mode == NRAPS_MODE_COMPAT;
    bool bank = o->mode == NRAPS_MODE_BANK;
    std::vector<float> flux(G * nc, 0.0f), fs(nc, 0.0f), kres(v.generations, 0.0f), kf(v.generations, 0.0f);
    std::vector<double> k64(v.generations, 0.0), ent(v.generations, 0.0);
    std::vector<Site<T>> src;
    float k_new = p->k_new;
    double k64_prev = p->k_new;
    nraps_stats st; std::memset(&st, 0, sizeof st);
    for (uint64_t x = 0; x < gens; ++x) {
        float k = k_new; k_new = 0.0f;
        std::vector<A> tally(G * nc, A(0));
        /* thread split, mc_code.rs:302-307: [start, end] inclusive (Q3)    */
        uint64_t h = N / threads;
        std::vector<uint64_t> first(threads), count(threads);
        uint64_t ordinal = 0;
        for (uint32_t th = 0; th < threads; ++th) {
            uint64_t s = th * h, e = (th + 1 < threads) ? (th + 1) * h : N;
            uint64_t n = compat ? (e - s + 1) : (e - s);
            first[th] = ordinal; count[th] = n; ordinal += n;
        }
        if (!compat) { /* PHYSICS/BANK: exactly N histories, same split    */
            ordinal = 0;
            for (uint32_t th = 0; th < threads; ++th) { first[th] = ordinal; ordinal += count[th]; }
        }
        std::vector<std::vector<A>> tl(threads, std::vector<A>(G * nc, A(0)));
        std::vector<GenOut> outs(threads);
        std::vector<std::thread> pool;
        for (uint32_t th = 0; th < threads; ++th)
            pool.emplace_back([&, th] {
                run_generation<T, A>(t, *o, x, k64_prev, bank && !src.empty() ? &src : nullptr, N,
                                     first[th], first[th] + count[th], tl[th].data(), outs[th], false);
            });
        for (auto& th : pool) th.join();
        for (uint32_t th = 0; th < threads; ++th)
            for (uint64_t i = 0; i < G * nc; ++i) tally[i] += tl[th][i];
        st.histories += ordinal;
        double k_gen64;
        if (compat) {
            /* mc_code.rs:340-363, f32 as written */
            float fund = 1.0f / (float)(uint64_t)(v.generations - (v.skip - 1));
            for (uint64_t e = 0; e < G; ++e)
                for (uint64_t c = 0; c < nc; ++c) {
                    float dx = p->mesh.delta_x[c];
                    uint64_t xs = p->mesh.matid[c] + (uint64_t)v.mattypes * e;
                    float flx = (float)tally[e * nc + c] / (k * (float)N * dx);
                    float fsrc = p->xsdata.nut[xs] * p->xsdata.sigf[xs] * flx;
                    k_new += k * dx * fsrc;
                    if (x >= v.skip) {
                        float conversion = (3565e6f * k * 36.2f) /
                            (200e6f * 1.602176634e-19f * p->xsdata.nut[0 + v.mattypes * 1] * p->mesh.mesh_right[nc - 1]);
                        flux[e * nc + c] += flx * conversion * fund;
                        fs[c] += fsrc * fund;
                    }
                }
            kres[x] = k_new;
            k_gen64 = k_new;
        } else {
            uint64_t kq = 0; for (auto& go : outs) kq += go.kq;
            k_gen64 = nr_unfix(kq) / (double)N;
            double fund = 1.0 / (double)(v.generations - v.skip);
            double kk = k64_prev;
            for (uint64_t e = 0; e < G; ++e)
                for (uint64_t c = 0; c < nc; ++c) {
                    double dx = p->mesh.delta_x[c];
                    uint64_t xs = p->mesh.matid[c] + (uint64_t)v.mattypes * e;
                    double flx = (double)tally[e * nc + c] / (kk * (double)N * dx);
                    double fsrc = (double)p->xsdata.nut[xs] * (double)p->xsdata.sigf[xs] * flx;
                    if (x >= v.skip) {
                        double conversion = (3565e6 * kk * 36.2) /
                            (200e6 * 1.602176634e-19 * (double)p->xsdata.nut[0 + v.mattypes * 1] * (double)p->mesh.mesh_right[nc - 1]);
                        flux[e * nc + c] += (float)(flx * conversion * fund);
                        fs[c] += (float)(fsrc * fund);
                    }
                }
            kres[x] = (float)k_gen64;
            k_new = (float)k_gen64;
        }
        k64[x] = k_gen64;
        if (bank) {
            /* ordered bank = concatenation over threads (ids ascend)         */
            std::vector<Site<T>> nb;
            for (auto& go : outs) for (auto& s : go.sites) nb.push_back(Site<T>{(T)s.x, s.cell, s.group});
            if (nb.empty()) return NRAPS_ERR_EMPTY_BANK;
            std::vector<uint64_t> cnt(nc, 0);
            for (auto& s : nb) cnt[s.cell]++;
            double H = 0.0;
            for (uint64_t c = 0; c < nc; ++c) if (cnt[c]) { double pp = (double)cnt[c] / nb.size(); H -= pp * std::log2(pp); }
            ent[x] = H;
            st.sites += nb.size();
            src.swap(nb);
        }
        k64_prev = k_gen64;
    }
    /* average_assembly (mc_code.rs:259-274), f32 */
    std::vector<float> avg(G * nc, 0.0f);
    uint64_t na = v.numass ? v.numass : 1, ma = nc / na;
    for (uint64_t e = 0; e < G; ++e)
        for (uint64_t a = 1; a <= na; ++a) {
            float s = 0.0f;
            for (uint64_t i = (a - 1) * ma; i < a * ma; ++i) s += flux[e * nc + i];
            float av = s / (float)ma;
            for (uint64_t i = (a - 1) * ma; i < a * ma; ++i) avg[e * nc + i] = av;
        }
    /* k_fund (mc_code.rs:368-376) */
    if (v.skip < gens) {
        kf[v.skip] = kres[v.skip];
        for (uint64_t g2 = v.skip + 1; g2 < gens; ++g2) {
            float s = 0.0f;
            for (uint64_t i = v.skip; i <= g2; ++i) s += kres[i];
            kf[g2] = s / (float)(uint64_t)(g2 - (v.skip - 1));
        }
    }
    if (res->flux) std::memcpy(res->flux, flux.data(), flux.size() * 4);
    if (res->assembly_average) std::memcpy(res->assembly_average, avg.data(), avg.size() * 4);
    if (res->fission_source) std::memcpy(res->fission_source, fs.data(), fs.size() * 4);
    if (res->k) std::memcpy(res->k, kres.data(), kres.size() * 4);
    if (res->k_fund) std::memcpy(res->k_fund, kf.data(), kf.size() * 4);
    if (res->k64) std::memcpy(res->k64, k64.data(), k64.size() * 8);
    if (res->entropy) std::memcpy(res->entropy, ent.data(), ent.size() * 8);
    if (v.skip < gens) {
        double s = 0, s2 = 0; uint64_t n = gens - v.skip;
        for (uint64_t i = v.skip; i < gens; ++i) { s += k64[i]; s2 += k64[i] * k64[i]; }
        st.k_mean = s / n;
        st.k_sigma = n > 1 ? std::sqrt(std::max(0.0, (s2 / n - st.k_mean * st.k_mean)) / (n - 1)) : 0.0;
    }
    if (res->stats) *res->stats = st;
    return NRAPS_OK;
}

extern "C" {
int oracle_monte_carlo(const nraps_problem* p, const nraps_opts* o, uint32_t threads,
                       int acc64, uint64_t max_generations, nraps_result* res) {
    if (!p || !o || !res) return NRAPS_ERR_INVALID;
    if (p->variables.skip >= p->variables.generations) return NRAPS_ERR_INVALID;
    if (o->precision == NRAPS_PREC_FP32)
        return acc64 ? mc_impl<float, double>(p, o, threads, max_generations, res)
                     : mc_impl<float, float>(p, o, threads, max_generations, res);
    return mc_impl<double, double>(p, o, threads, max_generations, res);
}

/* One event-form generation, histories in id order (exact_log semantics). */
int oracle_trace_woodcock(const nraps_problem* p, const nraps_opts* o, uint64_t gen, double k,
                          const nraps_site* sites_in, uint64_t n_in,
                          nraps_history_record* records, uint64_t n_records, double* tally,
                          nraps_site* sites_out, uint64_t cap_out, uint64_t* n_out, uint64_t* kq_out) {
    uint64_t N = p->variables.histories;
    if (n_records != N) return NRAPS_ERR_INVALID;
    WTab t = make_wtab(*p);
    uint64_t seed = gen_seed(o->seed, gen);
    uint64_t maxev = o->max_events ? o->max_events : (1ULL << 24);
    bool bank = o->mode == NRAPS_MODE_BANK;
    float inv_k = (float)(1.0 / k);
    std::vector<double> tl((uint64_t)t.G * t.nc, 0.0);
    std::vector<SiteU> sites;
    uint64_t kq = 0;
    for (uint64_t h = 0; h < N; ++h) {
        Pcg32 rng(seed, h);
        nraps_history_record r; std::memset(&r, 0, sizeof r);
        const nraps_site* src = nullptr;
        if (bank && sites_in && n_in) src = &sites_in[(h * n_in) / N];
        woodcock_history(t, rng, tl.data(), kq, r, maxev, bank, inv_k, src, (uint32_t)h, bank ? &sites : nullptr);
        records[h] = r;
    }
    if (tally) std::memcpy(tally, tl.data(), tl.size() * 8);
    if (kq_out) *kq_out = kq;
    if (n_out) *n_out = sites.size();
    if (sites_out) {
        uint64_t n = std::min<uint64_t>(cap_out, sites.size());
        for (uint64_t i = 0; i < n; ++i) sites_out[i] = nraps_site{sites[i].x, sites[i].cell, sites[i].group, 0};
        if (sites.size() > cap_out) return NRAPS_ERR_CAPACITY;
    }
    return NRAPS_OK;
}

unsigned oracle_hardware_threads(void) { return std::thread::hardware_concurrency(); }

} /* extern "C" */
