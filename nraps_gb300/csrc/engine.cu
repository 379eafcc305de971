/*
 * engine.cu — contexts, device-resident sessions and the C ABI of
 * include/nraps_gpu.h.
 *
 * nraps_monte_carlo replaces NRAPS's monte_carlo (src/mc_code.rs:276-380):
 * it uploads the borrowed problem once, runs `generations` generations
 * back to back on the context's stream with no host round trip per
 * generation (k, the generation index and the bank size live in device
 * memory), then copies the SolutionResults out.  average_assembly
 * (src/mc_code.rs:259-274) and k_fund (:368-376) are computed on the host from
 * the FP64 per-generation results, as the reference computes them after the
 * generation loop.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "engine.cuh"
#include "event.cuh"
#include "host_common.hpp"
#include "tables.hpp"
#include "engine_internal.hpp"

/* ---- thread-local error text for calls without a context ---------------- */
namespace nraps_host {
static thread_local std::string g_err;
void set_error(const std::string& msg) { g_err = msg; }
const char* last_error() { return g_err.c_str(); }
void set_ctx_error(nraps_ctx* ctx, const std::string& msg) {
    if (ctx) ctx->err = msg; else g_err = msg;
}
}  // namespace nraps_host

using nrint::DevMem;
using nrint::set_err;

#define CK(call)                                                                        \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess)                                                          \
            return set_err(ctx, nrint::cuda_status(e_), std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

namespace nrint {

int validate_problem(nraps_ctx* ctx, const nraps_problem* p, const nraps_opts& o) {
    if (!p) return set_err(ctx, NRAPS_ERR_INVALID, "problem is NULL");
    const nraps_variables& v = p->variables;
    if (o.abi_version != NRAPS_ABI_VERSION) return set_err(ctx, NRAPS_ERR_INVALID, "opts.abi_version mismatch");
    if (o.mode < 0 || o.mode > 2) return set_err(ctx, NRAPS_ERR_INVALID, "opts.mode must be COMPAT, PHYSICS or BANK");
    if (o.precision < 0 || o.precision > 1) return set_err(ctx, NRAPS_ERR_INVALID, "opts.precision must be FP64 or FP32");
    if (o.tracking < 0 || o.tracking > 1) return set_err(ctx, NRAPS_ERR_INVALID, "opts.tracking must be SURFACE or WOODCOCK");
    if (o.tracking == NRAPS_TRACK_WOODCOCK && (o.mode == NRAPS_MODE_COMPAT || o.precision != NRAPS_PREC_FP32))
        return set_err(ctx, NRAPS_ERR_INVALID, "WOODCOCK tracking runs PHYSICS or BANK mode in FP32");
    if (o.entropy_bins != 0) return set_err(ctx, NRAPS_ERR_INVALID, "entropy_bins must be 0 (one bin per cell)");
    if (o.initial_source > 1) return set_err(ctx, NRAPS_ERR_INVALID, "initial_source must be 0 (uniform fuel) or 1 (diffusion)");
    if (o.initial_source && o.mode != NRAPS_MODE_BANK)
        return set_err(ctx, NRAPS_ERR_INVALID, "initial_source = 1 needs BANK mode (a fission bank to start from)");
    if (v.histories == 0) return set_err(ctx, NRAPS_ERR_INVALID, "Histories is 0");
    if (v.histories + o.compat_threads >= (1ULL << 32)) return set_err(ctx, NRAPS_ERR_INVALID, "at most 2^32-1 histories per generation");
    if (v.generations == 0) return set_err(ctx, NRAPS_ERR_INVALID, "Generations is 0");
    if (v.skip >= v.generations)
        return set_err(ctx, NRAPS_ERR_INVALID, "Skip must be smaller than Generations (the reference indexes k_fund[skip])");
    if (!p->mesh.matid || !p->mesh.mesh_left || !p->mesh.mesh_right || !p->mesh.delta_x)
        return set_err(ctx, NRAPS_ERR_INVALID, "mesh arrays are NULL");
    if (!p->xsdata.sigt || !p->xsdata.sigs || !p->xsdata.mu || !p->xsdata.siga || !p->xsdata.sigf ||
        !p->xsdata.nut || !p->xsdata.chit || !p->xsdata.scat_matrix || !p->xsdata.inv_sigtr)
        return set_err(ctx, NRAPS_ERR_INVALID, "cross-section arrays are NULL");
    if (!(p->k_new > 0.0f)) return set_err(ctx, NRAPS_ERR_INVALID, "k_new must be positive");
    return NRAPS_OK;
}

cudaMemPool_t ctx_pool(nraps_ctx* ctx) {
    if (ctx->pool) return ctx->pool;
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = ctx->device;
    cudaMemPool_t p = nullptr;
    if (cudaMemPoolCreate(&p, &props) != cudaSuccess) return nullptr;
    /* keep freed memory in the pool: admissions after retirements reuse it */
    uint64_t keep = ~0ULL;
    cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
    ctx->pool = p;
    return p;
}

cudaError_t InstBuffers::alloc(uint64_t G_, uint64_t nc_, uint64_t gens_, uint64_t N, double bank_factor, bool bank,
                               double k0, GenState* st_ext, cudaStream_t s, cudaMemPool_t pool, DeviceArena* arena) {
    G = G_; nc = nc_; gens = gens_;
    double bf = bank_factor > 0 ? bank_factor : 3.0;
    cap = bank ? (uint64_t)(bf * (double)N) + 1024 : 0;
    uint64_t nb = G * nc;
    cudaError_t e = cudaSuccess;
    auto A = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
    /* small buffers at 64 KB strides from the arena, when there is one */
    auto take = [&](DevMem& d, size_t bytes) { A(arena ? d.alloc_in(*arena, bytes) : d.alloc(bytes, pool, s)); };
    /* a small tally keeps its bins one per 32 B sector (see ev_tally_shift) */
    tally_shift = ev_tally_shift(nb);
    take(tally, (nb << tally_shift) * 8); take(flux_acc, nb * 8); take(flux_sum, nb * 8); take(flux_sq, nb * 8);
    take(fs_acc, nc * 8); take(k64, gens * 8); take(entropy, gens * 8);
    if (bank) {
        take(bank0, cap * sizeof(nraps_site)); take(bank1, cap * sizeof(nraps_site));
        take(hist, ev_hist_words(nc) * 4);
        if (e == cudaSuccess) A(cudaMemsetAsync(hist.p, 0, ev_hist_words(nc) * 4, s));
    }
    if (st_ext) st = st_ext;
    else { take(own_state, sizeof(GenState)); st = own_state.as<GenState>(); }
    if (e != cudaSuccess) return e;
    A(cudaMemsetAsync(tally.p, 0, (nb << tally_shift) * 8, s)); A(cudaMemsetAsync(flux_acc.p, 0, nb * 8, s));
    A(cudaMemsetAsync(flux_sum.p, 0, nb * 8, s)); A(cudaMemsetAsync(flux_sq.p, 0, nb * 8, s));
    A(cudaMemsetAsync(fs_acc.p, 0, nc * 8, s)); A(cudaMemsetAsync(k64.p, 0, gens * 8, s));
    A(cudaMemsetAsync(entropy.p, 0, gens * 8, s));
    GenState g0;
    std::memset(&g0, 0, sizeof g0);
    g0.k = k0;
    g0.inv_kf = (float)(1.0 / k0);
    /* from pageable memory: the copy is staged before the call returns, so
       g0 may go out of scope */
    A(cudaMemcpyAsync(st, &g0, sizeof g0, cudaMemcpyHostToDevice, s));
    return e;
}

EvBuffers InstBuffers::view(uint64_t skip, uint64_t seed) const {
    EvBuffers b;
    b.st = st; b.tally = tally.as<double>(); b.tally_shift = tally_shift;
    b.flux_acc = flux_acc.as<double>(); b.fs_acc = fs_acc.as<double>();
    b.flux_sum = flux_sum.as<double>(); b.flux_sq = flux_sq.as<double>();
    b.k64 = k64.as<double>(); b.entropy = entropy.as<double>();
    b.bank[0] = bank0.as<nraps_site>(); b.bank[1] = bank1.as<nraps_site>();
    b.bank_cap = cap; b.hist = hist.as<uint32_t>();
    b.generations = gens; b.skip = skip; b.seed = seed;
    return b;
}

int fetch_results(nraps_ctx* ctx, const ResultsView& v, nraps_result* out) {
    uint64_t nb = v.G * v.nc, gens = v.gens, done = v.done, skip = v.skip;
    std::vector<double> flux(nb), fsum(nb), fsq(nb), fs(v.nc), k64(gens), ent(gens);
    CK(cudaMemcpy(flux.data(), v.flux_acc, nb * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(fsum.data(), v.flux_sum, nb * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(fsq.data(), v.flux_sq, nb * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(fs.data(), v.fs_acc, v.nc * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(k64.data(), v.k64, gens * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(ent.data(), v.entropy, gens * 8, cudaMemcpyDeviceToHost));
    GenState g;
    CK(cudaMemcpy(&g, v.st, sizeof g, cudaMemcpyDeviceToHost));
    std::vector<float> fl(nb), kf(gens, 0.0f), kk(gens, 0.0f);
    for (uint64_t i = 0; i < nb; ++i) fl[i] = (float)flux[i];
    for (uint64_t i = 0; i < gens; ++i) kk[i] = (float)k64[i];
    if (out->flux) std::memcpy(out->flux, fl.data(), nb * 4);
    if (out->fission_source) for (uint64_t c = 0; c < v.nc; ++c) out->fission_source[c] = (float)fs[c];
    if (out->k) std::memcpy(out->k, kk.data(), gens * 4);
    /* average_assembly (src/mc_code.rs:259-274), on the f32 flux */
    if (out->assembly_average) {
        std::vector<float> avg(nb, 0.0f);
        uint64_t na = v.numass ? v.numass : 1, ma = v.nc / na;
        for (uint64_t e = 0; e < v.G; ++e)
            for (uint64_t a = 1; a <= na && ma > 0; ++a) {
                float sum = 0.0f;
                for (uint64_t i = (a - 1) * ma; i < a * ma; ++i) sum += fl[e * v.nc + i];
                float av = sum / (float)ma;
                for (uint64_t i = (a - 1) * ma; i < a * ma; ++i) avg[e * v.nc + i] = av;
            }
        std::memcpy(out->assembly_average, avg.data(), nb * 4);
    }
    /* k_fund (src/mc_code.rs:368-376), running mean of k over active gens */
    if (skip < done) {
        double run = 0.0;
        for (uint64_t i = skip; i < done; ++i) { run += k64[i]; kf[i] = (float)(run / (double)(i - skip + 1)); }
    }
    if (out->k_fund) std::memcpy(out->k_fund, kf.data(), gens * 4);
    if (out->k64) std::memcpy(out->k64, k64.data(), gens * 8);
    if (out->entropy) std::memcpy(out->entropy, ent.data(), gens * 8);
    uint64_t na = done > skip ? done - skip : 0;
    if (out->flux_mean || out->flux_sem) {
        for (uint64_t i = 0; i < nb; ++i) {
            double m = na ? fsum[i] / (double)na : 0.0;
            double var = na > 1 ? std::max(0.0, fsq[i] / (double)na - m * m) / (double)(na - 1) : 0.0;
            if (out->flux_mean) out->flux_mean[i] = m;
            if (out->flux_sem) out->flux_sem[i] = std::sqrt(var);
        }
    }
    if (out->stats) {
        nraps_stats& t = *out->stats;
        std::memset(&t, 0, sizeof t);
        if (na) {
            double sum = 0, sq = 0;
            for (uint64_t i = skip; i < done; ++i) { sum += k64[i]; sq += k64[i] * k64[i]; }
            t.k_mean = sum / (double)na;
            t.k_sigma = na > 1 ? std::sqrt(std::max(0.0, sq / (double)na - t.k_mean * t.k_mean) / (double)(na - 1)) : 0.0;
        }
        t.histories = v.histories;
        t.collisions = g.tot_collisions; t.virtual_collisions = g.tot_virtual;
        t.crossings = g.tot_crossings; t.absorbed = g.tot_absorbed; t.leaked = g.tot_leaked;
        t.capped = g.tot_capped; t.sites = g.tot_sites;
        t.transport_ms = v.transport_ms; t.total_ms = v.total_ms;
        t.transport_launches = v.transport_launches;
        t.gpu_launches = v.gpu_launches;
    }
    return NRAPS_OK;
}

uint64_t InstBuffers::bytes() const {
    return tally.n + flux_acc.n + flux_sum.n + flux_sq.n + fs_acc.n + k64.n + entropy.n + bank0.n + bank1.n +
           hist.n + own_state.n;
}

}  // namespace nrint

namespace {
using nrint::validate_problem;
}  // namespace

struct nraps_session {
    /* small buffers of the session and its engine, each on its own 64 KB
       (declared first: destroyed after every buffer it handed out) */
    DeviceArena arena;
    nraps_ctx* ctx = nullptr;
    nraps_opts o{};
    nraps_variables v{};
    uint64_t N = 0, n_hist = 0, nc = 0, G = 0, M = 0, gens = 0;
    uint64_t cap = 0;
    std::vector<float> cell_dx_host;
    TableLayout L{};
    DevMem tables, tally, flux_acc, flux_sum, flux_sq, fs_acc, k64, entropy, state, partials;
    DevMem sx, scell, sgroup, sparent, sseq, scount, offsets, block_sums, bank0, bank1, hist, records;
    PlainArgs<float> pf{};
    PlainArgs<double> pd{};
    BankArgs ba{};
    FinalizeArgs fa{};
    std::unique_ptr<EventEngine> ev;
    cudaGraphExec_t gexec = nullptr;
    uint64_t graph_kernels = 0;
    uint64_t enqueued = 0;
    bool profile = false;
    std::vector<cudaEvent_t> tev;      /* pairs around transport phases        */
    std::vector<cudaEvent_t> gev;      /* pairs around whole generations        */
    double transport_ms = 0.0, total_ms = 0.0;
    uint64_t transport_launches = 0;
    /* autotuning of the event engine over the inactive generations */
    std::vector<EvParams> tune_cand;
    std::vector<float> tune_ms;          /* whole generation per candidate        */
    std::vector<double> tune_score;      /* ms per real collision                 */
    unsigned long long tune_coll = 0;    /* collisions before the next candidate  */
    size_t tune_next = 0;
    bool tuned = false;
    std::array<uint64_t, 6> tune_key{};  /* the context's cache entry it fills   */
    ~nraps_session() {
        if (gexec) cudaGraphExecDestroy(gexec);
        for (cudaEvent_t e : tev) cudaEventDestroy(e);
        for (cudaEvent_t e : gev) cudaEventDestroy(e);
    }
};

namespace {

template <class T>
void fill_plain(nraps_session* s, PlainArgs<T>& a) {
    unsigned char* b = s->tables.as<unsigned char>();
    const TableLayout& L = s->L;
    a.sigt = (const T*)(b + L.sigt); a.sigs = (const T*)(b + L.sigs); a.siga = (const T*)(b + L.siga);
    a.inv_sigtr = (const T*)(b + L.inv_sigtr); a.nsf = (const T*)(b + L.nsf);
    a.nsf_sigtr = (const T*)(b + L.nsf_sigtr); a.pabs = (const T*)(b + L.pabs);
    a.scat = (const T*)(b + L.scat); a.chi_cdf = (const T*)(b + L.chi_cdf);
    a.phys_cdf = (const T*)(b + L.phys_cdf);
    a.left = (const T*)(b + L.left); a.right = (const T*)(b + L.right); a.dx = (const T*)(b + L.dx);
    a.mat = (const uint8_t*)(b + L.mat); a.fuel = (const uint64_t*)(b + L.fuel);
    a.M = (uint32_t)s->M; a.G = (uint32_t)s->G; a.nc = s->nc; a.nfuel = 0;
    a.boundl = (T)s->v.boundl; a.boundr = (T)s->v.boundr;
    a.base_seed = s->o.seed; a.n_hist = s->n_hist; a.N = s->N;
    a.max_events = s->o.max_events ? s->o.max_events : (1ULL << 24);
    a.st = s->state.as<GenState>();
    a.tally = s->tally.as<double>();
    a.bank[0] = s->bank0.as<nraps_site>(); a.bank[1] = s->bank1.as<nraps_site>();
    a.sink = s->ba.sink;
    a.records = nullptr;
}

int create_session(nraps_ctx* ctx, const nraps_problem* p, bool with_records, nraps_session** out) {
    *out = nullptr;
    int st = validate_problem(ctx, p, ctx->opts);
    if (st) return st;
    std::unique_ptr<nraps_session> s(new nraps_session());
    s->ctx = ctx;
    s->o = ctx->opts;
    s->v = p->variables;
    s->M = p->variables.mattypes; s->G = p->variables.energygroups; s->nc = p->mesh.n_cells;
    s->N = p->variables.histories; s->gens = p->variables.generations;
    s->n_hist = s->N + (s->o.mode == NRAPS_MODE_COMPAT ? s->o.compat_threads : 0);
    std::vector<unsigned char> blob;
    std::string err;
    int bt = (s->o.precision == NRAPS_PREC_FP32) ? build_tables<float>(*p, blob, s->L, err)
                                                 : build_tables<double>(*p, blob, s->L, err);
    if (bt) return set_err(ctx, NRAPS_ERR_INVALID, err);
    cudaStream_t sm = ctx->stream;
    CK(s->tables.alloc_in(s->arena, blob.size()));
    CK(cudaMemcpyAsync(s->tables.p, blob.data(), blob.size(), cudaMemcpyHostToDevice, sm));
    uint64_t nb = s->G * s->nc;
    bool bank = s->o.mode == NRAPS_MODE_BANK;
    bool woodcock = s->o.tracking == NRAPS_TRACK_WOODCOCK;
    /* a Woodcock BANK session scores generation g into half g & 1 of a
       two-half tally, so the event engine may fold a generation beside the
       next one's transport (traces read one tally: they keep one) */
    const uint64_t tally_halves = (woodcock && bank && !with_records) ? 2 : 1;
    /* and keeps a small tally's bins one per 32 B sector */
    const uint32_t tally_shift = (woodcock && !with_records) ? ev_tally_shift(nb) : 0u;
    const uint64_t tally_words = tally_halves * (nb << tally_shift);
    CK(s->tally.alloc_in(s->arena, tally_words * 8));
    CK(s->flux_acc.alloc_in(s->arena, nb * 8)); CK(s->flux_sum.alloc_in(s->arena, nb * 8)); CK(s->flux_sq.alloc_in(s->arena, nb * 8));
    CK(s->fs_acc.alloc_in(s->arena, s->nc * 8));
    CK(s->k64.alloc_in(s->arena, s->gens * 8)); CK(s->entropy.alloc_in(s->arena, s->gens * 8));
    CK(s->state.alloc_in(s->arena, sizeof(GenState)));
    uint32_t nfb = finalize_blocks_for(s->nc);
    CK(s->partials.alloc_in(s->arena, 2 * (size_t)nfb * 8));
    double bf = s->o.bank_factor > 0 ? s->o.bank_factor : 3.0;
    s->cap = bank ? (uint64_t)(bf * (double)s->N) + 1024 : 0;
    if (bank) {
        if (!woodcock) {   /* the event engine keeps its own site slabs */
            CK(s->sx.alloc_in(s->arena, s->cap * 4)); CK(s->scell.alloc_in(s->arena, s->cap * 4)); CK(s->sgroup.alloc_in(s->arena, s->cap * 4));
            CK(s->sparent.alloc_in(s->arena, s->cap * 4)); CK(s->sseq.alloc_in(s->arena, s->cap * 4));
            CK(s->scount.alloc_in(s->arena, s->n_hist * 4)); CK(s->offsets.alloc_in(s->arena, (s->n_hist + 1) * 4));
            CK(s->block_sums.alloc_in(s->arena, ((s->n_hist + 4095) / 4096 + 1) * 4));
            CK(cudaMemsetAsync(s->scount.p, 0, s->n_hist * 4, sm));
        }
        CK(s->bank0.alloc_in(s->arena, s->cap * sizeof(nraps_site))); CK(s->bank1.alloc_in(s->arena, s->cap * sizeof(nraps_site)));
        uint64_t hist_words = woodcock ? ev_hist_words(s->nc) : s->nc;
        CK(s->hist.alloc_in(s->arena, hist_words * 4));
        CK(cudaMemsetAsync(s->hist.p, 0, hist_words * 4, sm));
    }
    if (with_records) {
        CK(s->records.alloc_in(s->arena, s->n_hist * sizeof(nraps_history_record)));
        CK(cudaMemsetAsync(s->records.p, 0, s->n_hist * sizeof(nraps_history_record), sm));
    }
    CK(cudaMemsetAsync(s->tally.p, 0, tally_words * 8, sm));
    CK(cudaMemsetAsync(s->flux_acc.p, 0, nb * 8, sm));
    CK(cudaMemsetAsync(s->flux_sum.p, 0, nb * 8, sm));
    CK(cudaMemsetAsync(s->flux_sq.p, 0, nb * 8, sm));
    CK(cudaMemsetAsync(s->fs_acc.p, 0, s->nc * 8, sm));
    CK(cudaMemsetAsync(s->k64.p, 0, s->gens * 8, sm));
    CK(cudaMemsetAsync(s->entropy.p, 0, s->gens * 8, sm));
    GenState g0;
    std::memset(&g0, 0, sizeof g0);
    g0.k = (double)p->k_new;
    g0.inv_kf = (float)(1.0 / g0.k);
    if (bank && s->o.initial_source == 1) {
        /* generation 0 starts from the diffusion fission source instead of
           the uniform fuel source: the kernels take a non-empty bank */
        std::vector<nraps_site> sites(s->N);
        int ds = nraps_diffusion_source(p, s->N, sites.data(), nullptr);
        if (ds != NRAPS_OK) return set_err(ctx, ds, nraps_host::last_error());
        CK(cudaStreamSynchronize(sm));
        CK(cudaMemcpy(s->bank0.p, sites.data(), s->N * sizeof(nraps_site), cudaMemcpyHostToDevice));
        g0.n_bank = s->N;
    }
    CK(cudaMemcpyAsync(s->state.p, &g0, sizeof g0, cudaMemcpyHostToDevice, sm));

    s->ba.st = s->state.as<GenState>();
    s->ba.sink = SiteSink{s->sx.as<float>(), s->scell.as<uint32_t>(), s->sgroup.as<uint32_t>(),
                          s->sparent.as<uint32_t>(), s->sseq.as<uint32_t>(), s->cap, s->scount.as<uint32_t>()};
    s->ba.n_hist = s->n_hist;
    s->ba.offsets = s->offsets.as<uint32_t>();
    s->ba.block_sums = s->block_sums.as<uint32_t>();
    s->ba.bank[0] = s->bank0.as<nraps_site>(); s->ba.bank[1] = s->bank1.as<nraps_site>();
    s->ba.bank_cap = s->cap;
    s->ba.hist = s->hist.as<uint32_t>();

    if (s->o.precision == NRAPS_PREC_FP32) {
        fill_plain(s.get(), s->pf);
        s->pf.nfuel = p->n_fuel; s->pf.dx_fuel = p->delta_x.fuel;
        if (with_records) s->pf.records = s->records.as<nraps_history_record>();
    } else {
        fill_plain(s.get(), s->pd);
        s->pd.nfuel = p->n_fuel; s->pd.dx_fuel = (double)p->delta_x.fuel;
        if (with_records) s->pd.records = s->records.as<nraps_history_record>();
    }
    unsigned char* b = s->tables.as<unsigned char>();
    FinalizeArgs& f = s->fa;
    f.st = s->state.as<GenState>();
    f.tally = s->tally.as<double>();
    f.nsf64 = (const double*)(b + s->L.nsf64);
    f.dx64 = (const double*)(b + s->L.dx64);
    f.mat = (const uint8_t*)(b + s->L.mat);
    f.M = (uint32_t)s->M; f.G = (uint32_t)s->G; f.nc = s->nc; f.N = s->N;
    f.generations = s->gens; f.skip = s->v.skip; f.mode = s->o.mode;
    f.conv_const = s->L.conv_const;
    f.flux_acc = s->flux_acc.as<double>(); f.fs_acc = s->fs_acc.as<double>();
    f.flux_sum = s->flux_sum.as<double>(); f.flux_sq = s->flux_sq.as<double>();
    f.k64 = s->k64.as<double>(); f.entropy = s->entropy.as<double>();
    f.hist = s->hist.as<uint32_t>(); f.hist_w = s->hist.as<uint32_t>();
    f.partials = s->partials.as<double>(); f.n_blocks = nfb;
    f.bank_mode = bank ? 1 : 0;
    f.bank_cap = s->cap;
    if (woodcock) {
        s->ev.reset(new EventEngine());
        s->ev->set_arena(&s->arena);
        std::string e2;
        int est = s->ev->configure(s->o, e2);
        if (est) return set_err(ctx, est, e2);
        EvBuffers eb;
        eb.st = s->state.as<GenState>(); eb.tally = s->tally.as<double>();
        eb.tally_shift = tally_shift;
        eb.tally_stride = tally_halves == 2 ? nb << tally_shift : 0;
        eb.flux_acc = s->flux_acc.as<double>(); eb.fs_acc = s->fs_acc.as<double>();
        eb.flux_sum = s->flux_sum.as<double>(); eb.flux_sq = s->flux_sq.as<double>();
        eb.k64 = s->k64.as<double>(); eb.entropy = s->entropy.as<double>();
        eb.bank[0] = s->bank0.as<nraps_site>(); eb.bank[1] = s->bank1.as<nraps_site>();
        eb.bank_cap = s->cap; eb.hist = s->hist.as<uint32_t>();
        eb.generations = s->gens; eb.skip = s->v.skip; eb.seed = s->o.seed;
        if (s->ev->add_instance(*p, eb, e2) < 0) return set_err(ctx, NRAPS_ERR_INVALID, e2);
        if (with_records) s->ev->set_records(s->records.as<nraps_history_record>());
        est = s->ev->commit(sm, e2);
        if (est) return set_err(ctx, est, e2);
        /* tune block size, collisions per pass and pass count unless all given */
        const std::array<uint64_t, 6> key = {s->M, s->G, s->nc, s->N, (uint64_t)s->o.mode, (uint64_t)s->o.exact_log};
        const auto hit = ctx->tuned.find(key);
        if (!with_records && s->o.block_size == 0 && s->o.events_per_pass == 0 && s->o.passes == 0 &&
            s->o.tail_lanes == 0 && s->o.sort_rounds == 0 && s->o.range_len == 0 && hit != ctx->tuned.end()) {
            /* tuned before on this context for a problem of this shape */
            s->ev->params = hit->second;
            int gs = s->ev->size_grid();
            if (gs) return set_err(ctx, gs, "event engine: launch shape");
            s->tuned = true;
        } else if (!with_records && s->o.block_size == 0 && s->o.events_per_pass == 0 && s->o.passes == 0 &&
            s->o.tail_lanes == 0 && s->o.sort_rounds == 0 && s->o.range_len == 0) {
            s->tune_key = key;
            /* likeliest first: short inactive phases try only the head.
               {block, K, passes, tail, sort rounds, range} */
            const uint32_t X = NRAPS_ONE_PASS;
            const uint32_t cand[][6] = {{256, X, 0, 0, 0, 0}, {128, X, 0, 0, 0, 0}, {128, X, 0, 0, 8, 0},
                                        {128, X, 0, 0, 0, 1024}, {128, X, 0, 0, 0, 4096},
                                        {256, X, 0, 0, 0, 2048}, {128, X, 0, 0, 0, 2048}, {128, X, 0, 0, 12, 0},
                                        {128, X, 0, 0, 0, 512}, {256, 16, 1, 0, 0, 0}, {256, X, 1, 12, 0, 0},
                                        {256, 4, 1, 0, 0, 0}};
            size_t n = sizeof(cand) / sizeof(cand[0]);
            size_t budget = (size_t)std::min<uint64_t>(s->v.skip, n);
            for (size_t i = 0; i < budget; ++i) {
                EvParams pr;
                pr.block = cand[i][0]; pr.K = cand[i][1]; pr.passes = cand[i][2]; pr.tail = cand[i][3];
                pr.sort = cand[i][4]; pr.range = cand[i][5];
                s->tune_cand.push_back(pr);
            }
            s->tuned = s->tune_cand.size() < 2;
        } else {
            s->tuned = true;
        }
    }
    s->cell_dx_host.assign(p->mesh.delta_x, p->mesh.delta_x + s->nc);
    CK(cudaStreamSynchronize(sm));
    *out = s.release();
    return NRAPS_OK;
}

/* Enqueue the transport phase of one (plain) generation; returns kernels launched. */
int enqueue_transport(nraps_session* s, cudaStream_t sm) {
    int block = (int)s->o.block_size;
    if (s->o.precision == NRAPS_PREC_FP32) return launch_plain<float>(s->pf, s->o.mode, block, sm);
    return launch_plain<double>(s->pd, s->o.mode, block, sm);
}

/* Whole generation: transport, bank ordering, finalize. */
int enqueue_generation(nraps_session* s, cudaStream_t sm, cudaEvent_t t0, cudaEvent_t t1) {
    if (s->ev) return s->ev->enqueue_generation(sm, true, t0, t1);
    int n = 0, r;
    if (t0) cudaEventRecord(t0, sm);
    r = enqueue_transport(s, sm);
    if (r < 0) return r;
    n += r;
    if (t1) cudaEventRecord(t1, sm);
    if (s->o.mode == NRAPS_MODE_BANK) {
        r = launch_bank_order(s->ba, sm);
        if (r < 0) return r;
        n += r;
    }
    r = launch_finalize(s->fa, sm);
    if (r < 0) return r;
    return n + r;
}

int read_state(nraps_session* s, GenState& g) {
    nraps_ctx* ctx = s->ctx;
    CK(cudaMemcpy(&g, s->state.p, sizeof g, cudaMemcpyDeviceToHost));
    return NRAPS_OK;
}

int state_status(nraps_session* s, const GenState& g) {
    if (g.error & NR_ERR_STALLED)
        return set_err(s->ctx, NRAPS_ERR_CUDA, "a bounded device wait ran out (a range's chunk id)");
    if (g.error & NR_ERR_CAPACITY)
        return set_err(s->ctx, NRAPS_ERR_CAPACITY, "fission bank overflowed its capacity (raise opts.bank_factor)");
    if (g.error & NR_ERR_EMPTY)
        return set_err(s->ctx, NRAPS_ERR_EMPTY_BANK, "fission bank empty: no source for the next generation");
    if (g.error & NR_ERR_CAPPED)
        return set_err(s->ctx, NRAPS_ERR_CAPPED, "a history reached the per-history event cap (opts.max_events)");
    return NRAPS_OK;
}

}  // namespace

extern "C" {

void nraps_opts_default(nraps_opts* o) {
    if (!o) return;
    std::memset(o, 0, sizeof *o);
    o->abi_version = NRAPS_ABI_VERSION;
    o->device = -1;
    o->seed = 1;
    o->mode = NRAPS_MODE_COMPAT;
    o->precision = NRAPS_PREC_FP64;
    o->tracking = NRAPS_TRACK_SURFACE;
}

int nraps_create(nraps_ctx** out, const nraps_opts* opts) {
    nraps_ctx* ctx = nullptr;
    if (!out) return set_err(nullptr, NRAPS_ERR_INVALID, "out is NULL");
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return set_err(nullptr, NRAPS_ERR_NO_DEVICE,
                       std::string("no CUDA device: ") + (e != cudaSuccess ? cudaGetErrorString(e) : "0 devices"));
    std::unique_ptr<nraps_ctx> c(new nraps_ctx());
    if (opts) c->opts = *opts; else nraps_opts_default(&c->opts);
    if (c->opts.abi_version != NRAPS_ABI_VERSION)
        return set_err(nullptr, NRAPS_ERR_INVALID, "opts.abi_version mismatch");
    if (c->opts.device >= 0) {
        if (c->opts.device >= ndev) return set_err(nullptr, NRAPS_ERR_INVALID, "opts.device out of range");
        e = cudaSetDevice(c->opts.device);
        if (e != cudaSuccess) return set_err(nullptr, NRAPS_ERR_CUDA, cudaGetErrorString(e));
    }
    cudaGetDevice(&c->device);
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return set_err(nullptr, NRAPS_ERR_CUDA, cudaGetErrorString(e));
    *out = c.release();
    return NRAPS_OK;
}

void nraps_destroy(nraps_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) { cudaStreamSynchronize(ctx->stream); cudaStreamDestroy(ctx->stream); }
    if (ctx->pool) cudaMemPoolDestroy(ctx->pool);
    delete ctx;
}

const char* nraps_last_error(const nraps_ctx* ctx) {
    return ctx ? ctx->err.c_str() : nraps_host::last_error();
}

int nraps_set_opts(nraps_ctx* ctx, const nraps_opts* o) {
    if (!ctx || !o) return set_err(ctx, NRAPS_ERR_INVALID, "NULL argument");
    if (o->abi_version != NRAPS_ABI_VERSION) return set_err(ctx, NRAPS_ERR_INVALID, "opts.abi_version mismatch");
    int dev = ctx->opts.device;
    ctx->opts = *o;
    ctx->opts.device = dev;
    return NRAPS_OK;
}

int nraps_get_opts(const nraps_ctx* ctx, nraps_opts* out) {
    if (!ctx || !out) return NRAPS_ERR_INVALID;
    *out = ctx->opts;
    return NRAPS_OK;
}

uint64_t nraps_launch_count(const nraps_ctx* ctx) { return ctx ? ctx->launches : 0; }

void* nraps_ctx_stream(nraps_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int nraps_session_create(nraps_ctx* ctx, const nraps_problem* problem, nraps_session** out) {
    if (!ctx || !out) return set_err(ctx, NRAPS_ERR_INVALID, "NULL argument");
    cudaSetDevice(ctx->device);
    return create_session(ctx, problem, false, out);
}

void nraps_session_destroy(nraps_session* s) {
    if (!s) return;
    cudaSetDevice(s->ctx->device);
    cudaStreamSynchronize(s->ctx->stream);
    delete s;
}

uint64_t nraps_session_generation(const nraps_session* s) { return s ? s->enqueued : 0; }

int nraps_session_set_profile(nraps_session* s, int on) {
    if (!s) return NRAPS_ERR_INVALID;
    s->profile = on != 0;
    return NRAPS_OK;
}

int nraps_session_run(nraps_session* s, uint64_t n) {
    if (!s) return NRAPS_ERR_INVALID;
    nraps_ctx* ctx = s->ctx;
    cudaSetDevice(ctx->device);
    cudaStream_t sm = ctx->stream;
    if (s->enqueued + n > s->gens) n = s->gens - s->enqueued;
    for (uint64_t i = 0; i < n; ++i) {
        if (s->ev && !s->tuned) {
            /* one candidate per generation: histories do not depend on the
               candidate, so tuning leaves every result unchanged */
            EvParams& pr = s->tune_cand[s->tune_next];
            s->ev->params = pr;
            s->ev->size_grid();
            /* a candidate is scored by its whole generation (transport, bank
               ordering, finalize) per real collision: the source still moves
               during the inactive generations, so histories get longer or
               shorter from one candidate to the next */
            cudaEvent_t e[4];
            for (int j = 0; j < 4; ++j) CK(cudaEventCreate(&e[j]));
            CK(cudaEventRecord(e[0], sm));
            int r = s->ev->enqueue_generation(sm, true, e[1], e[2]);
            if (r < 0) return set_err(ctx, NRAPS_ERR_CUDA, std::string("kernel launch failed: ") + cudaGetErrorString(cudaGetLastError()));
            CK(cudaEventRecord(e[3], sm));
            ctx->launches += (uint64_t)r;
            s->transport_launches += s->ev->launches_per_generation();
            CK(cudaEventSynchronize(e[3]));
            float ms = 0.f, tms = 0.f;
            CK(cudaEventElapsedTime(&ms, e[0], e[3]));
            CK(cudaEventElapsedTime(&tms, e[1], e[2]));
            for (int j = 0; j < 4; ++j) cudaEventDestroy(e[j]);
            GenState g;
            CK(cudaMemcpy(&g, s->state.p, sizeof g, cudaMemcpyDeviceToHost));
            const unsigned long long coll = g.tot_collisions - s->tune_coll;
            s->tune_coll = g.tot_collisions;
            s->tune_ms.push_back(ms);
            s->tune_score.push_back(coll ? (double)ms / (double)coll : (double)ms);
            s->transport_ms += tms;
            if (++s->tune_next == s->tune_cand.size()) {
                size_t best = 0;
                for (size_t j = 1; j < s->tune_score.size(); ++j) if (s->tune_score[j] < s->tune_score[best]) best = j;
                s->ev->params = s->tune_cand[best];
                s->ev->size_grid();
                s->tuned = true;
                ctx->tuned[s->tune_key] = s->tune_cand[best];
            }
            s->enqueued++;
            continue;
        }
        if (s->profile) {
            cudaEvent_t e[4];
            for (int j = 0; j < 4; ++j) CK(cudaEventCreate(&e[j]));
            CK(cudaEventRecord(e[0], sm));
            int r = enqueue_generation(s, sm, e[1], e[2]);
            if (r < 0) return set_err(ctx, NRAPS_ERR_CUDA, std::string("kernel launch failed: ") + cudaGetErrorString(cudaGetLastError()));
            CK(cudaEventRecord(e[3], sm));
            s->tev.push_back(e[1]); s->tev.push_back(e[2]);
            s->gev.push_back(e[0]); s->gev.push_back(e[3]);
            ctx->launches += (uint64_t)r;
            s->transport_launches += s->ev ? s->ev->launches_per_generation() : 1;
        } else if (s->o.use_graphs) {
            if (!s->gexec) {
                cudaGraph_t graph;
                CK(cudaStreamBeginCapture(sm, cudaStreamCaptureModeThreadLocal));
                int r = enqueue_generation(s, sm, nullptr, nullptr);
                cudaError_t ce = cudaStreamEndCapture(sm, &graph);
                if (r < 0 || ce != cudaSuccess)
                    return set_err(ctx, NRAPS_ERR_CUDA, std::string("graph capture failed: ") + cudaGetErrorString(ce));
                cudaError_t ie = cudaGraphInstantiate(&s->gexec, graph, 0);
                cudaGraphDestroy(graph);
                if (ie != cudaSuccess) return set_err(ctx, NRAPS_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie));
                s->graph_kernels = (uint64_t)r;
            }
            CK(cudaGraphLaunch(s->gexec, sm));
            ctx->launches += s->graph_kernels;
            s->transport_launches += s->ev ? s->ev->launches_per_generation() : 1;
        } else {
            int r = enqueue_generation(s, sm, nullptr, nullptr);
            if (r < 0) return set_err(ctx, NRAPS_ERR_CUDA, std::string("kernel launch failed: ") + cudaGetErrorString(cudaGetLastError()));
            ctx->launches += (uint64_t)r;
            s->transport_launches += s->ev ? s->ev->launches_per_generation() : 1;
        }
        s->enqueued++;
    }
    return NRAPS_OK;
}

int nraps_session_flush(nraps_session* s) {
    if (!s) return NRAPS_ERR_INVALID;
    nraps_ctx* ctx = s->ctx;
    cudaSetDevice(ctx->device);
    if (s->ev) {
        /* flux, fission source and entropy of a deferred last generation */
        const int r = s->ev->flush_fold(ctx->stream);
        if (r < 0) return set_err(ctx, NRAPS_ERR_CUDA, "fold flush launch failed");
        ctx->launches += (uint64_t)r;
    }
    return NRAPS_OK;
}

int nraps_session_sync(nraps_session* s) {
    if (!s) return NRAPS_ERR_INVALID;
    nraps_ctx* ctx = s->ctx;
    cudaSetDevice(ctx->device);
    const int fl = nraps_session_flush(s);
    if (fl) return fl;
    CK(cudaStreamSynchronize(ctx->stream));
    for (size_t i = 0; i + 1 < s->tev.size(); i += 2) {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, s->tev[i], s->tev[i + 1]));
        s->transport_ms += ms;
        cudaEventDestroy(s->tev[i]); cudaEventDestroy(s->tev[i + 1]);
    }
    s->tev.clear();
    for (size_t i = 0; i + 1 < s->gev.size(); i += 2) {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, s->gev[i], s->gev[i + 1]));
        s->total_ms += ms;
        cudaEventDestroy(s->gev[i]); cudaEventDestroy(s->gev[i + 1]);
    }
    s->gev.clear();
    GenState g;
    int st = read_state(s, g);
    if (st) return st;
    return state_status(s, g);
}

int nraps_session_tuning(nraps_session* s, uint32_t* block, uint32_t* events_per_pass, uint32_t* passes,
                         uint32_t* tail_lanes, uint32_t* sort_rounds, uint32_t* range_len, uint32_t* n_tried,
                         float* tried_ms, uint32_t tried_cap) {
    if (!s) return NRAPS_ERR_INVALID;
    if (!s->ev) return set_err(s->ctx, NRAPS_ERR_INVALID, "tuning applies to WOODCOCK sessions");
    if (block) *block = s->ev->params.block;
    if (events_per_pass) *events_per_pass = s->ev->params.K;
    if (passes) *passes = s->ev->params.passes;
    if (tail_lanes) *tail_lanes = s->ev->params.tail;
    if (sort_rounds) *sort_rounds = s->ev->params.sort;
    if (range_len) *range_len = s->ev->params.range;
    if (n_tried) *n_tried = (uint32_t)s->tune_ms.size();
    for (uint32_t i = 0; tried_ms && i < tried_cap && i < s->tune_ms.size(); ++i) tried_ms[i] = s->tune_ms[i];
    return NRAPS_OK;
}

int nraps_session_timing(nraps_session* s, double* transport_ms, double* total_ms,
                         uint64_t* transport_launches, uint64_t* collisions, uint64_t* histories) {
    if (!s) return NRAPS_ERR_INVALID;
    int st = nraps_session_sync(s);
    GenState g;
    int st2 = read_state(s, g);
    if (st2) return st2;
    if (transport_ms) *transport_ms = s->transport_ms;
    if (total_ms) *total_ms = s->total_ms;
    if (transport_launches) *transport_launches = s->transport_launches;
    if (collisions) *collisions = g.tot_collisions;
    if (histories) *histories = s->enqueued * s->n_hist;
    return st;
}

int nraps_session_results(nraps_session* s, nraps_result* out) {
    if (!s || !out) return set_err(s ? s->ctx : nullptr, NRAPS_ERR_INVALID, "NULL argument");
    int st = nraps_session_sync(s);
    if (st) return st;
    nrint::ResultsView v;
    v.G = s->G; v.nc = s->nc; v.gens = s->gens; v.skip = s->v.skip; v.numass = s->v.numass;
    v.done = std::min(s->enqueued, s->gens); v.histories = s->enqueued * s->n_hist;
    v.flux_acc = s->flux_acc.as<double>(); v.flux_sum = s->flux_sum.as<double>();
    v.flux_sq = s->flux_sq.as<double>(); v.fs_acc = s->fs_acc.as<double>();
    v.k64 = s->k64.as<double>(); v.entropy = s->entropy.as<double>();
    v.st = s->state.as<GenState>();
    v.transport_ms = s->transport_ms; v.total_ms = s->total_ms;
    v.transport_launches = s->transport_launches; v.gpu_launches = s->ctx->launches;
    return nrint::fetch_results(s->ctx, v, out);
}

int nraps_solve(nraps_ctx* ctx, const nraps_problem* problem, nraps_result* out) {
    if (!ctx || !problem || !out) return set_err(ctx, NRAPS_ERR_INVALID, "NULL argument");
    nraps_session* s = nullptr;
    int st = nraps_session_create(ctx, problem, &s);
    if (st) return st;
    st = nraps_session_run(s, problem->variables.generations);
    if (!st) st = nraps_session_results(s, out);
    nraps_session_destroy(s);
    return st;
}

int nraps_monte_carlo(nraps_ctx* ctx, const nraps_variables* variables, const nraps_xsdata* xsdata,
                      const nraps_delta_x* delta_x, const nraps_mesh* meshid,
                      const uint64_t* fuel_indices, uint64_t n_fuel, float k_new, nraps_result* out) {
    if (!variables || !xsdata || !delta_x || !meshid)
        return set_err(ctx, NRAPS_ERR_INVALID, "NULL argument");
    nraps_problem p;
    p.variables = *variables; p.xsdata = *xsdata; p.delta_x = *delta_x; p.mesh = *meshid;
    p.fuel_indices = fuel_indices; p.n_fuel = n_fuel; p.k_new = k_new;
    return nraps_solve(ctx, &p, out);
}

int nraps_trace_generation(nraps_ctx* ctx, const nraps_problem* problem, uint64_t generation, double k,
                           const nraps_site* sites_in, uint64_t n_sites_in,
                           nraps_history_record* records, uint64_t n_records, double* tally,
                           nraps_site* sites_out, uint64_t cap_sites_out, uint64_t* n_sites_out,
                           uint64_t* k_fixed_out) {
    if (!ctx || !problem || !records) return set_err(ctx, NRAPS_ERR_INVALID, "NULL argument");
    cudaSetDevice(ctx->device);
    nraps_problem p = *problem;
    if (p.variables.generations <= generation) p.variables.generations = generation + 1;
    if (p.variables.skip >= p.variables.generations) p.variables.skip = p.variables.generations - 1;
    nraps_session* s = nullptr;
    int st = create_session(ctx, &p, true, &s);
    if (st) return st;
    std::unique_ptr<nraps_session> hold(s);
    if (n_records != s->n_hist) return set_err(ctx, NRAPS_ERR_INVALID, "n_records must equal the histories simulated");
    cudaStream_t sm = ctx->stream;
    GenState g0;
    std::memset(&g0, 0, sizeof g0);
    g0.gen = generation; g0.k = k; g0.inv_kf = (float)(1.0 / k);
    if (sites_in && n_sites_in) {
        if (s->o.mode != NRAPS_MODE_BANK) return set_err(ctx, NRAPS_ERR_INVALID, "sites_in needs BANK mode");
        if (n_sites_in > s->cap) return set_err(ctx, NRAPS_ERR_CAPACITY, "sites_in exceeds the bank capacity");
        void* dst = (generation & 1) ? s->bank1.p : s->bank0.p;
        CK(cudaMemcpyAsync(dst, sites_in, n_sites_in * sizeof(nraps_site), cudaMemcpyHostToDevice, sm));
        g0.n_bank = n_sites_in;
    }
    CK(cudaMemcpyAsync(s->state.p, &g0, sizeof g0, cudaMemcpyHostToDevice, sm));
    if (s->ev) {
        int r = s->ev->enqueue_generation(sm, false);
        if (r < 0) return set_err(ctx, NRAPS_ERR_CUDA, std::string("kernel launch failed: ") + cudaGetErrorString(cudaGetLastError()));
        ctx->launches += (uint64_t)r;
    } else {
        int r = enqueue_transport(s, sm);
        if (r < 0) return set_err(ctx, NRAPS_ERR_CUDA, std::string("kernel launch failed: ") + cudaGetErrorString(cudaGetLastError()));
        ctx->launches += (uint64_t)r;
        if (s->o.mode == NRAPS_MODE_BANK) {
            r = launch_bank_order(s->ba, sm);
            if (r < 0) return set_err(ctx, NRAPS_ERR_CUDA, "bank ordering launch failed");
            ctx->launches += (uint64_t)r;
        }
    }
    CK(cudaStreamSynchronize(sm));
    CK(cudaMemcpy(records, s->records.p, s->n_hist * sizeof(nraps_history_record), cudaMemcpyDeviceToHost));
    if (tally) CK(cudaMemcpy(tally, s->tally.p, s->G * s->nc * 8, cudaMemcpyDeviceToHost));
    GenState g;
    CK(cudaMemcpy(&g, s->state.p, sizeof g, cudaMemcpyDeviceToHost));
    if (k_fixed_out) *k_fixed_out = g.kq;
    uint64_t B = 0;
    if (s->o.mode == NRAPS_MODE_BANK) {
        if (s->ev) {
            uint32_t tot = 0;
            CK(cudaMemcpy(&tot, s->ev->offsets() + s->ev->n_total(), 4, cudaMemcpyDeviceToHost));
            B = std::min<uint64_t>(tot, s->cap);
        } else {
            B = std::min<uint64_t>(g.n_bank_next, s->cap);
        }
    }
    if (n_sites_out) *n_sites_out = B;
    if (sites_out && B) {
        void* src = ((generation + 1) & 1) ? s->bank1.p : s->bank0.p;
        CK(cudaMemcpy(sites_out, src, std::min(B, cap_sites_out) * sizeof(nraps_site), cudaMemcpyDeviceToHost));
        if (B > cap_sites_out) return set_err(ctx, NRAPS_ERR_CAPACITY, "sites_out too small");
    }
    if (g.error & NR_ERR_CAPACITY) return set_err(ctx, NRAPS_ERR_CAPACITY, "fission bank overflowed");
    return NRAPS_OK;
}

int nraps_pcg32_stream(nraps_ctx* ctx, uint64_t seed, const uint64_t* streams, uint64_t n_streams,
                       uint32_t per_stream, uint32_t* out) {
    if (!ctx || !streams || !out) return set_err(ctx, NRAPS_ERR_INVALID, "NULL argument");
    cudaSetDevice(ctx->device);
    DevMem ds, dout;
    CK(ds.alloc(n_streams * 8));
    CK(dout.alloc(n_streams * per_stream * 4));
    CK(cudaMemcpy(ds.p, streams, n_streams * 8, cudaMemcpyHostToDevice));
    int r = launch_pcg_stream(seed, ds.as<uint64_t>(), n_streams, per_stream, dout.as<uint32_t>(), ctx->stream);
    if (r < 0) return set_err(ctx, NRAPS_ERR_CUDA, "pcg kernel launch failed");
    ctx->launches += (uint64_t)r;
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(out, dout.p, n_streams * per_stream * 4, cudaMemcpyDeviceToHost));
    return NRAPS_OK;
}

int nraps_log_eval(nraps_ctx* ctx, const double* x, uint64_t n, double* out64, float* out32) {
    if (!ctx || !x || !out64 || !out32) return set_err(ctx, NRAPS_ERR_INVALID, "NULL argument");
    cudaSetDevice(ctx->device);
    DevMem dx, d64, d32;
    CK(dx.alloc(n * 8)); CK(d64.alloc(n * 8)); CK(d32.alloc(n * 4));
    CK(cudaMemcpy(dx.p, x, n * 8, cudaMemcpyHostToDevice));
    int r = launch_log_eval(dx.as<double>(), n, d64.as<double>(), d32.as<float>(), ctx->stream);
    if (r < 0) return set_err(ctx, NRAPS_ERR_CUDA, "log kernel launch failed");
    ctx->launches += (uint64_t)r;
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(out64, d64.p, n * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(out32, d32.p, n * 4, cudaMemcpyDeviceToHost));
    return NRAPS_OK;
}

}  /* extern "C" */
