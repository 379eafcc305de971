/*
 * serve.cu — batched instances and the request server (host runtime).
 *
 * Batch: several independent slab problems advance one generation each per
 * launch sequence of the event engine (one persistent launch per pass for all
 * instances).  With opts.use_graphs the sequence is captured once as a CUDA
 * graph and replayed every generation; generation indices, k and bank sizes
 * live in device memory, so the replay needs no host work.
 *
 * Server: a continuous-batching loop for k-eigenvalue requests.  Submitted
 * requests wait in a FIFO; each step admits waiting requests while device
 * slots and the HBM budget allow (their tables, tallies and both fission
 * banks stay resident until the request is released), runs one generation of
 * every admitted request together, reads back every request's k statistics
 * with one copy, and retires requests whose k standard error reached the
 * target (or whose generation cap was hit).  A request's result does not
 * depend on which other requests shared its steps: every particle owns a
 * PCG32 stream of its request's seed, and k is accumulated exactly.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "engine_internal.hpp"

using nrint::DevMem;
using nrint::InstBuffers;
using nrint::set_err;

#define CK(call)                                                                        \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess)                                                          \
            return set_err(ctx, nrint::cuda_status(e_), std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

namespace {

/* A deep copy of a problem: the caller's arrays may go away after submit. */
struct ProblemCopy {
    nraps_problem p{};
    std::vector<float> sigt, sigs, mu, siga, sigf, nut, chit, scat, inv, dx, left, right;
    std::vector<uint8_t> mat;
    std::vector<uint64_t> fuel;
    void take(const nraps_problem& src) {
        p = src;
        uint64_t nx = src.xsdata.n_xs, ns = src.xsdata.n_scat, nc = src.mesh.n_cells;
        auto cp = [](const float* a, uint64_t n) { return std::vector<float>(a, a + n); };
        sigt = cp(src.xsdata.sigt, nx); sigs = cp(src.xsdata.sigs, nx); mu = cp(src.xsdata.mu, nx);
        siga = cp(src.xsdata.siga, nx); sigf = cp(src.xsdata.sigf, nx); nut = cp(src.xsdata.nut, nx);
        chit = cp(src.xsdata.chit, nx); inv = cp(src.xsdata.inv_sigtr, nx); scat = cp(src.xsdata.scat_matrix, ns);
        dx = cp(src.mesh.delta_x, nc); left = cp(src.mesh.mesh_left, nc); right = cp(src.mesh.mesh_right, nc);
        mat.assign(src.mesh.matid, src.mesh.matid + nc);
        fuel.assign(src.fuel_indices, src.fuel_indices + src.n_fuel);
        p.xsdata.sigt = sigt.data(); p.xsdata.sigs = sigs.data(); p.xsdata.mu = mu.data();
        p.xsdata.siga = siga.data(); p.xsdata.sigf = sigf.data(); p.xsdata.nut = nut.data();
        p.xsdata.chit = chit.data(); p.xsdata.scat_matrix = scat.data(); p.xsdata.inv_sigtr = inv.data();
        p.mesh.matid = mat.data(); p.mesh.delta_x = dx.data(); p.mesh.mesh_left = left.data();
        p.mesh.mesh_right = right.data(); p.fuel_indices = fuel.data();
    }
};

nrint::ResultsView view_of(const InstBuffers& b, const nraps_variables& v, uint64_t done, uint64_t hist,
                           double ms, uint64_t launches, uint64_t gpu_launches) {
    nrint::ResultsView r;
    r.G = b.G; r.nc = b.nc; r.gens = b.gens; r.skip = v.skip; r.numass = v.numass;
    r.done = done; r.histories = hist;
    r.flux_acc = b.flux_acc.as<double>(); r.flux_sum = b.flux_sum.as<double>();
    r.flux_sq = b.flux_sq.as<double>(); r.fs_acc = b.fs_acc.as<double>();
    r.k64 = b.k64.as<double>(); r.entropy = b.entropy.as<double>();
    r.st = b.st;
    r.transport_ms = ms; r.total_ms = ms; r.transport_launches = launches; r.gpu_launches = gpu_launches;
    return r;
}

int check_opts(nraps_ctx* ctx) {
    const nraps_opts& o = ctx->opts;
    if (o.tracking != NRAPS_TRACK_WOODCOCK || o.precision != NRAPS_PREC_FP32 ||
        (o.mode != NRAPS_MODE_BANK && o.mode != NRAPS_MODE_PHYSICS))
        return set_err(ctx, NRAPS_ERR_INVALID, "batches and the server run the WOODCOCK engine (FP32, PHYSICS or BANK)");
    return NRAPS_OK;
}

}  // namespace

/* ======================================================================== */
struct nraps_batch {
    /* small buffers of the batch's instances and engine at 64 KB strides
       (declared first: destroyed after every buffer it handed out) */
    DeviceArena arena;
    nraps_ctx* ctx = nullptr;
    EventEngine ev;
    std::vector<std::unique_ptr<InstBuffers>> buf;
    std::vector<nraps_variables> vars;
    std::vector<uint64_t> n_hist;
    uint64_t enqueued = 0, max_gens = 0, histories_per_gen = 0;
    cudaGraphExec_t gexec = nullptr;
    uint64_t graph_kernels = 0;
    std::vector<cudaEvent_t> ev_pairs;
    double ms = 0.0;
    /* autotuning over the first inactive generations: {block, range} */
    std::vector<std::pair<uint32_t, uint32_t>> tune_cand;
    std::vector<float> tune_ms;
    std::vector<double> tune_score;
    unsigned long long tune_coll = 0;
    bool tuned = true;
    ~nraps_batch() {
        if (gexec) cudaGraphExecDestroy(gexec);
        for (cudaEvent_t e : ev_pairs) cudaEventDestroy(e);
    }
};

extern "C" {

int nraps_batch_create(nraps_ctx* ctx, const nraps_problem* problems, uint32_t n, const uint64_t* seeds,
                       nraps_batch** out) {
    if (!ctx || !problems || !out || n == 0) return set_err(ctx, NRAPS_ERR_INVALID, "NULL argument or empty batch");
    *out = nullptr;
    cudaSetDevice(ctx->device);
    int st = check_opts(ctx);
    if (st) return st;
    std::unique_ptr<nraps_batch> b(new nraps_batch());
    b->ctx = ctx;
    std::string err;
    b->ev.set_arena(&b->arena);
    if ((st = b->ev.configure(ctx->opts, err))) return set_err(ctx, st, err);
    /* one ranged pass (every particle to its end; each block a 4096-history
       range of one instance, its tables in shared memory): the fastest
       measured shape for 256 mixed instances, 4.1 ms per generation against
       9.4 ms for one persistent pass reading tables through L1 */
    if (ctx->opts.block_size == 0) b->ev.params.block = 128;
    if (ctx->opts.events_per_pass == 0 && ctx->opts.passes == 0) {
        b->ev.params.K = NRAPS_ONE_PASS; b->ev.params.passes = 0;
        b->ev.params.range = ctx->opts.range_len ? ctx->opts.range_len : 4096;
    } else if (ctx->opts.passes == 0 && b->ev.params.K != NRAPS_ONE_PASS) {
        b->ev.params.passes = 1;
    }
    /* with no shape given, the first inactive generations each try one
       (block, range length) of a ranged pass -- blocks of 128, 256 and 512
       threads, ranges of 1024..8192 histories -- and keep the one with the
       least time per real collision; likeliest first, so short inactive
       phases try only the head.  Results do not depend on the shape. */
    if (ctx->opts.block_size == 0 && ctx->opts.range_len == 0 && ctx->opts.events_per_pass == 0 &&
        ctx->opts.passes == 0) {
        const uint32_t cand[][2] = {{128, 4096}, {256, 4096}, {512, 4096}, {128, 2048}, {256, 8192},
                                    {512, 8192}, {128, 8192}, {256, 2048}, {512, 2048}, {128, 1024},
                                    {256, 1024}, {512, 1024}};
        uint64_t skip = ~0ULL;
        for (uint32_t i = 0; i < n; ++i) skip = std::min<uint64_t>(skip, problems[i].variables.skip);
        const size_t budget = (size_t)std::min<uint64_t>(skip, sizeof(cand) / sizeof(cand[0]));
        for (size_t i = 0; i < budget; ++i) b->tune_cand.emplace_back(cand[i][0], cand[i][1]);
        b->tuned = b->tune_cand.size() < 2;
    }
    bool bank = ctx->opts.mode == NRAPS_MODE_BANK;
    for (uint32_t i = 0; i < n; ++i) {
        const nraps_problem& p = problems[i];
        if ((st = nrint::validate_problem(ctx, &p, ctx->opts))) return st;
        std::unique_ptr<InstBuffers> ib(new InstBuffers());
        cudaError_t e = ib->alloc(p.variables.energygroups, p.mesh.n_cells, p.variables.generations,
                                  p.variables.histories, ctx->opts.bank_factor, bank, (double)p.k_new, nullptr,
                                  ctx->stream, nullptr, &b->arena);
        if (e != cudaSuccess) return set_err(ctx, nrint::cuda_status(e), std::string("batch buffers: ") + cudaGetErrorString(e));
        uint64_t seed = seeds ? seeds[i] : ctx->opts.seed + i;
        if (b->ev.add_instance(p, ib->view(p.variables.skip, seed), err) < 0)
            return set_err(ctx, NRAPS_ERR_INVALID, "instance " + std::to_string(i) + ": " + err);
        b->buf.push_back(std::move(ib));
        b->vars.push_back(p.variables);
        b->n_hist.push_back(p.variables.histories);
        b->max_gens = std::max<uint64_t>(b->max_gens, p.variables.generations);
        b->histories_per_gen += p.variables.histories;
    }
    if ((st = b->ev.commit(ctx->stream, err))) return set_err(ctx, st, err);
    CK(cudaStreamSynchronize(ctx->stream));
    *out = b.release();
    return NRAPS_OK;
}

int nraps_batch_run(nraps_batch* b, uint64_t n) {
    if (!b) return NRAPS_ERR_INVALID;
    nraps_ctx* ctx = b->ctx;
    cudaSetDevice(ctx->device);
    cudaStream_t sm = ctx->stream;
    if (b->enqueued + n > b->max_gens) n = b->max_gens - b->enqueued;
    for (uint64_t i = 0; i < n; ++i) {
        if (!b->tuned) {
            /* one candidate per generation, timed synchronously */
            const size_t c = b->tune_ms.size();
            b->ev.params.block = b->tune_cand[c].first;
            b->ev.params.range = b->tune_cand[c].second;
            if (b->ev.size_grid()) return set_err(ctx, NRAPS_ERR_NOMEM, "batch: ranged launch buffers");
            cudaEvent_t e0, e1;
            CK(cudaEventCreate(&e0)); CK(cudaEventCreate(&e1));
            CK(cudaEventRecord(e0, sm));
            int r = b->ev.enqueue_generation(sm);
            if (r < 0) return set_err(ctx, NRAPS_ERR_CUDA, std::string("kernel launch failed: ") + cudaGetErrorString(cudaGetLastError()));
            ctx->launches += (uint64_t)r;
            CK(cudaEventRecord(e1, sm));
            CK(cudaEventSynchronize(e1));
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, e0, e1));
            cudaEventDestroy(e0); cudaEventDestroy(e1);
            GenState g;
            CK(cudaMemcpy(&g, b->ev.n_instances() == 1 ? b->buf[0]->st : b->ev.batch_stats(), sizeof g,
                          cudaMemcpyDeviceToHost));
            const unsigned long long coll = g.tot_collisions - b->tune_coll;
            b->tune_coll = g.tot_collisions;
            b->tune_ms.push_back(ms);
            b->tune_score.push_back(coll ? (double)ms / (double)coll : (double)ms);
            b->ms += ms;
            if (b->tune_ms.size() == b->tune_cand.size()) {
                size_t best = 0;
                for (size_t j = 1; j < b->tune_score.size(); ++j) if (b->tune_score[j] < b->tune_score[best]) best = j;
                b->ev.params.block = b->tune_cand[best].first;
                b->ev.params.range = b->tune_cand[best].second;
                if (b->ev.size_grid()) return set_err(ctx, NRAPS_ERR_NOMEM, "batch: ranged launch buffers");
                b->tuned = true;
            }
            b->enqueued++;
            continue;
        }
        cudaEvent_t e0, e1;
        CK(cudaEventCreate(&e0)); CK(cudaEventCreate(&e1));
        CK(cudaEventRecord(e0, sm));
        if (ctx->opts.use_graphs) {
            if (!b->gexec) {
                cudaGraph_t graph;
                CK(cudaStreamBeginCapture(sm, cudaStreamCaptureModeThreadLocal));
                int r = b->ev.enqueue_generation(sm);
                cudaError_t ce = cudaStreamEndCapture(sm, &graph);
                if (r < 0 || ce != cudaSuccess)
                    return set_err(ctx, NRAPS_ERR_CUDA, std::string("graph capture failed: ") + cudaGetErrorString(ce));
                cudaError_t ie = cudaGraphInstantiate(&b->gexec, graph, 0);
                cudaGraphDestroy(graph);
                if (ie != cudaSuccess) return set_err(ctx, NRAPS_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie));
                b->graph_kernels = (uint64_t)r;
            }
            CK(cudaGraphLaunch(b->gexec, sm));
            ctx->launches += b->graph_kernels;
        } else {
            int r = b->ev.enqueue_generation(sm);
            if (r < 0) return set_err(ctx, NRAPS_ERR_CUDA, std::string("kernel launch failed: ") + cudaGetErrorString(cudaGetLastError()));
            ctx->launches += (uint64_t)r;
        }
        CK(cudaEventRecord(e1, sm));
        b->ev_pairs.push_back(e0); b->ev_pairs.push_back(e1);
        b->enqueued++;
    }
    return NRAPS_OK;
}

int nraps_batch_sync(nraps_batch* b) {
    if (!b) return NRAPS_ERR_INVALID;
    nraps_ctx* ctx = b->ctx;
    cudaSetDevice(ctx->device);
    CK(cudaStreamSynchronize(ctx->stream));
    for (size_t i = 0; i + 1 < b->ev_pairs.size(); i += 2) {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, b->ev_pairs[i], b->ev_pairs[i + 1]));
        b->ms += ms;
        cudaEventDestroy(b->ev_pairs[i]); cudaEventDestroy(b->ev_pairs[i + 1]);
    }
    b->ev_pairs.clear();
    for (size_t i = 0; i < b->buf.size(); ++i) {
        GenState g;
        CK(cudaMemcpy(&g, b->buf[i]->st, sizeof g, cudaMemcpyDeviceToHost));
        if (g.error & NR_ERR_STALLED) return set_err(ctx, NRAPS_ERR_CUDA, "instance " + std::to_string(i) + ": a bounded device wait ran out");
        if (g.error & NR_ERR_CAPACITY) return set_err(ctx, NRAPS_ERR_CAPACITY, "instance " + std::to_string(i) + ": fission bank overflowed");
        if (g.error & NR_ERR_EMPTY) return set_err(ctx, NRAPS_ERR_EMPTY_BANK, "instance " + std::to_string(i) + ": fission bank empty");
        if (g.error & NR_ERR_CAPPED) return set_err(ctx, NRAPS_ERR_CAPPED, "instance " + std::to_string(i) + ": event cap reached");
    }
    return NRAPS_OK;
}

int nraps_batch_results(nraps_batch* b, uint32_t i, nraps_result* out) {
    if (!b || !out || i >= b->buf.size()) return set_err(b ? b->ctx : nullptr, NRAPS_ERR_INVALID, "bad batch index");
    int st = nraps_batch_sync(b);
    if (st) return st;
    uint64_t done = std::min(b->enqueued, (uint64_t)b->vars[i].generations);
    return nrint::fetch_results(b->ctx, view_of(*b->buf[i], b->vars[i], done, b->enqueued * b->n_hist[i], b->ms,
                                                b->enqueued * b->ev.launches_per_generation(), b->ctx->launches),
                                out);
}

int nraps_batch_tuning(nraps_batch* b, uint32_t* block, uint32_t* range_len, uint32_t* n_tried, float* tried_ms,
                       uint32_t tried_cap) {
    if (!b) return NRAPS_ERR_INVALID;
    if (block) *block = b->ev.params.block;
    if (range_len) *range_len = b->ev.params.range;
    if (n_tried) *n_tried = (uint32_t)b->tune_ms.size();
    for (uint32_t i = 0; tried_ms && i < tried_cap && i < b->tune_ms.size(); ++i) tried_ms[i] = b->tune_ms[i];
    return NRAPS_OK;
}

int nraps_batch_timing(nraps_batch* b, double* ms, uint64_t* histories, uint64_t* collisions) {
    if (!b) return NRAPS_ERR_INVALID;
    int st = nraps_batch_sync(b);
    if (st) return st;
    nraps_ctx* ctx = b->ctx;
    if (ms) *ms = b->ms;
    if (histories) *histories = b->enqueued * b->histories_per_gen;
    if (collisions) {
        GenState g;
        CK(cudaMemcpy(&g, b->ev.batch_stats(), sizeof g, cudaMemcpyDeviceToHost));
        *collisions = g.tot_collisions;
    }
    return NRAPS_OK;
}

uint32_t nraps_batch_size(const nraps_batch* b) { return b ? (uint32_t)b->buf.size() : 0; }

void nraps_batch_destroy(nraps_batch* b) {
    if (!b) return;
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->ctx->stream);
    delete b;
}

}  /* extern "C" */

/* ======================================================================== */
namespace {

struct Request {
    uint64_t id = 0;
    int32_t state = NRAPS_REQ_QUEUED;
    ProblemCopy prob;
    uint64_t seed = 0;
    uint64_t bytes = 0;
    std::unique_ptr<InstBuffers> buf;
    uint32_t slot = 0;
    uint64_t gens_run = 0;
    double k_mean = 0.0, k_sigma = 0.0;
    double t_submit = 0.0, t_admit = 0.0, t_done = 0.0;
    int32_t status = NRAPS_OK;
};

double now_s(const std::chrono::steady_clock::time_point& t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

/* most generations one server step runs without a host round trip */
constexpr uint64_t SERVER_MAX_STEP_GENERATIONS = 4;

}  // namespace

struct nraps_server {
    nraps_ctx* ctx = nullptr;
    nraps_server_opts o{};
    EventEngine ev;
    std::mutex mu;
    std::map<uint64_t, std::unique_ptr<Request>> reqs;
    std::deque<uint64_t> waiting;
    std::vector<uint64_t> running;       /* in event-engine instance order */
    DevMem states;                       /* GenState per slot             */
    std::vector<uint32_t> free_slots;
    std::vector<GenState> host_states;
    std::deque<uint64_t> finished;       /* retired, not yet reported by nraps_server_finished */
    uint64_t next_id = 1, bytes_in_use = 0, histories = 0, completed = 0;
    double busy_ms = 0.0;
    bool dirty = false;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
};

extern "C" {

void nraps_server_opts_default(nraps_server_opts* o) {
    if (!o) return;
    std::memset(o, 0, sizeof *o);
    o->hbm_budget_bytes = 120ULL << 30;
    o->sigma_k_target = 50e-5;
    o->min_active = 10;
    o->max_slots = 1024;
}

int nraps_server_create(nraps_ctx* ctx, const nraps_server_opts* opts, nraps_server** out) {
    if (!ctx || !out) return set_err(ctx, NRAPS_ERR_INVALID, "NULL argument");
    *out = nullptr;
    cudaSetDevice(ctx->device);
    int st = check_opts(ctx);
    if (st) return st;
    std::unique_ptr<nraps_server> s(new nraps_server());
    s->ctx = ctx;
    if (opts) s->o = *opts; else nraps_server_opts_default(&s->o);
    if (s->o.max_slots == 0 || s->o.max_slots > 4095) return set_err(ctx, NRAPS_ERR_INVALID, "max_slots must be in [1, 4095]");
    if (s->o.hbm_budget_bytes == 0) s->o.hbm_budget_bytes = 120ULL << 30;
    std::string err;
    if ((st = s->ev.configure(ctx->opts, err))) return set_err(ctx, st, err);
    if (ctx->opts.block_size == 0) s->ev.params.block = 128;
    if (ctx->opts.events_per_pass == 0 && ctx->opts.passes == 0) {
        s->ev.params.K = NRAPS_ONE_PASS; s->ev.params.passes = 0;
        s->ev.params.range = ctx->opts.range_len ? ctx->opts.range_len : 4096;
    } else if (ctx->opts.passes == 0 && s->ev.params.K != NRAPS_ONE_PASS) {
        s->ev.params.passes = 1;
    }
    /* admitted requests' buffers and tables come from the context's
       stream-ordered pool: admissions and retirements then neither call
       cudaMalloc/cudaFree nor synchronise the device */
    cudaMemPool_t pool = nrint::ctx_pool(ctx);
    if (pool) s->ev.set_pool(pool, ctx->stream);
    CK(s->states.alloc((size_t)s->o.max_slots * sizeof(GenState)));
    for (uint32_t i = s->o.max_slots; i > 0; --i) s->free_slots.push_back(i - 1);
    s->host_states.resize(s->o.max_slots);
    *out = s.release();
    return NRAPS_OK;
}

int nraps_server_submit(nraps_server* s, const nraps_problem* p, uint64_t seed, uint64_t* req_id) {
    if (!s || !p || !req_id) return set_err(s ? s->ctx : nullptr, NRAPS_ERR_INVALID, "NULL argument");
    nraps_ctx* ctx = s->ctx;
    int st = nrint::validate_problem(ctx, p, ctx->opts);
    if (st) return st;
    std::unique_ptr<Request> r(new Request());
    r->prob.take(*p);
    r->seed = seed;
    uint64_t N = p->variables.histories, G = p->variables.energygroups, nc = p->mesh.n_cells;
    double bf = ctx->opts.bank_factor > 0 ? ctx->opts.bank_factor : 3.0;
    uint64_t cap = (uint64_t)(bf * (double)N) + 1024;
    /* resident: the tally (bins spread as InstBuffers lays them out),
       flux accumulators, both banks, entropy counters, tables, plus its
       share of the per-generation queues and site slabs */
    r->bytes = ((G * nc) << ev_tally_shift(G * nc)) * 8 + G * nc * 8 * 3 + nc * 8 + 2 * cap * sizeof(nraps_site) +
               ev_hist_words(nc) * 4 +
               EventEngine::table_bytes(*p) + N * (24 * 2 + 8) + (cap + 2 * N) * 16 + p->variables.generations * 16;
    std::lock_guard<std::mutex> lk(s->mu);
    if (r->bytes > s->o.hbm_budget_bytes) {
        r->state = NRAPS_REQ_REJECTED;
        r->status = NRAPS_ERR_REJECTED;
    }
    r->id = s->next_id++;
    r->t_submit = now_s(s->t0);
    *req_id = r->id;
    bool rejected = r->state == NRAPS_REQ_REJECTED;
    if (!rejected) s->waiting.push_back(r->id);
    s->reqs[r->id] = std::move(r);
    return rejected ? set_err(ctx, NRAPS_ERR_REJECTED, "request exceeds the HBM budget") : NRAPS_OK;
}

int nraps_server_step(nraps_server* s, uint32_t* n_running, uint32_t* n_finished) {
    if (!s) return NRAPS_ERR_INVALID;
    nraps_ctx* ctx = s->ctx;
    cudaSetDevice(ctx->device);
    cudaStream_t sm = ctx->stream;
    std::lock_guard<std::mutex> lk(s->mu);
    std::string err;
    bool bank = ctx->opts.mode == NRAPS_MODE_BANK;
    /* admit in arrival order while a slot and the budget allow */
    while (!s->waiting.empty() && !s->free_slots.empty()) {
        Request& r = *s->reqs[s->waiting.front()];
        if (s->bytes_in_use + r.bytes > s->o.hbm_budget_bytes) break;
        s->waiting.pop_front();
        r.slot = s->free_slots.back();
        s->free_slots.pop_back();
        r.buf.reset(new InstBuffers());
        const nraps_problem& p = r.prob.p;
        GenState* slot_state = s->states.as<GenState>() + r.slot;
        cudaError_t e = r.buf->alloc(p.variables.energygroups, p.mesh.n_cells, p.variables.generations,
                                     p.variables.histories, ctx->opts.bank_factor, bank, (double)p.k_new,
                                     slot_state, sm, nrint::ctx_pool(ctx));
        if (e != cudaSuccess) {
            r.state = NRAPS_REQ_DONE; r.status = nrint::cuda_status(e); r.t_done = now_s(s->t0);
            s->free_slots.push_back(r.slot);
            r.buf.reset();
            continue;
        }
        if (s->ev.add_instance(p, r.buf->view(p.variables.skip, r.seed), err) < 0) {
            r.state = NRAPS_REQ_DONE; r.status = NRAPS_ERR_INVALID; r.t_done = now_s(s->t0);
            s->free_slots.push_back(r.slot);
            r.buf.reset();
            continue;
        }
        r.state = NRAPS_REQ_RUNNING;
        r.t_admit = now_s(s->t0);
        s->bytes_in_use += r.bytes;
        s->running.push_back(r.id);
        s->dirty = true;
    }
    if (n_finished) *n_finished = 0;
    if (s->running.empty()) { if (n_running) *n_running = 0; return NRAPS_OK; }
    if (s->dirty) {
        int st = s->ev.commit(sm, err);
        if (st) return set_err(ctx, st, err);
        s->dirty = false;
    }
    /* generations this step: as many as no running request could retire
       within (a request needs max(2, min_active) active generations before
       its k can count as converged, and stops at its generation cap), at
       most SERVER_MAX_STEP_GENERATIONS -- young requests then cost one host
       round trip per few generations instead of one per generation */
    uint64_t ng = SERVER_MAX_STEP_GENERATIONS;
    for (uint64_t id : s->running) {
        const Request& q = *s->reqs[id];
        const nraps_variables& v = q.prob.p.variables;
        const uint64_t first_retire = v.skip + std::max<uint32_t>(2, s->o.min_active);
        uint64_t room = first_retire > q.gens_run ? first_retire - q.gens_run : 1;
        room = std::min<uint64_t>(room, v.generations > q.gens_run ? v.generations - q.gens_run : 1);
        ng = std::min<uint64_t>(ng, std::max<uint64_t>(1, room));
    }
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0)); CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0, sm));
    for (uint64_t j = 0; j < ng; ++j) {
        int r = s->ev.enqueue_generation(sm);
        if (r < 0) { cudaEventDestroy(e0); cudaEventDestroy(e1); return set_err(ctx, NRAPS_ERR_CUDA, std::string("kernel launch failed: ") + cudaGetErrorString(cudaGetLastError())); }
        ctx->launches += (uint64_t)r;
    }
    CK(cudaEventRecord(e1, sm));
    /* only the slots up to the highest one in use (slots are handed out
       lowest first) */
    uint32_t hi_slot = 0;
    for (uint64_t id : s->running) hi_slot = std::max(hi_slot, s->reqs[id]->slot);
    CK(cudaMemcpyAsync(s->host_states.data(), s->states.p, (size_t)(hi_slot + 1) * sizeof(GenState),
                       cudaMemcpyDeviceToHost, sm));
    CK(cudaStreamSynchronize(sm));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    s->busy_ms += ms;
    /* retire converged requests (engine indices shift as they leave) */
    uint32_t fin = 0;
    double t = now_s(s->t0);
    for (size_t i = 0; i < s->running.size();) {
        Request& q = *s->reqs[s->running[i]];
        const GenState& g = s->host_states[q.slot];
        s->histories += (g.gen - std::min<uint64_t>(q.gens_run, g.gen)) * q.prob.p.variables.histories;
        q.gens_run = g.gen;
        uint64_t na = g.nactive;
        if (na) {
            q.k_mean = g.ksum / (double)na;
            double var = na > 1 ? std::max(0.0, g.ksum2 / (double)na - q.k_mean * q.k_mean) / (double)(na - 1) : 1.0;
            q.k_sigma = std::sqrt(var);
        }
        bool err_bits = g.error != 0;
        bool converged = na >= std::max<uint32_t>(2, s->o.min_active) && q.k_sigma <= s->o.sigma_k_target;
        bool capped = g.gen >= q.prob.p.variables.generations;
        if (err_bits || converged || capped) {
            q.state = NRAPS_REQ_DONE;
            q.t_done = t;
            q.status = err_bits ? ((g.error & NR_ERR_STALLED) ? NRAPS_ERR_CUDA
                                   : (g.error & NR_ERR_CAPACITY) ? NRAPS_ERR_CAPACITY
                                   : (g.error & NR_ERR_EMPTY) ? NRAPS_ERR_EMPTY_BANK : NRAPS_ERR_CAPPED)
                                : NRAPS_OK;
            s->ev.remove_instance((uint32_t)i);
            s->running.erase(s->running.begin() + i);
            s->dirty = true;
            s->completed++;
            s->finished.push_back(q.id);
            ++fin;
        } else {
            ++i;
        }
    }
    if (n_running) *n_running = (uint32_t)s->running.size();
    if (n_finished) *n_finished = fin;
    return NRAPS_OK;
}

int nraps_server_finished(nraps_server* s, uint64_t* ids, uint32_t cap, uint32_t* n) {
    if (!s || !n || (cap && !ids)) return NRAPS_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    uint32_t k = 0;
    while (k < cap && !s->finished.empty()) {
        ids[k++] = s->finished.front();
        s->finished.pop_front();
    }
    *n = k;
    return NRAPS_OK;
}

int nraps_server_poll(nraps_server* s, uint64_t req_id, nraps_result* out, nraps_request_info* info) {
    if (!s) return NRAPS_ERR_INVALID;
    nraps_ctx* ctx = s->ctx;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(req_id);
    if (it == s->reqs.end()) return set_err(ctx, NRAPS_ERR_NOT_FOUND, "unknown request id");
    Request& q = *it->second;
    if (info) {
        info->id = q.id; info->state = q.state; info->status = q.status;
        info->generations_run = q.gens_run; info->k_mean = q.k_mean; info->k_sigma = q.k_sigma;
        info->t_submit = q.t_submit; info->t_admit = q.t_admit; info->t_done = q.t_done;
        info->histories_per_generation = q.prob.p.variables.histories;
    }
    if (q.state == NRAPS_REQ_REJECTED) return set_err(ctx, NRAPS_ERR_REJECTED, "request exceeded the HBM budget");
    if (q.state != NRAPS_REQ_DONE) return NRAPS_ERR_PENDING;
    if (q.status != NRAPS_OK && q.status != NRAPS_ERR_CAPPED) return set_err(ctx, q.status, "request failed");
    if (out && q.buf) {
        cudaSetDevice(ctx->device);
        uint64_t done = std::min<uint64_t>(q.gens_run, q.prob.p.variables.generations);
        int st = nrint::fetch_results(ctx, view_of(*q.buf, q.prob.p.variables, done,
                                                   done * q.prob.p.variables.histories, 0.0, 0, ctx->launches),
                                      out);
        if (st) return st;
    }
    return q.status;
}

int nraps_server_release(nraps_server* s, uint64_t req_id) {
    if (!s) return NRAPS_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(req_id);
    if (it == s->reqs.end()) return set_err(s->ctx, NRAPS_ERR_NOT_FOUND, "unknown request id");
    Request& q = *it->second;
    if (q.state == NRAPS_REQ_RUNNING || q.state == NRAPS_REQ_QUEUED)
        return set_err(s->ctx, NRAPS_ERR_PENDING, "request still queued or running");
    if (q.buf) {
        cudaSetDevice(s->ctx->device);
        cudaStreamSynchronize(s->ctx->stream);
        s->bytes_in_use -= q.bytes;
        s->free_slots.push_back(q.slot);
    }
    s->reqs.erase(it);
    return NRAPS_OK;
}

int nraps_server_stats(nraps_server* s, uint64_t* histories, uint64_t* completed, uint32_t* running,
                       uint32_t* waiting, double* busy_ms, uint64_t* bytes_in_use) {
    if (!s) return NRAPS_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    if (histories) *histories = s->histories;
    if (completed) *completed = s->completed;
    if (running) *running = (uint32_t)s->running.size();
    if (waiting) *waiting = (uint32_t)s->waiting.size();
    if (busy_ms) *busy_ms = s->busy_ms;
    if (bytes_in_use) *bytes_in_use = s->bytes_in_use;
    return NRAPS_OK;
}

double nraps_server_clock(const nraps_server* s) { return s ? now_s(s->t0) : 0.0; }

void nraps_server_destroy(nraps_server* s) {
    if (!s) return;
    cudaSetDevice(s->ctx->device);
    cudaStreamSynchronize(s->ctx->stream);
    delete s;
}

}  /* extern "C" */
