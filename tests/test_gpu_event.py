"""Event-based Woodcock engine through the C ABI.

exact_log mode: every per-history record, the fixed-point k score and the
ordered fission bank equal the CPU restatement of the Woodcock history bit for
bit, for several (events per pass, passes, block size) shapes of the queue
machinery.  Fast mode (hardware log): results do not depend on the shape, and
agree statistically with the plain FP64 kernel (k within 3 sigma, flux chi^2
per group on independent generations).
"""
import numpy as np
import pytest
from scipy import stats as sps

from nraps_gb300 import abi, api, synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SHAPES = [dict(events_per_pass=1, passes=4, block_size=128),
          dict(events_per_pass=4, passes=2, block_size=256),
          dict(events_per_pass=16, passes=1, block_size=256),
          dict(events_per_pass=abi.ONE_PASS, passes=0, block_size=256),
          dict(events_per_pass=abi.ONE_PASS, passes=1, block_size=128, tail_lanes=12)]


def small(hist=3000, gens=12, skip=4, seed=3):
    return synth.plain_small(seed).with_(histories=hist, generations=gens, skip=skip)


def _records_equal(g, w):
    for f in ("collisions", "crossings", "fate", "final_cell", "final_group", "n_sites", "draws"):
        bad = np.nonzero(g[f] != w[f])[0]
        assert bad.size == 0, (f, bad[:5], g[f][bad[:5]], w[f][bad[:5]])
    for f in ("final_x", "track", "nsf_track"):
        bad = np.nonzero(g[f].view(np.int64) != w[f].view(np.int64))[0]
        assert bad.size == 0, (f, bad[:5], g[f][bad[:5]], w[f][bad[:5]])


@pytest.mark.parametrize("shape", SHAPES, ids=["K1P4b128", "K4P2b256", "K16P1b256", "onepass256", "tail12b128"])
@pytest.mark.parametrize("mode", [abi.MODE_PHYSICS, abi.MODE_BANK])
def test_event_trace_bitexact(ctx_factory, mode, shape):
    p = small()
    opts = dict(seed=41, mode=mode, precision=abi.PREC_FP32, tracking=abi.TRACK_WOODCOCK, exact_log=1, **shape)
    o = abi.make_opts(**opts)
    ctx = ctx_factory(**opts)
    sites_in = None
    gen = 2
    if mode == abi.MODE_BANK:
        _, _, sites_in, _ = O.trace_woodcock(p, o, 0, 1.0)
        gen = 1
    grec, gt, gs, gkq = ctx.trace(p, gen, 0.95, sites_in=sites_in)
    wrec, wt, ws, wkq = O.trace_woodcock(p, o, gen, 0.95, sites_in=sites_in)
    _records_equal(grec, wrec)
    assert gkq == wkq
    np.testing.assert_allclose(gt, wt, rtol=1e-12, atol=0)
    if mode == abi.MODE_BANK:
        assert len(gs) == len(ws) and np.array_equal(gs, ws)


def test_event_reflective_bitexact(ctx_factory):
    import os
    from .conftest import GOLDEN
    inp = api.process_input(os.path.join(GOLDEN, "inputs", "TestCaseC.txt"))
    mesh, fuel = api.mesh_gen(inp.matid, inp.variables, inp.delta_x)
    p = api.problem_from_input(inp, mesh, fuel).with_(histories=2000, generations=3, skip=1)
    opts = dict(seed=5, mode=abi.MODE_PHYSICS, precision=abi.PREC_FP32, tracking=abi.TRACK_WOODCOCK, exact_log=1)
    grec, gt, _, gkq = ctx_factory(**opts).trace(p, 0, 1.0)
    wrec, wt, _, wkq = O.trace_woodcock(p, abi.make_opts(**opts), 0, 1.0)
    _records_equal(grec, wrec)
    assert gkq == wkq and np.all(grec["fate"] != abi.FATE_LEAKED)


# sorted transport (event-type queues, one instance) and ranged launches
SORT_SHAPES = [dict(sort_rounds=1), dict(sort_rounds=8), dict(range_len=64), dict(range_len=1024)]


def test_event_results_independent_of_queue_shape(ctx_factory):
    p = small(hist=20000, gens=10, skip=3)
    ks = []
    for shape in SHAPES + SORT_SHAPES:
        r = ctx_factory(seed=7, mode=abi.MODE_BANK, precision=abi.PREC_FP32,
                        tracking=abi.TRACK_WOODCOCK, **shape).solve(p)
        ks.append(r.k64)
    assert all(np.array_equal(ks[0], k) for k in ks[1:])


def test_event_graph_replay_equals_direct(ctx_factory):
    p = small(hist=20000, gens=10, skip=3)
    base = dict(seed=9, mode=abi.MODE_BANK, precision=abi.PREC_FP32, tracking=abi.TRACK_WOODCOCK)
    a = ctx_factory(use_graphs=1, **base).solve(p)
    b = ctx_factory(use_graphs=0, **base).solve(p)
    assert np.array_equal(a.k64, b.k64)
    np.testing.assert_allclose(a.flux_mean, b.flux_mean, rtol=1e-11, atol=0)
    np.testing.assert_allclose(a.entropy, b.entropy, rtol=0, atol=1e-12)


def test_event_k_agrees_with_plain_fp64_bank(ctx_factory):
    # same seeds, same physics, different tracking and precision
    p = small(hist=40000, gens=60, skip=20)
    ev = ctx_factory(seed=11, mode=abi.MODE_BANK, precision=abi.PREC_FP32, tracking=abi.TRACK_WOODCOCK).solve(p)
    pl = ctx_factory(seed=11, mode=abi.MODE_BANK, precision=abi.PREC_FP64).solve(p)
    d = abs(ev.stats.k_mean - pl.stats.k_mean)
    # generations of a power iteration are correlated: inflate sigma by 2
    sig = 2.0 * np.hypot(ev.stats.k_sigma, pl.stats.k_sigma)
    assert d < 3 * sig, (ev.stats.k_mean, pl.stats.k_mean, sig)
    assert ev.stats.virtual_collisions > 0 and ev.stats.crossings == 0


def test_event_flux_chi2_against_plain_fp64(ctx_factory):
    # PHYSICS mode: every generation restarts from the fresh source, so
    # generations are independent and the per-bin standard errors are valid
    p = small(hist=40000, gens=40, skip=2)
    ev = ctx_factory(seed=13, mode=abi.MODE_PHYSICS, precision=abi.PREC_FP32, tracking=abi.TRACK_WOODCOCK).solve(p)
    pl = ctx_factory(seed=13, mode=abi.MODE_PHYSICS, precision=abi.PREC_FP64).solve(p)
    G, nc = p.energygroups, p.n_cells
    m1, s1 = ev.flux_mean.reshape(G, nc), ev.flux_sem.reshape(G, nc)
    m2, s2 = pl.flux_mean.reshape(G, nc), pl.flux_sem.reshape(G, nc)
    for g in range(G):
        ok = (s1[g] > 0) & (s2[g] > 0)
        chi2 = float((((m1[g] - m2[g]) ** 2) / (s1[g] ** 2 + s2[g] ** 2))[ok].sum())
        dof = int(ok.sum())
        pval = sps.chi2.sf(chi2, dof)
        assert pval > 1e-4, (g, chi2, dof, pval)
    assert abs(ev.stats.k_mean - pl.stats.k_mean) < 3 * np.hypot(ev.stats.k_sigma, pl.stats.k_sigma)


def test_event_fast_log_matches_exact_log(ctx_factory):
    p = small(hist=20000, gens=10, skip=3)
    base = dict(seed=17, mode=abi.MODE_BANK, precision=abi.PREC_FP32, tracking=abi.TRACK_WOODCOCK)
    fast = ctx_factory(exact_log=0, **base).solve(p)
    exact = ctx_factory(exact_log=1, **base).solve(p)
    assert abs(fast.stats.k_mean - exact.stats.k_mean) < 3 * 2 * np.hypot(fast.stats.k_sigma, exact.stats.k_sigma)


def test_event_bank_overflow_is_reported(ctx_factory):
    p = small(hist=5000, gens=4, skip=1)
    ctx = ctx_factory(seed=3, mode=abi.MODE_BANK, precision=abi.PREC_FP32, tracking=abi.TRACK_WOODCOCK,
                      bank_factor=0.01)
    with pytest.raises(api.NrapsError) as e:
        ctx.solve(p)
    assert e.value.status == abi.ERR_CAPACITY


def test_ranged_bank_overflow_is_reported(ctx_factory):
    """Ranged launches append sites to chunks of a pool sized by the bank
    capacity: a bank that cannot hold the generation's sites is reported
    the same way."""
    p = small(hist=5000, gens=4, skip=1)
    ctx = ctx_factory(seed=3, mode=abi.MODE_BANK, precision=abi.PREC_FP32, tracking=abi.TRACK_WOODCOCK,
                      bank_factor=0.01, range_len=1024)
    with pytest.raises(api.NrapsError) as e:
        ctx.solve(p)
    assert e.value.status == abi.ERR_CAPACITY


def test_autotuner_leaves_results_unchanged(ctx_factory):
    p = small(hist=20000, gens=16, skip=12)
    base = dict(seed=21, mode=abi.MODE_BANK, precision=abi.PREC_FP32, tracking=abi.TRACK_WOODCOCK)
    ctx = ctx_factory(**base)                      # shape left to the tuner
    s = ctx.session(p)
    s.run(p.generations)
    r = s.results()
    t = s.tuning()
    s.close()
    fixed = ctx_factory(events_per_pass=4, passes=3, block_size=256, **base).solve(p)
    assert np.array_equal(r.k64, fixed.k64)
    # shapes that close a generation in the scatter and fold it in the next
    # transport launch alternate with shapes that finalize in their own launch
    np.testing.assert_allclose(r.flux_mean, fixed.flux_mean, rtol=1e-11, atol=0)
    np.testing.assert_allclose(r.fission_source, fixed.fission_source, rtol=1e-6, atol=0)
    np.testing.assert_allclose(r.entropy, fixed.entropy, rtol=0, atol=1e-12)
    assert len(t["tried_ms"]) == 12 and min(t["tried_ms"]) > 0
    assert t["block"] in (128, 256) and t["events_per_pass"] >= 1
    # one-pass shapes run every particle to its end (no queue passes)
    assert t["passes"] >= 1 or t["events_per_pass"] == abi.ONE_PASS


@pytest.mark.parametrize("mode", [abi.MODE_PHYSICS, abi.MODE_BANK])
def test_sorted_transport_exact_log_matches(ctx_factory, mode):
    """The sorted transport (flight and collision kernels over event-type
    queues, then one pass for the survivors) against the warp transport with
    the shared software logarithm: every history identical, so k, tallies and
    bank order (entropy) agree exactly; 2R+1 transport launches per
    generation."""
    p = small(hist=7000, gens=8, skip=3)
    base = dict(seed=77, mode=mode, precision=abi.PREC_FP32, tracking=abi.TRACK_WOODCOCK, exact_log=1)
    warp = ctx_factory(block_size=128, events_per_pass=abi.ONE_PASS, passes=0, **base).solve(p)
    for rounds in (1, 4, 16):
        srt = ctx_factory(sort_rounds=rounds, **base).solve(p)
        assert np.array_equal(srt.k64, warp.k64), rounds
        np.testing.assert_allclose(srt.flux_mean, warp.flux_mean, rtol=1e-12, atol=0)
        np.testing.assert_allclose(srt.entropy, warp.entropy, rtol=0, atol=1e-12)
        assert srt.stats.collisions == warp.stats.collisions
        assert srt.stats.virtual_collisions == warp.stats.virtual_collisions
        assert srt.stats.transport_launches == p.generations * (2 * rounds + 1)


def test_sort_rounds_validated(ctx_factory):
    p = small(hist=1000, gens=3, skip=1)
    with pytest.raises(api.NrapsError) as e:
        ctx_factory(seed=1, mode=abi.MODE_BANK, precision=abi.PREC_FP32, tracking=abi.TRACK_WOODCOCK,
                    sort_rounds=17).solve(p)
    assert e.value.status == abi.ERR_INVALID


@pytest.mark.parametrize("tracking", [abi.TRACK_WOODCOCK, abi.TRACK_SURFACE])
def test_diffusion_initial_source(ctx_factory, tracking):
    """Generation 0 from the diffusion fission source: the first generations
    differ from the uniform-fuel start, the two runs' entropies approach each
    other (one converged source), and the diffusion start is reproducible."""
    p = synth.single_large(2).with_(histories=20000, generations=30, skip=10)
    prec = abi.PREC_FP32 if tracking == abi.TRACK_WOODCOCK else abi.PREC_FP64
    base = dict(seed=5, mode=abi.MODE_BANK, precision=prec, tracking=tracking)
    uni = ctx_factory(**base).solve(p)
    dif = ctx_factory(initial_source=1, **base).solve(p)
    dif2 = ctx_factory(initial_source=1, **base).solve(p)
    assert np.array_equal(dif.k64, dif2.k64)
    assert dif.entropy[0] != uni.entropy[0] and not np.array_equal(dif.k64[:3], uni.k64[:3])
    # the two starts approach one converged source from either side
    gap0 = abs(dif.entropy[0] - uni.entropy[0])
    assert abs(dif.entropy[-5:].mean() - uni.entropy[-5:].mean()) < 0.6 * gap0
    with pytest.raises(api.NrapsError):
        ctx_factory(seed=5, mode=abi.MODE_PHYSICS, precision=prec, tracking=tracking, initial_source=1).solve(p)


@pytest.mark.parametrize("mode", [abi.MODE_PHYSICS, abi.MODE_BANK])
def test_ranged_launch_exact_log_matches(ctx_factory, mode):
    """Ranged launches (one block per range of one instance, the tables in
    shared memory) against the persistent warp transport with the shared
    logarithm: identical histories, so identical k, tallies and bank order
    (BANK: each range orders its own sites)."""
    p = small(hist=7000, gens=8, skip=3)
    base = dict(seed=78, mode=mode, precision=abi.PREC_FP32, tracking=abi.TRACK_WOODCOCK, exact_log=1)
    warp = ctx_factory(block_size=256, events_per_pass=abi.ONE_PASS, passes=0, **base).solve(p)
    for rl, block in ((64, 128), (1000, 256), (8192, 128), (32768, 256)):
        r = ctx_factory(range_len=rl, block_size=block, **base).solve(p)
        assert np.array_equal(r.k64, warp.k64), rl
        np.testing.assert_allclose(r.flux_mean, warp.flux_mean, rtol=1e-12, atol=0)
        np.testing.assert_allclose(r.entropy, warp.entropy, rtol=0, atol=1e-12)
        assert r.stats.collisions == warp.stats.collisions
    with pytest.raises(api.NrapsError) as e:
        ctx_factory(range_len=32769, **base).solve(p)
    assert e.value.status == abi.ERR_INVALID


def test_tuner_choice_cached_per_shape(ctx_factory):
    """A second session of the same problem shape on one context starts with
    the first session's choice and tries nothing; results are unchanged."""
    p = small(hist=20000, gens=14, skip=12)
    ctx = ctx_factory(seed=23, mode=abi.MODE_BANK, precision=abi.PREC_FP32, tracking=abi.TRACK_WOODCOCK)
    s1 = ctx.session(p)
    s1.run(p.generations)
    r1, t1 = s1.results(), s1.tuning()
    s1.close()
    s2 = ctx.session(p)
    s2.run(p.generations)
    r2, t2 = s2.results(), s2.tuning()
    s2.close()
    assert len(t1["tried_ms"]) == 12 and len(t2["tried_ms"]) == 0
    for key in ("block", "events_per_pass", "passes", "tail_lanes", "sort_rounds", "range_len"):
        assert t1[key] == t2[key], key
    assert np.array_equal(r1.k64, r2.k64)


# deferred end of generation: one pass, one instance, few cells (the scatter's
# last block closes a generation, the next transport launch folds it)
DEFERRED = dict(events_per_pass=abi.ONE_PASS, passes=0, block_size=128)
CLASSIC = dict(events_per_pass=4, passes=2, block_size=256)


def _same_results(a, b, gens):
    # k is exact; flux sums FP64 tallies whose atomic order varies from run to run
    assert np.array_equal(a.k64, b.k64)
    for f in ("flux_mean", "flux_sem"):
        np.testing.assert_allclose(getattr(a, f), getattr(b, f), rtol=1e-11, atol=0, err_msg=f)
    np.testing.assert_allclose(a.flux, b.flux, rtol=1e-6, atol=0)
    np.testing.assert_allclose(a.fission_source, b.fission_source, rtol=1e-6, atol=0)
    np.testing.assert_allclose(a.entropy[:gens], b.entropy[:gens], rtol=0, atol=1e-12)
    assert np.all(a.entropy[:gens] > 0)


def test_deferred_fold_matches_classic_finalize(ctx_factory):
    p = small(hist=20000, gens=12, skip=4)
    base = dict(seed=23, mode=abi.MODE_BANK, precision=abi.PREC_FP32, tracking=abi.TRACK_WOODCOCK)
    d = ctx_factory(**DEFERRED, **base).solve(p)
    c = ctx_factory(**CLASSIC, **base).solve(p)
    _same_results(d, c, p.generations)


def test_deferred_fold_split_runs(ctx_factory):
    """Reading results between runs completes the pending fold; later runs
    carry on as if never interrupted (also through a classic-shape session
    on the same context)."""
    p = small(hist=20000, gens=14, skip=4)
    base = dict(seed=29, mode=abi.MODE_BANK, precision=abi.PREC_FP32, tracking=abi.TRACK_WOODCOCK)
    ctx = ctx_factory(**DEFERRED, **base)
    s = ctx.session(p)
    s.run(5)
    mid = s.results()
    s.run(3)
    s.flush()
    s.run(p.generations - 8)
    r = s.results()
    s.close()
    whole = ctx_factory(**DEFERRED, **base).solve(p)
    _same_results(r, whole, p.generations)
    assert np.array_equal(mid.k64[:5], whole.k64[:5]) and np.all(mid.k64[5:] == 0)
    np.testing.assert_allclose(mid.entropy[:5], whole.entropy[:5], rtol=0, atol=1e-12)
    assert np.all(mid.entropy[5:] == 0)
