"""CUDA plain kernel against the CPU oracle, through the C ABI.

Bit-exact: PCG32 streams, the shared logarithm, every per-history record
(collision/crossing counts, fate, final cell/group, final position, summed
track length and k score), the fixed-point k score and the ordered fission
bank.  Tallies are FP64 atomics whose summation order differs from the CPU's:
they are compared with rtol 1e-12.
"""
import numpy as np
import pytest

from nraps_gb300 import abi, api, synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

MODES = [(abi.MODE_COMPAT, abi.PREC_FP32), (abi.MODE_COMPAT, abi.PREC_FP64),
         (abi.MODE_PHYSICS, abi.PREC_FP32), (abi.MODE_PHYSICS, abi.PREC_FP64),
         (abi.MODE_BANK, abi.PREC_FP32), (abi.MODE_BANK, abi.PREC_FP64)]


def small(hist=2000, gens=12, skip=4, seed=3):
    return synth.plain_small(seed).with_(histories=hist, generations=gens, skip=skip)


def test_pcg32_stream_bitexact(ctx_factory):
    ctx = ctx_factory()
    streams = np.array([0, 1, 54, 12345, (1 << 40) + 3], np.uint64)
    for seed in (42, 7, 0xDEADBEEFCAFEBABE):
        got = ctx.pcg32(seed, streams, 64)
        for i, s in enumerate(streams):
            assert np.array_equal(got[i], O.pcg32(seed, int(s), 64))
    assert [int(v) for v in ctx.pcg32(42, [54], 6)[0]] == \
        [0xa15c02b7, 0x7b47f409, 0xba1d3330, 0x83d2f293, 0xbfa4784b, 0xcbed606e]


def test_shared_log_bitexact(ctx_factory):
    ctx = ctx_factory()
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.random(50000) + 1e-15, np.exp(rng.uniform(-700, 700, 5000)),
                        [1.0, 0.5, 2.0, 5e-324, 1e-310, 0.0, -1.0]])
    g64, g32 = ctx.log_eval(x)
    w64 = np.array([O.log64(float(v)) for v in x])
    w32 = np.array([O.log32(np.float32(v)) for v in x], np.float32)
    assert np.array_equal(g64.view(np.int64), w64.view(np.int64))
    assert np.array_equal(g32.view(np.int32), w32.view(np.int32))


def _compare_records(g, w):
    for f in ("collisions", "crossings", "reflections", "segments", "fate", "final_cell",
              "final_group", "n_sites", "draws"):
        bad = np.nonzero(g[f] != w[f])[0]
        assert bad.size == 0, (f, bad[:5], g[f][bad[:5]], w[f][bad[:5]])
    for f in ("final_x", "track", "nsf_track"):
        gb, wb = g[f].view(np.int64), w[f].view(np.int64)
        bad = np.nonzero(gb != wb)[0]
        assert bad.size == 0, (f, bad[:5], g[f][bad[:5]], w[f][bad[:5]])


@pytest.mark.parametrize("mode,prec", MODES)
def test_trace_generation_bitexact(ctx_factory, mode, prec):
    p = small()
    opts = dict(seed=17, mode=mode, precision=prec, compat_threads=7 if mode == abi.MODE_COMPAT else 0)
    ctx = ctx_factory(**opts)
    o = abi.make_opts(**opts)
    sites_in = None
    if mode == abi.MODE_BANK:
        # a generation-0 bank from the oracle feeds generation 1 on both sides
        _, _, sites_in, _ = O.trace_generation(p, o, 0, 1.0)
        assert len(sites_in) > 0
    gen = 1 if mode == abi.MODE_BANK else 3
    grec, gtally, gsites, gkq = ctx.trace(p, gen, 0.97, sites_in=sites_in)
    wrec, wtally, wsites, wkq = O.trace_generation(p, o, gen, 0.97, sites_in=sites_in)
    assert len(grec) == len(wrec) == p.histories + opts["compat_threads"]
    _compare_records(grec, wrec)
    np.testing.assert_allclose(gtally, wtally, rtol=1e-12, atol=0)
    if mode != abi.MODE_COMPAT:
        assert gkq == wkq
    if mode == abi.MODE_BANK:
        assert len(gsites) == len(wsites) == int(wrec["n_sites"].sum())
        assert np.array_equal(gsites, wsites)


def test_bank_solve_fp64_matches_oracle(ctx_factory):
    p = small()
    opts = dict(seed=23, mode=abi.MODE_BANK, precision=abi.PREC_FP64)
    g = ctx_factory(**opts).solve(p)
    w = O.monte_carlo(p, abi.make_opts(**opts), threads=4)
    # fixed-point k and deterministic bank order: identical k every generation
    assert np.array_equal(g.k64, w.k64)
    np.testing.assert_allclose(g.entropy, w.entropy, rtol=0, atol=1e-12)
    np.testing.assert_allclose(g.flux, w.flux, rtol=2e-6, atol=0)
    np.testing.assert_allclose(g.fission_source, w.fission_source, rtol=2e-6, atol=1e-30)
    assert g.stats.collisions > 0 and g.stats.histories == p.histories * p.generations


def test_compat_solve_matches_reference_f32_arithmetic(ctx_factory):
    # COMPAT FP32 is the reference's arithmetic; the GPU accumulates tallies in
    # FP64, the oracle both in f32 (as the reference) and in FP64
    p = small(hist=3000, gens=6, skip=2)
    opts = dict(seed=31, mode=abi.MODE_COMPAT, precision=abi.PREC_FP32, compat_threads=7)
    g = ctx_factory(**opts).solve(p)
    w64 = O.monte_carlo(p, abi.make_opts(**opts), threads=7, acc64=True)
    w32 = O.monte_carlo(p, abi.make_opts(**opts), threads=7, acc64=False)
    # the oracle finalizes in f32 as the reference does (k summed over 2000
    # bins in f32): 2e-5 relative; the GPU sums in FP64
    np.testing.assert_allclose(g.k, w64.k, rtol=2e-5)
    np.testing.assert_allclose(g.k, w32.k, rtol=1e-3)
    np.testing.assert_allclose(g.k_fund[2:], w64.k_fund[2:], rtol=2e-5)
    np.testing.assert_allclose(g.flux, w64.flux, rtol=1e-5)
    np.testing.assert_allclose(g.assembly_average, w64.assembly_average, rtol=1e-5)


def test_monte_carlo_call_equals_solve(ctx_factory):
    p = small(hist=1000, gens=5, skip=1)
    ctx = ctx_factory(seed=5, mode=abi.MODE_PHYSICS, precision=abi.PREC_FP64)
    a = ctx.monte_carlo(p)
    b = ctx.solve(p)
    assert np.array_equal(a.k64, b.k64)


def test_graph_replay_equals_direct_launches(ctx_factory):
    p = small(hist=2000, gens=10, skip=3)
    a = ctx_factory(seed=8, mode=abi.MODE_BANK, precision=abi.PREC_FP64, use_graphs=1).solve(p)
    b = ctx_factory(seed=8, mode=abi.MODE_BANK, precision=abi.PREC_FP64, use_graphs=0).solve(p)
    assert np.array_equal(a.k64, b.k64)


def test_session_runs_in_pieces(ctx_factory):
    p = small(hist=1500, gens=12, skip=3)
    ctx = ctx_factory(seed=4, mode=abi.MODE_BANK, precision=abi.PREC_FP64)
    s = ctx.session(p)
    s.run(5)
    s.sync()
    s.run(7)
    r = s.results()
    s.close()
    assert np.array_equal(r.k64, ctx.solve(p).k64)


def test_reflective_testcase_c(ctx_factory):
    import os
    from .conftest import GOLDEN
    inp = api.process_input(os.path.join(GOLDEN, "inputs", "TestCaseC.txt"))
    mesh, fuel = api.mesh_gen(inp.matid, inp.variables, inp.delta_x)
    p = api.problem_from_input(inp, mesh, fuel).with_(histories=2000, generations=3, skip=1)
    opts = dict(seed=3, mode=abi.MODE_COMPAT, precision=abi.PREC_FP32, compat_threads=7)
    ctx = ctx_factory(**opts)
    rec, _, _, _ = ctx.trace(p, 0, 1.0)
    wrec, _, _, _ = O.trace_generation(p, abi.make_opts(**opts), 0, 1.0)
    _compare_records(rec, wrec)
    assert rec["reflections"].sum() > 0 and np.all(rec["fate"] != abi.FATE_LEAKED)


def test_errors_are_status_codes(ctx_factory):
    p = small(hist=100, gens=4, skip=1)
    ctx = ctx_factory(seed=1, mode=abi.MODE_PHYSICS)
    with pytest.raises(api.NrapsError) as e:
        ctx.solve(p.with_(skip=4))
    assert e.value.status == abi.ERR_INVALID
    with pytest.raises(api.NrapsError) as e:
        ctx.solve(p.with_(fuel_indices=np.zeros(0, np.uint64)))
    assert e.value.status == abi.ERR_INVALID
    capped = ctx_factory(seed=1, mode=abi.MODE_PHYSICS, max_events=3)
    with pytest.raises(api.NrapsError) as e:
        capped.solve(p)
    assert e.value.status == abi.ERR_CAPPED
    bad = ctx_factory(seed=1, mode=abi.MODE_COMPAT, tracking=abi.TRACK_WOODCOCK)
    with pytest.raises(api.NrapsError) as e:
        bad.solve(p)
    assert e.value.status == abi.ERR_INVALID
    # the context is still usable after every error
    r = ctx.solve(p)
    assert np.all(np.isfinite(r.k64))
