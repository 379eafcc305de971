"""Batched instances and the request server (continuous batching).

Every particle owns a PCG32 stream of its instance's seed and k is summed
exactly, so an instance's k in every generation is the same bits whether it
runs alone, in a batch, or in a server whose other requests come and go.
Tallies are FP64 atomics (summation order differs): rtol 1e-9.
"""
import numpy as np
import pytest

from nraps_gb300 import abi, api, synth

pytestmark = pytest.mark.gpu

WC = dict(mode=abi.MODE_BANK, precision=abi.PREC_FP32, tracking=abi.TRACK_WOODCOCK)


def instances(n, seed=5, inactive=4, active=6):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        R = int(rng.integers(4, 12))
        G = int(rng.integers(2, 6))
        N = int(rng.integers(2000, 8000))
        out.append(synth.random_slab(rng, R, G, 0.5, 3.0, 10, N, inactive, active))
    return out


def test_many_small_instances_equal_alone(ctx_factory):
    """Many small instances whose sizes are not multiples of the 64-particle
    claim: nearly every chunk a warp takes spans two instances, so a lane
    prefetches records of one instance while flying a particle of another."""
    rng = np.random.default_rng(11)
    probs = []
    for _ in range(24):
        R = int(rng.integers(3, 10))
        G = int(rng.integers(2, 7))
        N = int(rng.integers(300, 1500))
        probs.append(synth.random_slab(rng, R, G, 0.5, 3.0, 10, N, 3, 4))
    seeds = [500 + i for i in range(len(probs))]
    ctx = ctx_factory(seed=1, **WC)
    b = api.Batch(ctx, probs, seeds=seeds)
    b.run(probs[0].generations)
    for i, p in enumerate(probs):
        r = b.results(i)
        alone = ctx_factory(seed=seeds[i], **WC).solve(p)
        assert np.array_equal(r.k64, alone.k64), i
        np.testing.assert_allclose(r.entropy, alone.entropy, rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(r.flux_mean, alone.flux_mean, rtol=1e-9, atol=0)
    b.close()


def test_more_instances_than_the_scatter_table(ctx_factory):
    """1,600 instances: more than the bank scatter stages in shared memory
    (1,536), so sites find their instance's bank through its descriptor;
    sampled instances equal the same instance run alone, bank (through k of
    the later generations) and site histogram (entropy) included."""
    rng = np.random.default_rng(5)
    probs = []
    for _ in range(1600):
        R = int(rng.integers(2, 6))
        G = int(rng.integers(2, 4))
        N = int(rng.integers(40, 200))
        probs.append(synth.random_slab(rng, R, G, 0.5, 3.0, 4, N, 3, 1))
    seeds = [9000 + i for i in range(len(probs))]
    ctx = ctx_factory(seed=1, **WC)
    b = api.Batch(ctx, probs, seeds=seeds)
    b.run(probs[0].generations)
    for i in range(0, len(probs), 97):
        r = b.results(i)
        alone = ctx_factory(seed=seeds[i], **WC).solve(probs[i])
        assert np.array_equal(r.k64, alone.k64), i
        np.testing.assert_allclose(r.entropy, alone.entropy, rtol=1e-12, atol=1e-12)
    b.close()


def test_batch_equals_each_instance_alone(ctx_factory):
    probs = instances(5)
    seeds = [101 + i for i in range(len(probs))]
    ctx = ctx_factory(seed=1, use_graphs=1, **WC)
    b = api.Batch(ctx, probs, seeds=seeds)
    b.run(probs[0].generations)
    for i, p in enumerate(probs):
        r = b.results(i)
        alone = ctx_factory(seed=seeds[i], **WC).solve(p)
        assert np.array_equal(r.k64, alone.k64), i
        np.testing.assert_allclose(r.entropy, alone.entropy, rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(r.flux_mean, alone.flux_mean, rtol=1e-9, atol=0)
    t = b.timing()
    assert t["histories"] == sum(p.histories for p in probs) * probs[0].generations and t["ms"] > 0
    b.close()


def _run_until_done(srv, rid, max_steps=500):
    for _ in range(max_steps):
        st, info, res = srv.poll(rid)
        if st != abi.ERR_PENDING:
            return st, info, res
        srv.step()
    raise AssertionError("request did not finish")


def test_server_result_same_alone_and_in_the_mix(ctx_factory):
    pool = instances(6, seed=9, inactive=4, active=60)
    A = pool[0]
    ctx = ctx_factory(seed=1, **WC)
    alone = api.Server(ctx, sigma_k_target=4e-3, min_active=5)
    ra = alone.submit(A, 777)
    st_a, info_a, res_a = _run_until_done(alone, ra)
    alone.close()
    mix = api.Server(ctx, sigma_k_target=4e-3, min_active=5)
    others = [mix.submit(pool[1], 1), mix.submit(pool[2], 2)]
    mix.step()
    mix.step()
    rm = mix.submit(A, 777)                 # arrives while others run
    mix.step()
    others.append(mix.submit(pool[3], 3))   # arrives while A runs
    others.append(mix.submit(pool[4], 4))
    st_m, info_m, res_m = _run_until_done(mix, rm)
    assert st_a == st_m == abi.OK
    assert info_a["generations_run"] == info_m["generations_run"]
    assert info_a["k_mean"] == info_m["k_mean"] and info_a["k_sigma"] == info_m["k_sigma"]
    assert np.array_equal(res_a.k64, res_m.k64)
    np.testing.assert_allclose(res_a.flux_mean, res_m.flux_mean, rtol=1e-9, atol=0)
    assert info_m["k_sigma"] <= 4e-3
    for rid in others:
        _run_until_done(mix, rid)
    s = mix.stats()
    assert s["completed"] == 5 and s["running"] == 0
    mix.close()


def test_server_budget(ctx_factory):
    p = instances(1, seed=3)[0]
    ctx = ctx_factory(seed=1, **WC)
    tiny = api.Server(ctx, hbm_budget_bytes=1 << 16)
    with pytest.raises(api.NrapsError) as e:
        tiny.submit(p, 1)
    assert e.value.status == abi.ERR_REJECTED
    tiny.close()
    # a budget that holds one request at a time: the second waits for the first's release
    probe = api.Server(ctx)
    rid = probe.submit(p, 1)
    probe.step()
    one = probe.stats()["bytes_in_use"]
    probe.close()
    srv = api.Server(ctx, hbm_budget_bytes=int(one * 1.5), sigma_k_target=1.0, min_active=2)
    r1, r2 = srv.submit(p, 1), srv.submit(p, 2)
    srv.step()
    s = srv.stats()
    assert s["running"] == 1 and s["waiting"] == 1
    _run_until_done(srv, r1)
    srv.release(r1)
    srv.step()
    assert srv.stats()["running"] + srv.stats()["completed"] >= 1
    st, info, _ = _run_until_done(srv, r2)
    assert st == abi.OK
    srv.close()


def test_server_finished_ids(ctx_factory):
    """nraps_server_finished reports each retired request once, in order."""
    probs = instances(3, seed=9)
    ctx = ctx_factory(seed=1, **WC)
    srv = api.Server(ctx, sigma_k_target=1.0, min_active=2)
    ids = [srv.submit(p, 10 + i) for i, p in enumerate(probs)]
    seen = []
    for _ in range(200):
        srv.step()
        seen += srv.finished()
        if len(seen) == len(ids):
            break
    assert sorted(seen) == sorted(ids) and len(set(seen)) == len(seen)
    assert srv.finished() == []
    for rid in seen:
        st, info, _ = srv.poll(rid, results=False)
        assert st == abi.OK and info["generations_run"] >= 2
    srv.close()


def test_batch_autotuner_tries_shapes_without_changing_results(ctx_factory):
    """A batch given no launch shape tries blocks of 128/256/512 threads with
    ranges of 1024..8192 histories over its first inactive generations; every
    instance's k sequence equals that of the same batch run at one fixed
    shape, and the choice is one of the candidates."""
    probs = instances(5, seed=13, inactive=12, active=4)
    seeds = [900 + i for i in range(len(probs))]
    tuned = api.Batch(ctx_factory(seed=1, **WC), probs, seeds=seeds)
    tuned.run(probs[0].generations)
    t = tuned.tuning()
    fixed = api.Batch(ctx_factory(seed=1, block_size=512, range_len=2048, **WC), probs, seeds=seeds)
    fixed.run(probs[0].generations)
    assert len(t["tried_ms"]) == 12 and min(t["tried_ms"]) > 0
    assert t["block"] in (128, 256, 512) and t["range_len"] in (1024, 2048, 4096, 8192)
    assert fixed.tuning()["tried_ms"] == [] and fixed.tuning()["block"] == 512
    for i in range(len(probs)):
        assert np.array_equal(tuned.results(i).k64, fixed.results(i).k64), i
    tuned.close()
    fixed.close()
