"""Edge cases of the event transport against the CPU restatement, in the
exact-log mode where every history is bit-comparable: populations smaller
than a warp or straddling the 64-particle claims, the largest group count,
meshes past the shared-memory site histogram, tables past shared memory,
and several generations chained through the ordered fission bank."""
from __future__ import annotations

import numpy as np
import pytest

from nraps_gb300 import abi, api, synth
from oracle import oracle as O

from .test_gpu_event import _records_equal

pytestmark = pytest.mark.gpu

EXACT = dict(precision=abi.PREC_FP32, tracking=abi.TRACK_WOODCOCK, exact_log=1)


@pytest.mark.parametrize("n", [1, 31, 65, 129])
@pytest.mark.parametrize("mode", [abi.MODE_PHYSICS, abi.MODE_BANK])
def test_tiny_populations(ctx_factory, mode, n):
    p = synth.plain_small(4).with_(histories=n, generations=3, skip=1)
    opts = dict(seed=9, mode=mode, **EXACT)
    ctx = ctx_factory(**opts)
    grec, gt, gs, gkq = ctx.trace(p, 1, 1.02)
    wrec, wt, ws, wkq = O.trace_woodcock(p, abi.make_opts(**opts), 1, 1.02)
    _records_equal(grec, wrec)
    assert gkq == wkq
    np.testing.assert_allclose(gt, wt, rtol=1e-12, atol=0)
    if mode == abi.MODE_BANK:
        assert np.array_equal(gs, ws)


def test_sixteen_groups(ctx_factory):
    rng = np.random.default_rng(21)
    p = synth.random_slab(rng, 6, 16, 0.5, 3.0, 10, 3000, 2, 2)
    opts = dict(seed=3, mode=abi.MODE_BANK, **EXACT)
    grec, gt, gs, gkq = ctx_factory(**opts).trace(p, 0, 1.0)
    wrec, wt, ws, wkq = O.trace_woodcock(p, abi.make_opts(**opts), 0, 1.0)
    _records_equal(grec, wrec)
    assert gkq == wkq and np.array_equal(gs, ws)
    assert grec["final_group"].max() > 7


def _chained_k(p, opts, gens):
    """k per generation on the CPU: each generation's ordered bank is the
    next one's source (particle i takes site floor(i*B/N))."""
    o = abi.make_opts(**opts)
    k, ks, sites = float(p.k_new), [], None
    for g in range(gens):
        _, _, sites, kq = O.trace_woodcock(p, o, g, k, sites_in=sites)
        k = kq * 2.0 ** -32 / p.histories
        ks.append(k)
    return np.array(ks)


@pytest.mark.parametrize("case", ["many_cells", "tables_past_smem"])
def test_chained_generations(ctx_factory, case):
    """15,000 cells (the site histogram no longer fits shared memory) and
    12,000 regions (the tables no longer fit shared memory): whole runs equal
    the CPU restatement generation by generation."""
    rng = np.random.default_rng(8)
    if case == "many_cells":
        p = synth.random_slab(rng, 10, 3, 0.5, 3.0, 1500, 2000, 1, 2)
    else:
        p = synth.random_slab(rng, 12000, 2, 0.5, 2.0, 1, 2000, 1, 2)
    opts = dict(seed=13, mode=abi.MODE_BANK, **EXACT)
    r = ctx_factory(**opts).solve(p)
    want = _chained_k(p, opts, p.generations)
    assert np.array_equal(r.k64, want)
    # ranged launches (tables staged, or read from global memory when they
    # do not fit), each range ordering its own sites
    rr = ctx_factory(range_len=700, **opts).solve(p)
    assert np.array_equal(rr.k64, want)
    np.testing.assert_allclose(rr.entropy, r.entropy, rtol=0, atol=1e-12)
    # the trace path on the same problem (records from the same kernels)
    grec, _, gs, gkq = ctx_factory(**opts).trace(p, 0, 1.0)
    wrec, _, ws, wkq = O.trace_woodcock(p, abi.make_opts(**opts), 0, 1.0)
    _records_equal(grec, wrec)
    assert gkq == wkq and np.array_equal(gs, ws)
