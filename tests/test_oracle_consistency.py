"""Self-consistency of the CPU oracle on small problems."""
import numpy as np

from nraps_gb300 import abi, synth
from oracle import oracle as O


def small(hist=500, gens=8, skip=3):
    return synth.plain_small(3).with_(histories=hist, generations=gens, skip=skip)


def test_bank_mode_independent_of_thread_count():
    p = small()
    o = abi.make_opts(seed=11, mode=abi.MODE_BANK, precision=abi.PREC_FP64)
    r1 = O.monte_carlo(p, o, threads=1)
    r3 = O.monte_carlo(p, o, threads=3)
    assert np.array_equal(r1.k64, r3.k64)
    assert np.allclose(r1.entropy, r3.entropy, rtol=0, atol=1e-12)


def test_trace_equals_monte_carlo_first_generation():
    p = small()
    o = abi.make_opts(seed=5, mode=abi.MODE_PHYSICS, precision=abi.PREC_FP64)
    rec, tally, _, kq = O.trace_generation(p, o, 0, 1.0)
    r = O.monte_carlo(p, o, threads=2)
    assert r.k64[0] == (kq * 2.0 ** -32) / p.histories
    assert np.isclose(rec["nsf_track"].sum() / p.histories, r.k64[0], rtol=1e-9)


def test_compat_runs_n_plus_t_histories():
    p = small(hist=100, gens=2, skip=1)
    o = abi.make_opts(seed=5, mode=abi.MODE_COMPAT, precision=abi.PREC_FP32, compat_threads=3)
    rec, _, _, _ = O.trace_generation(p, o, 0, 1.0)
    assert len(rec) == 103
    r = O.monte_carlo(p, o, threads=3)
    assert r.stats.histories == 2 * 103


def test_fp32_and_fp64_share_most_event_sequences():
    p = small(hist=400)
    recs = []
    for prec in (abi.PREC_FP32, abi.PREC_FP64):
        o = abi.make_opts(seed=2, mode=abi.MODE_PHYSICS, precision=prec)
        recs.append(O.trace_generation(p, o, 0, 1.0)[0])
    same = (recs[0]["collisions"] == recs[1]["collisions"]) & (recs[0]["final_cell"] == recs[1]["final_cell"])
    assert same.mean() > 0.95


def test_bank_sites_ordered_by_parent():
    p = small(hist=300)
    o = abi.make_opts(seed=9, mode=abi.MODE_BANK, precision=abi.PREC_FP64)
    rec, _, sites, _ = O.trace_generation(p, o, 0, 1.0)
    assert len(sites) == int(rec["n_sites"].sum())
    parents = np.repeat(np.arange(len(rec)), rec["n_sites"])
    cells = sites["cell"]
    assert np.all(cells < p.n_cells)
    assert np.all(np.isin(p.matid[cells], [0, 1]))   # fission only in fuel
    assert len(parents) == len(sites)
