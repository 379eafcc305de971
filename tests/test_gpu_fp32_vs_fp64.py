"""The chosen form against the plain FP64 kernel at the benchmark geometries.

Event-based Woodcock transport (FP32 flights, FP64 tallies, collision
estimators) and the plain FP64 history-per-thread kernel (surface tracking,
track-length estimators) run the same BANK power iteration from the same
seeds.  Their histories differ, so they agree in distribution:

* k: |k_event - k_plain| < 3 sigma, sigma from batch means of the active
  generations (generations of a power iteration are correlated; the plain
  side reaches sigma_k <= 50 pcm);
* flux: per group, the Welch normal scores of the per-bin batch-mean
  differences give chi^2 with p > 1e-3, and the group's integrated flux
  agrees within 4 sigma.

Tolerances are statistical (no FP tolerance applies: the two forms sample
different histories).  The bins are coarse (0.5 cm on the 2,000-cell slab,
50 regions on the 200,000-cell slab): neighbouring cells' scores come from
the same particles, so fine bins are strongly correlated and a chi^2 that
treats them as independent would be too wide.
"""
import numpy as np
import pytest

from nraps_gb300 import abi, parity, synth

pytestmark = pytest.mark.gpu

EVENT = dict(mode=abi.MODE_BANK, precision=abi.PREC_FP32, tracking=abi.TRACK_WOODCOCK)
PLAIN = dict(mode=abi.MODE_BANK, precision=abi.PREC_FP64, tracking=abi.TRACK_SURFACE)


def _run(ctx_factory, prob, arm, batch, seed, **extra):
    ctx = ctx_factory(seed=seed, **arm, **extra)
    s = ctx.session(prob)
    r = parity.run_batches(s, prob, batch)
    s.close()
    return r


def _check(c, plain_sigma_max_pcm=None):
    assert abs(c["z"]) < 3, c
    if plain_sigma_max_pcm is not None:
        assert c["sigma_b_pcm"] <= plain_sigma_max_pcm, c
    for g in c["flux"]:
        assert g["p_value"] > 1e-3, g
        assert abs(g["rel_diff"]) < 4 * g["rel_sigma"], g


def test_single_large_geometry(ctx_factory):
    """2,000 cells, 4 groups (the throughput workload), 2e5 histories,
    30 inactive + 100 active generations in 10 batches."""
    p = synth.single_large(1).with_(histories=200_000, generations=130, skip=30)
    ev = _run(ctx_factory, p, EVENT, 10, 1)
    pl = _run(ctx_factory, p, PLAIN, 10, 1)
    c = parity.compare(ev, pl, p.energygroups, p.n_cells, p.skip, coarse=40)
    _check(c, plain_sigma_max_pcm=50)


def test_scale_stress_geometry_8_groups(ctx_factory):
    """200,000 cells, 10,000 regions, 8 groups at 2e5 histories, both forms
    started from the diffusion fission source, 10 inactive + 40 active
    generations in 8 batches."""
    p = synth.scale_stress(1, histories=200_000).with_(generations=50, skip=10)
    ev = _run(ctx_factory, p, EVENT, 5, 2, initial_source=1)
    pl = _run(ctx_factory, p, PLAIN, 5, 2, initial_source=1)
    c = parity.compare(ev, pl, p.energygroups, p.n_cells, p.skip, coarse=1000)
    _check(c)
    assert len(c["flux"]) == 8 and all(g["dof"] == 200 for g in c["flux"])
