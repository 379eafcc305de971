"""The chosen form against the plain FP64 kernel at the benchmark geometries.

Event-based Woodcock transport (FP32 flights, FP64 tallies, collision
estimators) and the plain FP64 history-per-thread kernel (surface tracking,
track-length estimators) run the same BANK power iteration.  Their histories
differ, so they agree in distribution.  Each form runs R independent replicas
(the same seeds for both forms); a replica's mean k over its active
generations and its per-cell mean flux are one sample each, so the errors
come from the replicas' spread and do not depend on how strongly the
generations inside one replica are correlated:

* k: the Welch normal score of k_event - k_plain is below 3 in magnitude
  (the plain side's error is at most 50 pcm);
* flux: per group, the Welch normal scores of the per-bin differences give
  chi^2 with p > 1e-4, and the group's integrated flux agrees within 4 sigma.

Tolerances are statistical: the two forms sample different histories.  Bins
are coarse (100 cells = 1.25 cm on the 2,000-cell slab, 10,000 cells on the
200,000-cell slab): neighbouring cells' scores come from the same particles,
so fine bins are correlated and a chi^2 that treats them as independent
would be too wide.
"""
import numpy as np
import pytest

from nraps_gb300 import abi, parity, synth

pytestmark = pytest.mark.gpu

EVENT = dict(mode=abi.MODE_BANK, precision=abi.PREC_FP32, tracking=abi.TRACK_WOODCOCK)
PLAIN = dict(mode=abi.MODE_BANK, precision=abi.PREC_FP64, tracking=abi.TRACK_SURFACE)


def _check(c, plain_sigma_max_pcm=None):
    assert abs(c["z"]) < 3, c
    if plain_sigma_max_pcm is not None:
        assert c["sigma_b_pcm"] <= plain_sigma_max_pcm, c
    for g in c["flux"]:
        assert g["p_value"] > 1e-4, g
        assert abs(g["z_integrated"]) < 4, g


def test_single_large_geometry(ctx_factory):
    """2,000 cells, 4 groups (the throughput workload) at 2e5 histories, 8
    replicas of 20 inactive + 40 active generations per form."""
    p = synth.single_large(1).with_(histories=200_000, generations=60, skip=20)
    seeds = [101 + i for i in range(8)]
    ev = parity.run_replicas(ctx_factory, p, seeds, **EVENT)
    pl = parity.run_replicas(ctx_factory, p, seeds, **PLAIN)
    c = parity.compare_replicas(ev, pl, p.energygroups, p.n_cells, coarse=100)
    _check(c, plain_sigma_max_pcm=50)
    assert len(c["flux"]) == 4 and all(g["dof"] == 20 for g in c["flux"])


def test_scale_stress_geometry_8_groups(ctx_factory):
    """200,000 cells, 10,000 regions, 8 groups at 2e5 histories from the
    uniform fuel source, 6 replicas of 10 inactive + 20 active generations per
    form (the slab's source does not converge in so few generations, but both
    forms follow the same expected sequence of sources)."""
    p = synth.scale_stress(1, histories=200_000).with_(generations=30, skip=10)
    seeds = [201 + i for i in range(6)]
    ev = parity.run_replicas(ctx_factory, p, seeds, **EVENT)
    pl = parity.run_replicas(ctx_factory, p, seeds, **PLAIN)
    c = parity.compare_replicas(ev, pl, p.energygroups, p.n_cells, coarse=10_000)
    _check(c)
    assert len(c["flux"]) == 8 and all(g["dof"] == 20 for g in c["flux"])
