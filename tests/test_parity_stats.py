"""Host statistics behind the FP32-vs-FP64 agreement (nraps_gb300.parity).

Checked on synthetic series with known answers: batch-means errors of a
correlated (AR(1)) series match the analytic standard error, the Welch normal
scores give chi^2 / dof near 1 under the null with few batches, and a planted
flux bias or k shift is detected.
"""
import math

import numpy as np
import pytest

from nraps_gb300 import parity


def ar1(rng, n, phi, sigma=1.0):
    x = np.zeros(n)
    e = rng.normal(0, sigma, n)
    for i in range(1, n):
        x[i] = phi * x[i - 1] + e[i]
    return x


def test_batch_means_matches_ar1_standard_error():
    rng = np.random.default_rng(0)
    phi, n = 0.6, 4000
    # analytic variance of the mean of a stationary AR(1): sigma^2/(1-phi)^2 / n
    want = 1.0 / (1 - phi) / math.sqrt(n)
    got = [parity.batch_means(ar1(rng, n, phi), 20)[1] for _ in range(40)]
    assert abs(np.mean(got) / want - 1) < 0.15
    naive = parity.naive_sigma(ar1(rng, n, phi))
    assert naive < 0.6 * want          # the naive error is too small for correlated samples
    tau = parity.autocorr_time(ar1(rng, 20000, phi))
    assert abs(tau - (1 + phi) / (1 - phi)) < 0.6


def test_welch_scores_null_and_planted_bias():
    rng = np.random.default_rng(1)
    nbin, B = 2000, 10
    mean = rng.uniform(1, 2, nbin)
    xa = mean + rng.normal(0, 0.05, (B, nbin))
    xb = mean + rng.normal(0, 0.08, (B + 5, nbin))
    z = parity.welch_z(xa, xb)
    chi2 = float((z ** 2).sum())
    # with the t -> normal mapping the statistic is chi^2(nbin), not inflated by nu/(nu-2)
    assert abs(chi2 / nbin - 1) < 0.1
    xb2 = xb * 1.05
    z2 = parity.welch_z(xa, xb2)
    assert (z2 ** 2).sum() / nbin > 2


def _fake_run(rng, G, nc, k, bias=0.0, B=10, gens=100, skip=20):
    flux = np.tile(np.linspace(1, 2, nc), G)
    fb = flux * (1 + bias) + rng.normal(0, 0.02, (B, G * nc))
    k64 = np.concatenate([np.full(skip, k), k + ar1(rng, gens, 0.3, 2e-3)])
    return dict(k64=k64, flux_batches=fb)


def test_compare_reports_agreement_and_bias():
    rng = np.random.default_rng(2)
    G, nc, skip = 4, 200, 20
    a = _fake_run(rng, G, nc, 1.0)
    b = _fake_run(rng, G, nc, 1.0)
    c = parity.compare(a, b, G, nc, skip, coarse=10)
    assert abs(c["z"]) < 4
    for g in c["flux"]:
        assert g["dof"] == nc // 10 and g["p_value"] > 1e-4
        assert abs(g["rel_diff"]) < 5 * g["rel_sigma"]
    d = parity.compare(_fake_run(rng, G, nc, 1.01, bias=0.02), b, G, nc, skip, coarse=10)
    assert d["z"] > 5 and d["delta_k_pcm"] > 500
    assert all(g["p_value"] < 1e-6 and g["rel_diff"] > 0.01 for g in d["flux"])


def test_time_to_sigma():
    k = np.array([1.0, 1.02, 0.98, 1.01, 0.99, 1.0, 1.0, 1.0])
    t = parity.time_to_sigma(k, 2.0, 10, target=0.01)
    assert t is not None and t["active_generations"] >= 2
    assert t["ms"] == (10 + t["active_generations"]) * 2.0
    assert parity.time_to_sigma(np.array([1.0, 2.0, 1.0]), 1.0, 0, target=1e-6) is None
    with pytest.raises(ValueError):
        parity.batch_means([1.0], 2)


def test_replica_comparison_null_and_bias():
    rng = np.random.default_rng(3)
    G, nc, R = 2, 300, 8
    base = np.tile(np.linspace(1, 2, nc), G)

    def reps(k, bias):
        return dict(k_samples=k + rng.normal(0, 1e-3, R),
                    flux_samples=base * (1 + bias) + rng.normal(0, 0.02, (R, G * nc)))
    c = parity.compare_replicas(reps(1.0, 0.0), reps(1.0, 0.0), G, nc, coarse=10)
    assert abs(c["z"]) < 4 and c["replicas"] == [R, R]
    assert all(g["dof"] == 30 and g["p_value"] > 1e-4 and abs(g["z_integrated"]) < 4 for g in c["flux"])
    d = parity.compare_replicas(reps(1.01, 0.02), reps(1.0, 0.0), G, nc, coarse=10)
    assert d["z"] > 5 and all(g["z_integrated"] > 5 for g in d["flux"])


def test_run_replicas_uses_each_seed_once():
    calls = []

    class FakeResult:
        def __init__(self, seed):
            self.k64 = np.full(6, 1.0 + seed * 1e-4)
            self.flux_mean = np.full(4, float(seed))

    class FakeCtx:
        def __init__(self, seed, **kw):
            self.seed = seed
            calls.append((seed, kw))

        def solve(self, prob):
            return FakeResult(self.seed)

        def close(self):
            pass

    class P:
        skip = 2
    r = parity.run_replicas(FakeCtx, P(), [3, 4, 5], mode=2)
    assert [c[0] for c in calls] == [3, 4, 5] and all(c[1] == {"mode": 2} for c in calls)
    assert np.allclose(r["k_samples"], [1.0003, 1.0004, 1.0005]) and r["flux_samples"].shape == (3, 4)
