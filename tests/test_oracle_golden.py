"""The CPU oracle against the reference's own unit tests and known answers.

Restates src/mc_code.rs:392-556 (test_boundary, test_cross_mesh,
test_direction, test_scat_mat_calc) with the same inputs and expected values,
the pcg-c-basic known-answer stream that rand.rs's seeding reproduces, and
the shared logarithm's error bound against libm.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O


def approx(a, b):
    # float_cmp approx_eq with (epsilon 1e-9, 2 ulps) as the reference uses
    a, b = np.float32(a), np.float32(b)
    if abs(float(a) - float(b)) <= 1e-9:
        return True
    ia = np.array([a]).view(np.int32)[0]
    ib = np.array([b]).view(np.int32)[0]
    return abs(int(ia) - int(ib)) <= 2


def test_boundary():  # src/mc_code.rs:392-413
    cases = [((0.5, 0.5, 1.0, 1.0, 1.0), (-0.5, -0.5, 1.0)),
             ((-0.5, 0.5, -1.0, 1.0, 0.0), (0.5, 0.5, 0.0)),
             ((0.5, 0.5, 0.5, 1.0, 1.0), (-0.5, 0.0, 1.0)),
             ((-0.5, 0.5, -0.5, 1.0, 0.0), (0.5, 0.0, 0.0))]
    for args, want in cases:
        got = O.hit_boundary(*args)
        assert all(approx(g, w) for g, w in zip(got, want)), (args, got)


def test_cross_mesh():  # src/mc_code.rs:415-426
    ds, x, i = O.cross_mesh(1, 0.5, 0.5, 1.0, 1.0)
    assert approx(ds, 0.5) and approx(x, 1.0) and i == 2
    ds, x, i = O.cross_mesh(1, -0.5, 1.0, 0.5, -1.0)
    assert approx(ds, -0.5) and approx(x, 0.5) and i == 0


def test_direction():  # src/mc_code.rs:428-444
    for r, want in ((1.0, 1.0), (0.75, 0.5), (0.5, 0.0), (0.25, -0.5), (0.0, -1.0)):
        assert approx(O.direction(r), want)


SCAT_A = np.array([0.185, 0.015, 0.000, 0.800, 0.185, 0.015, 0.000, 0.800, 0.170, 0.030, 0.000, 1.100,
                   0.000, 0.000, 0.000, 0.100], np.float32)
SIGS_A = np.array([0.200, 0.200, 0.200, 0.0, 0.80, 0.80, 1.10, 0.1], np.float32)


def test_scat_mat_calc():  # src/mc_code.rs:464-556, exact f32 equality
    check = [[0.925, 1.0], [0.925, 1.0], [0.85, 1.0], None, [0.0, 1.0], [0.0, 1.0], [0.0, 1.0], [0.0, 1.0]]
    for g, mats in ((0, range(3)), (1, range(4))):
        for m in mats:
            inv = np.float32(1.0) / SIGS_A[m + 4 * g]
            got = O.scat_mat_calc(2, m, g, inv, SCAT_A)
            assert np.array_equal(got, np.array(check[g * 4 + m], np.float32)), (g, m, got)


def test_energy_partition_point():
    # the commented-out test_energy of src/mc_code.rs:446-462, on the same list
    cdf = [0.0, 0.0, 0.5, 1.0]
    assert O.energy_cdf(cdf, 1.0) == 3
    assert O.energy_cdf(cdf, 0.51) == 3
    assert O.energy_cdf(cdf, 0.5) == 2
    assert O.energy_cdf(cdf, 0.49) == 2
    assert O.energy_cdf(cdf, 1e-9) == 2


def test_partition_fresh_probe_count():
    # Rust's fixed-iteration binary search: ceil(log2 n) probes + 1 final
    for n, probes in ((2, 2), (3, 3), (4, 3), (8, 4)):
        _, d = O.partition_fresh(np.linspace(0.1, 1.0, n), 5, 9)
        assert d == probes


def test_pcg32_known_answer():
    # pcg32_srandom_r(42, 54) demo stream of pcg-c-basic; rand.rs seeds the
    # same way (src/rand.rs:49-71)
    want = [0xa15c02b7, 0x7b47f409, 0xba1d3330, 0x83d2f293, 0xbfa4784b, 0xcbed606e]
    assert [int(v) for v in O.pcg32(42, 54, 6)] == want


def test_rand_rs_next_f32_range():
    # next_f32 = (u as f32) * 2.3283064E-10 reaches 1.0 for u >= 2^32-128
    assert np.float32(np.float32(2**32 - 1) * np.float32(2.3283064e-10)) == 1.0
    assert np.float32(2.3283064e-10) == np.float32(2.0 ** -32)


@pytest.mark.parametrize("seed", [1, 2])
def test_shared_log_error_bound(seed):
    rng = np.random.default_rng(seed)
    xs = np.concatenate([rng.random(20000) + 1e-12, np.exp(rng.uniform(-700, 700, 2000)),
                         [1.0, 0.5, 2.0, 1e-300, 5e-324, 0.7071067811865476, 1.4142135623730951]])
    for x in xs:
        got = O.log64(float(x))
        want = math.log(x)
        ulp = abs(np.array([got]).view(np.int64)[0] - np.array([want]).view(np.int64)[0])
        assert ulp <= 2, (x, got, want)
        gf = O.log32(np.float32(x))
        xf = np.float32(x)
        if xf > 0:
            wf = np.float32(math.log(float(xf)))
            uf = abs(int(np.array([gf]).view(np.int32)[0]) - int(np.array([wf]).view(np.int32)[0]))
            assert uf <= 2, (x, gf, wf)
    assert O.log64(1.0) == 0.0 and math.isinf(O.log64(0.0)) and math.isnan(O.log64(-1.0))
