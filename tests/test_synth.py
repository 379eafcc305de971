"""Synthetic workload generator: the deterministic k that scales nu*sigf.

The Arnoldi solve used for the long scale-stress slab must give the power
iteration's eigenvalue, and a slab scaled by it must have diffusion k = 1.
"""
import numpy as np

from nraps_gb300 import synth


def test_arnoldi_diffusion_k_matches_power_iteration():
    p = synth.plain_small(3)
    rng = np.random.default_rng(3)
    xs = synth.xs_set(rng, 4)
    k_pi = synth.diffusion_k(p.matid, p.delta_x, xs, p.sigf.astype(np.float64))
    k_ar = synth.diffusion_k_large(p.matid, p.delta_x, xs, p.sigf.astype(np.float64))
    assert abs(k_ar / k_pi - 1) < 1e-6
    # the generator's own k for this slab (1 unless the sigf <= siga clamp bit)
    assert abs(k_pi - p.k_deterministic) < 1e-6


def test_long_slab_scaled_to_unit_k():
    rng = np.random.default_rng(7)
    p = synth.random_slab(rng, 400, 8, 0.5, 2.0, 5, 1000, 2, 2, k_method="diffusion_large")
    rng = np.random.default_rng(7)
    xs = synth.xs_set(rng, 8)
    k = synth.diffusion_k_large(p.matid, p.delta_x, xs, p.sigf.astype(np.float64))
    assert abs(k - 1.0) < 1e-4
    assert p.k_deterministic is not None and abs(p.k_deterministic - 1.0) < 1e-4
