"""Statistical agreement between two Monte Carlo solves of one problem.

The event-based form (Woodcock tracking, FP32 flights, collision estimators)
and the plain FP64 history-per-thread kernel (surface tracking, track-length
estimators) sample the same power iteration from the same PCG32 seeds, but
their histories differ, so they agree in distribution only.  This module
states that agreement for k_eff and for every group's flux:

* generations of a power iteration are correlated (each one's source is the
  previous one's bank), and in a slab the flux shape decorrelates slowly, so
  the agreement statistics use independent replicas (``run_replicas``: the
  same problem under different seeds, each replica's mean over its active
  generations one sample); within one long run, batch means
  (``batch_means``, ``run_batches``) give k's error and the integrated
  autocorrelation time shows how correlated the generations are;
* k: difference in pcm, combined sigma, z = difference / sigma;
* flux: per group, chi^2 of the per-bin differences over the combined
  variances, its degrees of freedom and upper-tail probability, and the
  relative difference of the group's integrated flux with its error -- the
  FP32-vs-FP64 bias of that result.

The reference's own estimator of k is the track-length estimator of
src/mc_code.rs:346-351; the plain kernel keeps it, the event form replaces it
with the collision estimator of the same quantity.
"""
from __future__ import annotations

import math
import time

import numpy as np


def batch_means(x, n_batches: int):
    """Mean of x and its standard error from n_batches consecutive batches
    (a trailing remainder shorter than a batch is dropped)."""
    x = np.asarray(x, np.float64)
    if n_batches < 2 or x.size < n_batches:
        raise ValueError("need at least two batches of one sample each")
    b = x.size // n_batches
    means = x[: b * n_batches].reshape(n_batches, b).mean(axis=1)
    return float(means.mean()), float(means.std(ddof=1) / math.sqrt(n_batches)), b


def autocorr_time(x, max_lag: int | None = None) -> float:
    """Integrated autocorrelation time 1 + 2 sum_t rho(t), summed until the
    first non-positive rho (initial positive sequence); 1.0 for white noise."""
    x = np.asarray(x, np.float64)
    n = x.size
    if n < 4:
        return 1.0
    d = x - x.mean()
    var = float(d @ d) / n
    if var <= 0.0:
        return 1.0
    tau = 1.0
    for t in range(1, min(max_lag or n // 4, n - 1) + 1):
        rho = float(d[:-t] @ d[t:]) / (n * var)
        if rho <= 0.0:
            break
        tau += 2.0 * rho
    return tau


def naive_sigma(x) -> float:
    """Standard error of the mean treating samples as independent (the
    engine's k_sigma)."""
    x = np.asarray(x, np.float64)
    return float(x.std(ddof=1) / math.sqrt(x.size)) if x.size > 1 else float("inf")


def time_to_sigma(k_active, ms_per_generation: float, inactive: int, target: float = 50e-5):
    """Wall time (ms) until the running standard error of k over the active
    generations first reaches `target` (50 pcm), counting the inactive
    generations before them; None if the run never reaches it."""
    k = np.asarray(k_active, np.float64)
    for n in range(2, k.size + 1):
        if naive_sigma(k[:n]) <= target:
            return dict(ms=(inactive + n) * ms_per_generation, active_generations=n,
                        sigma_pcm=naive_sigma(k[:n]) * 1e5)
    return None


def run_batches(session, prob, batch: int):
    """Run a session to its end, inactive generations first, then the active
    ones in batches of `batch`, reading the running flux mean after each.

    Returns dict(k64, flux_batches [B, G*cells] (each batch's per-bin mean),
    results (the final ResultArrays), ms_per_generation (device time of the
    active part / its generations, from the host clock around synchronised
    batches)."""
    session.run(prob.skip)
    session.sync()
    active = prob.generations - prob.skip
    n_b = active // batch
    if n_b < 2:
        raise ValueError("need at least two batches")
    prev = None
    batches = []
    t0 = time.perf_counter()
    busy = 0.0
    for j in range(n_b):
        t = time.perf_counter()
        session.run(batch)
        session.sync()
        busy += time.perf_counter() - t
        r = session.results()
        cum = r.flux_mean * ((j + 1) * batch)
        batches.append(cum if prev is None else cum - prev)
        prev = cum
    rest = prob.generations - session.generation
    if rest:
        session.run(rest)
    res = session.results()
    fb = np.stack(batches) / batch
    return dict(k64=res.k64, flux_batches=fb, results=res, batch=batch,
                active_ms_per_generation=1000.0 * busy / (n_b * batch),
                wall_s=time.perf_counter() - t0)


def welch_z(xa, xb):
    """Per-bin normal score of the difference of two batch-mean estimates.

    xa [Ba, n], xb [Bb, n] are batch means per bin.  The variances of the two
    means are themselves estimated from few batches, so the ratio
    t = (m_a - m_b) / sqrt(v_a + v_b) follows Student's t with the
    Welch-Satterthwaite degrees of freedom, not a normal; squaring it would
    give a chi^2 biased upward by nu / (nu - 2).  Each t is mapped through its
    t distribution to the normal score with the same tail probability, so the
    sum of squares is chi^2 with one degree of freedom per bin under the null.
    Bins with zero variance on both sides give NaN."""
    from scipy import stats as sps
    xa, xb = np.asarray(xa, np.float64), np.asarray(xb, np.float64)
    na, nb = xa.shape[0], xb.shape[0]
    va = xa.var(0, ddof=1) / na
    vb = xb.var(0, ddof=1) / nb
    v = va + vb
    with np.errstate(divide="ignore", invalid="ignore"):
        t = (xa.mean(0) - xb.mean(0)) / np.sqrt(v)
        nu = v ** 2 / (va ** 2 / (na - 1) + vb ** 2 / (nb - 1))
    z = np.full(t.shape, np.nan)
    ok = v > 0
    # two-sided tail of |t| under t(nu) -> the normal score with that tail
    p_half = sps.t.sf(np.abs(t[ok]), nu[ok])
    z[ok] = np.sign(t[ok]) * sps.norm.isf(np.maximum(p_half, 1e-300))
    return z


def run_replicas(make_context, prob, seeds, **opts):
    """Independent replicas of one solve: one context per seed (same problem,
    options), each run to its end.  A replica's k sample is its mean k over
    the active generations and its flux sample its per-bin mean flux, so the
    samples are independent and their spread is an honest error whatever the
    correlation between generations inside a replica.

    Returns dict(k_samples [R], flux_samples [R, G*cells], k64 [R, gens])."""
    ks, fl, k64 = [], [], []
    for sd in seeds:
        ctx = make_context(seed=int(sd), **opts)
        try:
            r = ctx.solve(prob)
        finally:
            close = getattr(ctx, "close", None)
            if close:
                close()
        ks.append(float(r.k64[prob.skip:].mean()))
        fl.append(r.flux_mean.copy())
        k64.append(r.k64.copy())
    return dict(k_samples=np.array(ks), flux_samples=np.stack(fl), k64=np.stack(k64))


def compare_replicas(a: dict, b: dict, G: int, nc: int, coarse: int = 1):
    """k and per-group flux agreement of replica sets `a` and `b`
    (run_replicas): Welch normal scores throughout."""
    from scipy import stats as sps
    ka, kb = np.asarray(a["k_samples"]), np.asarray(b["k_samples"])
    za = welch_z(ka[:, None], kb[:, None])[0]
    sa = ka.std(ddof=1) / math.sqrt(ka.size)
    sb = kb.std(ddof=1) / math.sqrt(kb.size)
    out = {"k_a": float(ka.mean()), "k_b": float(kb.mean()), "sigma_a_pcm": sa * 1e5, "sigma_b_pcm": sb * 1e5,
           "delta_k_pcm": float(ka.mean() - kb.mean()) * 1e5, "sigma_pcm": math.hypot(sa, sb) * 1e5,
           "z": float(za), "replicas": [int(ka.size), int(kb.size)]}
    fa = _coarse(a["flux_samples"], G, nc, coarse)
    fb = _coarse(b["flux_samples"], G, nc, coarse)
    groups = []
    for g in range(G):
        xa, xb = fa[:, g, :], fb[:, g, :]
        z = welch_z(xa, xb)
        ok = np.isfinite(z)
        chi2 = float((z[ok] ** 2).sum())
        dof = int(ok.sum())
        ia, ib = xa.sum(1), xb.sum(1)
        ma_i, mb_i = ia.mean(), ib.mean()
        se = math.hypot(ia.std(ddof=1) / math.sqrt(ia.size), ib.std(ddof=1) / math.sqrt(ib.size))
        zi = float(welch_z(ia[:, None], ib[:, None])[0])
        groups.append({"group": g, "chi2": chi2, "dof": dof, "chi2_per_dof": chi2 / dof if dof else None,
                       "p_value": float(sps.chi2.sf(chi2, dof)) if dof else None,
                       "rel_diff": float(ma_i / mb_i - 1.0) if mb_i else None,
                       "rel_sigma": float(se / mb_i) if mb_i else None, "z_integrated": zi})
    out["flux"] = groups
    out["coarse_cells_per_bin"] = coarse
    return out


def _coarse(a, G: int, nc: int, coarse: int):
    """Sum `coarse` consecutive cells of every group: [..., G*nc] -> [..., G, nc//coarse]."""
    a = np.asarray(a, np.float64)
    lead = a.shape[:-1]
    a = a.reshape(*lead, G, nc)
    m = nc // coarse
    return a[..., : m * coarse].reshape(*lead, G, m, coarse).sum(axis=-1)


def compare(a: dict, b: dict, G: int, nc: int, skip: int, coarse: int = 1, k_batches: int | None = None):
    """k and per-group flux agreement of run `a` against run `b` (dicts from
    run_batches).  coarse > 1 sums that many consecutive cells per bin first
    (meshes whose cells score too few collisions per batch)."""
    from scipy import stats as sps
    ka, kb = np.asarray(a["k64"][skip:]), np.asarray(b["k64"][skip:])
    nba = k_batches or a["flux_batches"].shape[0]
    nbb = k_batches or b["flux_batches"].shape[0]
    ma, sa, _ = batch_means(ka, nba)
    mb, sb, _ = batch_means(kb, nbb)
    sig = math.hypot(sa, sb)
    out = {"k_a": ma, "k_b": mb, "sigma_a_pcm": sa * 1e5, "sigma_b_pcm": sb * 1e5,
           "delta_k_pcm": (ma - mb) * 1e5, "sigma_pcm": sig * 1e5,
           "z": (ma - mb) / sig if sig > 0 else float("inf"),
           "batches": [nba, nbb],
           "autocorr_time": [autocorr_time(ka), autocorr_time(kb)],
           "naive_sigma_pcm": [naive_sigma(ka) * 1e5, naive_sigma(kb) * 1e5]}
    fa = _coarse(a["flux_batches"], G, nc, coarse)
    fb = _coarse(b["flux_batches"], G, nc, coarse)
    groups = []
    for g in range(G):
        xa, xb = fa[:, g, :], fb[:, g, :]
        z = welch_z(xa, xb)
        ok = np.isfinite(z)
        chi2 = float((z[ok] ** 2).sum())
        dof = int(ok.sum())
        # integrated flux of the group: one number per batch
        ia, ib = xa.sum(1), xb.sum(1)
        ma_i, mb_i = ia.mean(), ib.mean()
        se = math.hypot(ia.std(ddof=1) / math.sqrt(ia.size), ib.std(ddof=1) / math.sqrt(ib.size))
        groups.append({"group": g, "chi2": chi2, "dof": dof, "chi2_per_dof": chi2 / dof if dof else None,
                       "p_value": float(sps.chi2.sf(chi2, dof)) if dof else None,
                       "rel_diff": float(ma_i / mb_i - 1.0) if mb_i else None,
                       "rel_sigma": float(se / mb_i) if mb_i else None})
    out["flux"] = groups
    out["coarse_cells_per_bin"] = coarse
    return out
