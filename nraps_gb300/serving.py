"""Poisson-arrival driver for the request server (continuous batching).

Requests arrive as a Poisson stream; each is a k-eigenvalue solve whose
geometry and cross sections come from the batched-instance distribution
(regions U{4..64}, groups U{2..8}, widths U[0.5, 3] cm) and whose histories
per generation are log-uniform in [10k, 500k].  Every request carries the
accuracy target: it is done when the standard error of its k over its active
generations is at most sigma_k_target (after at least min_active active
generations).  The driver submits each request at its arrival time, steps the
server (one to four generations of every admitted request per step: as many
as no request could retire within), and records the time from arrival to
completion.
"""
from __future__ import annotations

import math
import time

import numpy as np

from . import abi, api, synth


def geometry_pool(seed: int, n: int, inactive: int, max_generations: int):
    """n distinct slab geometries (histories set per request later)."""
    rng = np.random.default_rng(seed)
    pool = []
    for _ in range(n):
        R = int(rng.integers(4, 65))
        G = int(rng.integers(2, 9))
        pool.append(synth.random_slab(rng, R, G, 0.5, 3.0, 10, 10_000, inactive,
                                      max_generations - inactive))
    return pool


def run_poisson(ctx: api.Context, rate: float = 200.0, seconds: float = 20.0, seed: int = 1,
                sigma_k_target: float = 50e-5, min_active: int = 10, inactive: int = 20,
                max_generations: int = 2000, drain_seconds: float = 60.0, pool_size: int = 32,
                hbm_budget_bytes: int = 120 << 30, pool=None) -> dict:
    rng = np.random.default_rng(seed + 17)
    pool = pool or geometry_pool(seed, pool_size, inactive, max_generations)
    n_req = int(rng.poisson(rate * seconds))
    arrivals = np.sort(rng.uniform(0.0, seconds, n_req))
    sizes = np.exp(rng.uniform(math.log(1e4), math.log(5e5), n_req)).astype(np.int64)
    geo = rng.integers(0, len(pool), n_req)
    srv = api.Server(ctx, hbm_budget_bytes=hbm_budget_bytes, sigma_k_target=sigma_k_target,
                     min_active=min_active, max_slots=4095)
    t0 = srv.clock
    submitted = {}            # rid -> (index, arrival)
    in_flight = set()
    lat, gens, hist_done = [], [], 0
    rejected = 0
    nxt = 0
    steps = 0
    busy0 = srv.stats()["busy_ms"]
    window_hist = None           # histories simulated by the end of the arrival window
    while True:
        now = srv.clock - t0
        if window_hist is None and now >= seconds:
            window_hist = srv.stats()["histories"]
        while nxt < n_req and arrivals[nxt] <= now:
            p = pool[geo[nxt]].with_(histories=int(sizes[nxt]))
            try:
                rid = srv.submit(p, int(1_000_003 * nxt + seed))
                submitted[rid] = (nxt, float(arrivals[nxt]))
                in_flight.add(rid)
            except api.NrapsError as e:
                if e.status != abi.ERR_REJECTED:
                    raise
                rejected += 1
            nxt += 1
        st = srv.stats()
        if st["running"] or st["waiting"]:
            _, fin = srv.step()
            steps += 1
            if fin:
                for rid in srv.finished():
                    s, info, _ = srv.poll(rid, results=False)
                    idx, arr = submitted[rid]
                    lat.append(info["t_done"] - t0 - arr)
                    gens.append(info["generations_run"])
                    hist_done += info["generations_run"] * info["histories_per_generation"]
                    in_flight.discard(rid)
                    srv.release(rid)
        elif nxt < n_req:
            time.sleep(max(0.0, min(0.01, arrivals[nxt] - now)))
        now = srv.clock - t0
        if nxt >= n_req and not in_flight:
            break
        if now > seconds + drain_seconds:
            break
    elapsed = srv.clock - t0
    st = srv.stats()
    srv.close()
    lat = np.array(lat) if lat else np.zeros(1)
    return {
        "rate_per_s": rate, "seconds": seconds, "submitted": len(submitted), "rejected": rejected,
        "completed": int(len(lat)) if len(submitted) else 0, "unfinished": len(in_flight),
        "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
        "mean_generations": float(np.mean(gens)) if gens else 0.0,
        "histories_per_s": st["histories"] / elapsed if elapsed > 0 else 0.0,
        "window_histories_per_s": (window_hist if window_hist is not None else st["histories"]) / seconds,
        "completed_histories": int(hist_done), "elapsed_s": elapsed, "steps": steps,
        "gpu_busy_fraction": (st["busy_ms"] - busy0) / 1000.0 / elapsed if elapsed > 0 else 0.0,
        "sigma_k_target": sigma_k_target, "min_active": min_active, "inactive": inactive,
    }
