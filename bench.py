"""Benchmark: histories/s of the Monte Carlo k-eigenvalue generation loop.

Workload (default): single_large — 1D fuel/water slab, 4 groups, 2,000 tally
cells, 1M histories per generation, fission-bank power iteration; a step is
one generation.  Warm-up steps are the inactive generations, timed steps the
active ones (defaults 50 + 200, the full workload), so sigma_k of the timed
generations is reported beside the throughput.

Arms:
  default            the chosen form (event-based Woodcock, FP32 flights, FP64
                     tallies/k), falling back to nothing: if the CUDA library
                     cannot run, the bench fails.
  --impl reference   the reference algorithm (CPU restatement of
                     src/mc_code.rs in COMPAT mode, f32, the reference's thread
                     policy T = cores - 1) on a bounded sample per step.

Timing: every step is bracketed by CUDA events on the engine's stream; the L2
(129 MB) is flushed between steps by writing a 256 MB buffer outside the
brackets.  `e2e` times the drop-in C-ABI call nraps_monte_carlo with host
buffers on the whole workload.  One JSON line is printed by rank 0.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

ALG_BYTES_PER_COLLISION = 48  # 24 B particle record read + written per real collision


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_per_collision():
    """DRAM bytes per real collision of the dominant kernel from the committed
    ncu summary (profiles/*traffic*.txt: 'bytes_per_collision = X'), or None."""
    d = os.path.join(ROOT, "profiles")
    if not os.path.isdir(d):
        return None
    for f in sorted(os.listdir(d)):
        if "traffic" in f and f.endswith(".txt"):
            for line in open(os.path.join(d, f)):
                if line.strip().startswith("bytes_per_collision"):
                    try:
                        return float(line.split("=")[1])
                    except ValueError:
                        pass
    return None


def replica_seed(base: int, rank: int) -> int:
    """Each rank of a multi-GPU run is an independent replica with its own seed."""
    return base + 1000 * rank


def max_over_ranks(x: float, device="cpu") -> float:
    """The slowest rank's time (all-reduce MAX; identity without a process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank: float, ms_max: float, world: int) -> float:
    """Whole-job units/s of `world` replicas that each processed units_per_rank
    in at most ms_max milliseconds."""
    return world * units_per_rank / (ms_max / 1000.0)


class Clocks:
    def __init__(self, index: int):
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"nraps_clocks_{os.getpid()}.csv")
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        loaded = [v for v in sm if v > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def full_workload(name: str, seed: int):
    """The workload as configured (its own histories and inactive + active
    generations)."""
    from nraps_gb300 import synth
    if name == "single_large":
        return synth.single_large(seed)
    if name == "plain_small":
        return synth.plain_small(seed)
    if name == "scale_stress":
        return synth.scale_stress(seed)
    raise SystemExit(f"unknown workload {name}")


def make_workload(name: str, seed: int, warmup: int, steps: int):
    """The workload with warm-up steps as inactive and timed steps as active
    generations."""
    return full_workload(name, seed).with_(generations=warmup + steps, skip=warmup)


def arm_config(args, prob, world: int) -> dict:
    """The `config` object of the JSON line: the workload, the same for both
    arms."""
    return {"workload": args.workload, "histories_per_step": prob.histories,
            "cells": prob.n_cells, "groups": prob.energygroups,
            "generations": f"{args.warmup} inactive (warm-up) + {args.steps} active (timed)",
            "l2": "flushed between steps (256 MB write)",
            "parallelism": f"replicas x{world}" if world > 1 else "1 GPU"}


ARMS = {
    "event": dict(mode=2, precision=1, tracking=1),
    "plain": dict(mode=2, precision=0, tracking=0),
}


def measure_device(prob, arm: str, steps: int, warmup: int, seed: int, device: int, shape=None, sort=0,
                   extra=None):
    """Device-resident throughput: per-step CUDA events on the engine stream.
    shape = (block, events_per_pass, passes[, tail_lanes]) fixes the event launch shape
    (no autotuning); None lets the engine tune it over the warm-up."""
    import torch
    from nraps_gb300 import api
    kw = dict(ARMS[arm])
    if shape:
        kw.update(block_size=shape[0], events_per_pass=shape[1], passes=shape[2])
        if len(shape) > 3:
            kw.update(tail_lanes=shape[3])
    if sort:
        kw.update(sort_rounds=sort)
    if extra:
        kw.update(extra)
    ctx = api.Context(seed=seed, device=device, **kw)
    s = ctx.session(prob)
    s.set_profile(True)
    ext = torch.cuda.ExternalStream(ctx.stream_ptr, device=device)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{device}")
    s.run(warmup)
    tuning = s.tuning() if arm == "event" else None
    t0 = s.timing()
    launches0 = ctx.launches
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    torch.cuda.synchronize(device)
    for i in range(steps):
        with torch.cuda.stream(ext):
            flush.zero_()
            ev[i][0].record(ext)
        s.run(1)
        if i == steps - 1:
            # a generation's fold may run inside the next one's transport
            # launch: the last one's goes inside the timed region too
            s.flush()
        with torch.cuda.stream(ext):
            ev[i][1].record(ext)
    torch.cuda.synchronize(device)
    t1 = s.timing()
    ms = sum(a.elapsed_time(b) for a, b in ev)
    res = s.results()
    out = dict(ms=ms, histories=steps * prob.histories, collisions=t1["collisions"] - t0["collisions"],
               transport_ms=t1["transport_ms"] - t0["transport_ms"],
               transport_launches=t1["transport_launches"] - t0["transport_launches"],
               launches=ctx.launches - launches0, k_mean=res.stats.k_mean, k_sigma=res.stats.k_sigma,
               tuning=tuning, k64=res.k64.copy())
    # the flush zero_() launches are torch's, not ours; ctx.launches counts ours
    s.close()
    ctx.close()
    return out


def measure_e2e(prob, arm: str, seed: int, device: int):
    """The drop-in call with host buffers: nraps_monte_carlo end to end over
    the workload's whole run (single_large: 50 inactive + 200 active
    generations, whatever --steps/--warmup say), uploads, tuning and
    downloads inside the timed region."""
    from nraps_gb300 import api
    ctx = api.Context(seed=seed, device=device, **ARMS[arm])
    # warm-up: one untimed call of the same size (module loading, the
    # allocations of a first call); then the mean of three timed calls
    ctx.monte_carlo(prob)
    reps = 3
    t = time.perf_counter()
    for _ in range(reps):
        r = ctx.monte_carlo(prob)
    dt = (time.perf_counter() - t) / reps
    ctx.close()
    inputs = [prob.sigt, prob.sigs, prob.mu, prob.siga, prob.sigf, prob.nut, prob.chit, prob.scat,
              prob.inv_sigtr, prob.matid, prob.delta_x, prob.mesh_left, prob.mesh_right, prob.fuel_indices]
    h2d = sum(a.nbytes for a in inputs)
    d2h = (r.flux.nbytes + r.assembly_average.nbytes + r.fission_source.nbytes + r.k.nbytes + r.k_fund.nbytes
           + r.k64.nbytes + r.entropy.nbytes + r.flux_mean.nbytes + r.flux_sem.nbytes)
    g = prob.generations
    return dict(value=prob.histories * g / dt, seconds=dt, h2d=h2d / g, d2h=d2h / g, k_mean=r.stats.k_mean,
                k_sigma=r.stats.k_sigma, generations=g, k64=r.k64.copy())


def measure_parity(full, seed: int, device: int, replicas: int = 6, inactive: int = 20, active: int = 30,
                   plain_ms_per_generation: float | None = None, event_ms_per_generation: float | None = None,
                   event_k64=None, coarse=(1, 100)):
    """The chosen form (event Woodcock, FP32 flights) against the plain FP64
    kernel on the same workload (geometry, cross sections, histories per
    generation), BANK mode both, from `replicas` independent seeds each
    (inactive + active generations per replica): k difference with its
    combined error, per-group flux chi^2 (per cell and over 100-cell bins)
    and the group's integrated-flux bias; the wall time each form needs to
    reach sigma_k <= 50 pcm."""
    from nraps_gb300 import api, parity
    p = full.with_(generations=inactive + active, skip=inactive)
    seeds = [seed * 7919 + 13 * i for i in range(replicas)]

    def make(**kw):
        return api.Context(device=device, **kw)

    ev = parity.run_replicas(make, p, seeds, **ARMS["event"])
    pl = parity.run_replicas(make, p, seeds, **ARMS["plain"])
    G, nc = full.energygroups, full.n_cells
    out = {"workload": full.name.split(":")[0], "mode": "BANK", "same_seeds": True,
           "replicas": replicas, "generations_per_replica": f"{inactive} + {active}"}
    for cz in coarse:
        c = parity.compare_replicas(ev, pl, G, nc, coarse=cz)
        if cz == coarse[0]:
            out.update({k: c[k] for k in ("k_a", "k_b", "sigma_a_pcm", "sigma_b_pcm", "delta_k_pcm",
                                          "sigma_pcm", "z")})
            out["k_event"], out["k_plain_fp64"] = out.pop("k_a"), out.pop("k_b")
            out["sigma_event_pcm"], out["sigma_plain_fp64_pcm"] = out.pop("sigma_a_pcm"), out.pop("sigma_b_pcm")
        out[f"flux_{cz}_cells_per_bin"] = c["flux"]
    if event_k64 is not None and event_ms_per_generation:
        out["event_time_to_50pcm"] = parity.time_to_sigma(event_k64[full.skip:], event_ms_per_generation,
                                                          full.skip)
    if plain_ms_per_generation:
        out["plain_fp64_time_to_50pcm"] = parity.time_to_sigma(pl["k64"][0][inactive:], plain_ms_per_generation,
                                                               inactive)
    return out


def measure_plain_small(seed: int, device: int, threads: int):
    """Config 0 (plain_small: 4 groups, 500 cells, 10k histories, 50 + 100
    generations) on the host cores (the oracle, COMPAT f32, the reference's
    thread policy) and on the plain FP64 GPU kernel (COMPAT, the same
    algorithm, and BANK): histories/s, k, sigma_k and time to 50 pcm."""
    from nraps_gb300 import abi, api, parity, synth
    from oracle import oracle as O
    p = synth.plain_small(seed)
    skip, active = p.skip, p.generations - p.skip
    out = {"workload": "plain_small", "cells": p.n_cells, "groups": p.energygroups,
           "histories_per_generation": p.histories, "generations": f"{skip} + {active}"}
    o = abi.make_opts(seed=12345, mode=abi.MODE_COMPAT, precision=abi.PREC_FP32, compat_threads=threads)
    t = time.perf_counter()
    r = O.monte_carlo(p, o, threads=threads, acc64=False)
    dt = time.perf_counter() - t
    k = r.k64[skip:]
    # COMPAT keeps the reference's 0/0 at a zero cosine (src/mc_code.rs:184):
    # a generation that drew mu == 0 exactly has a NaN k
    ok = np.isfinite(k)
    out["cpu_port_compat_f32"] = {
        "histories_per_s": (p.histories + threads) * p.generations / dt, "seconds": dt, "cores": threads,
        "k_mean": float(k[ok].mean()) if ok.any() else None,
        "sigma_pcm": parity.naive_sigma(k[ok]) * 1e5 if ok.sum() > 1 else None,
        "nan_generations": int((~ok).sum()),
        "time_to_50pcm": parity.time_to_sigma(k[ok], 1000.0 * dt / p.generations, skip)}
    for name, mode in (("gpu_plain_fp64_compat", abi.MODE_COMPAT), ("gpu_plain_fp64_bank", abi.MODE_BANK)):
        ctx = api.Context(seed=12345, device=device, mode=mode, precision=abi.PREC_FP64,
                          compat_threads=threads if mode == abi.MODE_COMPAT else 0)
        ctx.solve(p.with_(generations=4, skip=2))          # module load, first allocations
        s = ctx.session(p)
        s.set_profile(True)
        s.run(p.generations)
        tm = s.timing()
        res = s.results()
        s.close()
        ctx.close()
        k = res.k64[skip:]
        ok = np.isfinite(k)
        ms_gen = tm["total_ms"] / p.generations
        hist = (p.histories + (threads if mode == abi.MODE_COMPAT else 0)) * p.generations
        out[name] = {"histories_per_s": hist / (tm["total_ms"] / 1000.0), "ms_per_generation": ms_gen,
                     "k_mean": float(k[ok].mean()) if ok.any() else None,
                     "sigma_pcm": parity.naive_sigma(k[ok]) * 1e5 if ok.sum() > 1 else None,
                     "nan_generations": int((~ok).sum()),
                     "time_to_50pcm": parity.time_to_sigma(k[ok], ms_gen, skip)}
    out["note"] = ("10k histories per generation: sigma_k per generation is ~1100 pcm, so 100 active "
                   "generations reach ~110 pcm, not 50")
    return out


def measure_batched(seed: int, device: int, steps: int, warmup: int = 3, instances: int = 256, shape=None):
    """256 independent slabs (regions U{4..64}, groups U{2..8}, widths
    U[0.5,3] cm, histories log-uniform [10k,500k]) advancing together, one
    CUDA-graph replay per generation.  shape = (block, range_len) fixes the
    launch shape (no autotuning: for profiling, where ncu's serialisation
    would change the tuner's pick)."""
    import torch
    from nraps_gb300 import api, synth
    kw = dict(ARMS["event"])
    if shape:
        kw.update(block_size=shape[0], range_len=shape[1])
    else:
        # the batch's autotuner tries 12 launch shapes over its first inactive
        # generations: warm up past them so the timed generations run the choice
        warmup = max(warmup, 14)
    probs = synth.batched(seed, n=instances, inactive=max(20, warmup), active=max(20, steps))
    ctx = api.Context(seed=seed, device=device, use_graphs=1, **kw)
    b = api.Batch(ctx, probs, seeds=[seed * 1000 + i for i in range(len(probs))])
    b.run(warmup)
    tuning = b.tuning()
    t0 = b.timing()
    launches0 = ctx.launches
    b.run(steps)
    t1 = b.timing()
    ms = t1["ms"] - t0["ms"]
    hist = t1["histories"] - t0["histories"]
    out = {"instances": len(probs), "histories_per_generation": sum(p.histories for p in probs),
           "steps": steps, "ms_per_step": ms / steps, "histories_per_s": hist / (ms / 1000.0),
           "collisions_per_s": (t1["collisions"] - t0["collisions"]) / (ms / 1000.0),
           "gpu_launches": ctx.launches - launches0, "graphs": True,
           "groups": "U{2..8}", "regions": "U{4..64}",
           "launch_shape": {"block": tuning["block"], "range_len": tuning["range_len"],
                            "tried_ms": tuning["tried_ms"]}}
    b.close()
    ctx.close()
    return out


def measure_serving(seed: int, device: int, seconds: float, rate: float, drain_seconds: float = 60.0):
    from nraps_gb300 import api, serving
    ctx = api.Context(seed=seed, device=device, **ARMS["event"])
    r = serving.run_poisson(ctx, rate=rate, seconds=seconds, seed=seed, drain_seconds=drain_seconds)
    ctx.close()
    return r


def measure_scale_stress(seed: int, device: int, plain_active: int = 20):
    """8 groups, 10,000 regions, 200,000 cells, 10M histories, 20 + 50, nu*sigf
    scaled so the slab's diffusion k is 1.  Both forms start from the
    diffusion fission source (a 12,500 cm slab's dominance ratio is so close
    to one that 20 inactive generations cannot converge a uniform start); the
    plain FP64 kernel runs 20 + `plain_active` generations of the same slab
    and seeds, and the two k are compared over the same generations."""
    from nraps_gb300 import parity, synth
    prob = synth.scale_stress(seed)
    active = prob.generations - prob.skip
    d = measure_device(prob, "event", active, prob.skip, seed, device, extra=dict(initial_source=1))
    per_launch_ms = d["transport_ms"] / max(1, d["transport_launches"])
    coll_per_launch = d["collisions"] / max(1, d["transport_launches"])
    pp = prob.with_(generations=prob.skip + plain_active)
    dp = measure_device(pp, "plain", plain_active, prob.skip, seed, device, extra=dict(initial_source=1))
    # the same run from the reference's uniform fuel source, for comparison
    du = measure_device(prob, "event", active, prob.skip, seed, device)
    ke = d["k64"][prob.skip: prob.skip + plain_active]
    kp = dp["k64"][prob.skip: prob.skip + plain_active]
    me, se, _ = parity.batch_means(ke, 4)
    mp, sp, _ = parity.batch_means(kp, 4)
    sig = float(np.hypot(se, sp))
    return {"workload": "scale_stress", "cells": prob.n_cells, "regions": 10000, "groups": 8,
            "k_deterministic": prob.k_deterministic, "initial_source": "diffusion",
            "histories_per_step": prob.histories, "steps": active,
            "histories_per_s": d["histories"] / (d["ms"] / 1000.0),
            "collisions_per_s": d["collisions"] / (d["ms"] / 1000.0),
            "collisions_per_history": d["collisions"] / max(1, d["histories"]),
            "ms_per_step": d["ms"] / active, "k_mean": d["k_mean"], "sigma_k_pcm": d["k_sigma"] * 1e5,
            "achieved_GBs": ALG_BYTES_PER_COLLISION * coll_per_launch / (per_launch_ms / 1000.0) / 1e9
            if per_launch_ms > 0 else 0.0, "launch_shape": d["tuning"],
            "plain_fp64": {"generations": f"{prob.skip} + {plain_active}",
                           "histories_per_s": dp["histories"] / (dp["ms"] / 1000.0),
                           "collisions_per_s": dp["collisions"] / (dp["ms"] / 1000.0),
                           "ms_per_step": dp["ms"] / plain_active, "k_mean": dp["k_mean"],
                           "sigma_k_pcm": dp["k_sigma"] * 1e5},
            "event_vs_plain": {"generations": f"active {prob.skip}..{prob.skip + plain_active - 1} of both",
                               "k_event": me, "k_plain": mp, "delta_k_pcm": (me - mp) * 1e5,
                               "sigma_pcm": sig * 1e5, "z": (me - mp) / sig if sig > 0 else None,
                               "sigma_from": "batch means, 4 batches of 5 generations"},
            "uniform_source": {"k_mean": du["k_mean"], "sigma_k_pcm": du["k_sigma"] * 1e5,
                               "histories_per_s": du["histories"] / (du["ms"] / 1000.0)}}


def cpu_reference_rate(prob, budget_s: float, threads: int):
    """The reference algorithm on the host cores: COMPAT, f32 arithmetic and
    f32 tallies, T threads (histories split as src/mc_code.rs:300-307)."""
    from nraps_gb300 import abi
    from oracle import oracle as O
    o = abi.make_opts(seed=12345, mode=abi.MODE_COMPAT, precision=abi.PREC_FP32, compat_threads=threads)
    n = max(threads * 20, 1000)
    while True:
        q = prob.with_(histories=n, generations=2, skip=1)
        t = time.perf_counter()
        O.monte_carlo(q, o, threads=threads, acc64=False, max_generations=1)
        dt = time.perf_counter() - t
        if dt > 0.5 or n >= prob.histories:
            break
        n = min(prob.histories, n * 4)
    rate = n / dt
    n_sample = int(min(prob.histories, max(threads * 10, rate * budget_s)))
    return rate, n_sample


def run_reference_arm(args):
    from nraps_gb300 import abi
    from oracle import oracle as O
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    prob = make_workload(args.workload, args.seed, args.warmup, args.steps)
    threads = max(1, (os.cpu_count() or 2) - 1)
    per_step = max(0.05, min(1.0, args.reference_budget_s / max(1, args.steps + args.warmup)))
    rate, n = cpu_reference_rate(prob, per_step, threads)
    o = abi.make_opts(seed=12345, mode=abi.MODE_COMPAT, precision=abi.PREC_FP32, compat_threads=threads)
    q = prob.with_(histories=n, generations=2, skip=1)
    for _ in range(args.warmup):
        O.monte_carlo(q, o, threads=threads, acc64=False, max_generations=1)
    t = time.perf_counter()
    for _ in range(args.steps):
        O.monte_carlo(q, o, threads=threads, acc64=False, max_generations=1)
    dt = time.perf_counter() - t
    # the reference simulates N + T histories per generation (start..=end
    # per thread, src/mc_code.rs:226,302-307): all of them count as work
    hist = (n + threads) * args.steps
    value = hist / dt
    sample = (f"{args.steps} generations of {n}+{threads} histories sampled from {args.workload} "
              f"({prob.histories} histories per generation; COMPAT f32, CPU restatement of "
              f"src/mc_code.rs, the reference's thread policy)")
    world = int(os.environ.get("WORLD_SIZE", "1"))
    line = {"impl": "reference", "metric": "histories/s", "value": value, "unit": "histories/s",
            "n_gpus": 0, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": arm_config(args, prob, world),
            "form": "reference algorithm on the host cores (COMPAT, f32)",
            "cpu_baseline": {"value": value, "unit": "histories/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "histories/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=50)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="single_large")
    ap.add_argument("--arm", default="event", choices=["event", "plain"])
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--plain-steps", type=int, default=5)
    ap.add_argument("--cpu-budget-s", type=float, default=12.0)
    ap.add_argument("--reference-budget-s", type=float, default=120.0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline (profiling runs)")
    ap.add_argument("--batched-steps", type=int, default=10, help="timed generations of the 256-instance batch (0 = skip)")
    ap.add_argument("--batched-instances", type=int, default=256, help="instances of the batch (profiling a smaller case)")
    ap.add_argument("--batched-shape", type=str, default=None,
                    help="BLOCK,RANGE_LEN: fix the batch's launch shape (no autotuning)")
    ap.add_argument("--batched-warmup", type=int, default=3, help="untimed batch generations (at least 14 when autotuning)")
    ap.add_argument("--serve-seconds", type=float, default=60.0, help="Poisson arrival window of the serving run (config 3: 60 s; 0 = skip)")
    ap.add_argument("--serve-rate", type=float, default=200.0)
    ap.add_argument("--serve-sweep", default="400,800",
                    help="further Poisson rates (req/s) served for --serve-sweep-seconds each, up to and past "
                         "the saturation knee ('' = none)")
    ap.add_argument("--serve-sweep-seconds", type=float, default=10.0)
    ap.add_argument("--shape", type=lambda v: tuple(int(x) for x in v.split(",")), default=None,
                    help="block,events_per_pass,passes[,tail_lanes]: fixed event launch shape (profiling)")
    ap.add_argument("--sort", type=int, default=0, help="sorted transport with this many rounds (profiling)")
    ap.add_argument("--initial-source", type=int, default=0, help="1 = start from the diffusion fission source")
    ap.add_argument("--range", type=int, default=0, help="ranged launches of this many histories (profiling)")
    ap.add_argument("--scale-stress", type=int, default=1, help="1 = also run the 10M-history, 200k-cell slab")
    ap.add_argument("--histories", type=int, default=0,
                    help="histories per generation of the timed workload instead of its own (profiling)")
    ap.add_argument("--parity", type=int, default=1,
                    help="1 = event FP32 vs plain FP64 on the full workload (k, flux chi^2, time to 50 pcm)")
    ap.add_argument("--plain-small", type=int, default=1, help="1 = also run config 0 (CPU port vs plain FP64)")
    args = ap.parse_args()
    if args.warmup < 3:
        raise SystemExit("--warmup must be >= 3")
    if args.impl == "reference":
        return run_reference_arm(args)

    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    from nraps_gb300 import abi, api
    api.load()
    seed = replica_seed(args.seed, rank)
    prob = make_workload(args.workload, args.seed, args.warmup, args.steps)
    if args.histories:
        prob = prob.with_(histories=args.histories)

    # no fallback: if the chosen form cannot run, the bench fails
    arm = args.arm
    clocks = Clocks(local)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    extra = {}
    if args.initial_source:
        extra["initial_source"] = args.initial_source
    if args.range:
        extra["range_len"] = args.range
    d = measure_device(prob, arm, args.steps, args.warmup, seed, local, shape=args.shape, sort=args.sort,
                       extra=extra or None)
    ms = max_over_ranks(d["ms"], f"cuda:{local}")
    if world > 1:
        torch.distributed.barrier()
    value = replica_throughput(d["histories"], ms, world)

    # the plain FP64 history-per-thread kernel on the same workload, a few
    # generations (its throughput is the 10x target's denominator)
    plain = None
    if arm == "event" and args.plain_steps > 0:
        pp = prob.with_(generations=3 + args.plain_steps, skip=3)
        dp = measure_device(pp, "plain", args.plain_steps, 3, seed, local)
        plain = {"histories_per_s": dp["histories"] / (dp["ms"] / 1000.0),
                 "collisions_per_s": dp["collisions"] / (dp["ms"] / 1000.0),
                 "ms_per_step": dp["ms"] / args.plain_steps, "steps": args.plain_steps, "dtype": "f64",
                 "k_mean": dp["k_mean"], "sigma_k_pcm": dp["k_sigma"] * 1e5}

    full = full_workload(args.workload, args.seed)
    e2e = None
    e2e_k64 = None
    if not args.no_e2e:
        e = measure_e2e(full, arm, seed, local)
        e2e_k64 = e["k64"]
        e_sec = max_over_ranks(e["seconds"], f"cuda:{local}")
        e2e = {"value": replica_throughput(full.histories * full.generations, 1000.0 * e_sec, world),
               "unit": "histories/s", "h2d_bytes_per_step": e["h2d"],
               "d2h_bytes_per_step": e["d2h"], "seconds": e_sec, "call": "nraps_monte_carlo",
               "generations_per_call": e["generations"], "k_mean": e["k_mean"],
               "sigma_k_pcm": e["k_sigma"] * 1e5}

    fp = None
    if arm == "event" and args.parity and rank == 0:
        fp = measure_parity(full, seed, local, event_ms_per_generation=ms / args.steps,
                            plain_ms_per_generation=plain["ms_per_step"] if plain else None,
                            event_k64=e2e_k64)
        if plain:
            plain["k_mean"], plain["sigma_k_pcm"] = fp["k_plain_fp64"], fp["sigma_plain_fp64_pcm"]
            plain["k_from"] = f"fp32_vs_fp64 replicas ({fp['replicas']} x {fp['generations_per_replica']})"
    # the timed generations take a few milliseconds, shorter than the 200 ms
    # sampling period: the clock record spans the timed region and the GPU
    # work that follows it (plain kernel, drop-in calls, replicas)
    clk = clocks.stop()
    if clk:
        clk["window"] = "timed generations through the plain, e2e and fp32_vs_fp64 runs"

    peak, peak_kind = peaks()
    per_launch_ms = d["transport_ms"] / max(1, d["transport_launches"])
    coll_per_launch = d["collisions"] / max(1, d["transport_launches"])
    achieved = ALG_BYTES_PER_COLLISION * coll_per_launch / (per_launch_ms / 1000.0) / 1e9 if per_launch_ms > 0 else 0.0
    tpc = traffic_per_collision()
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_kind": peak_kind,
                "traffic": (tpc * coll_per_launch) if tpc else None,
                "traffic_source": ("DRAM bytes per real collision from the ncu capture in "
                                   "profiles/traffic_event_single_large.txt x this run's real collisions "
                                   "per launch") if tpc else None,
                "kernel": "event_transport" if arm == "event" else "plain_transport",
                "bytes_per_collision": ALG_BYTES_PER_COLLISION,
                "launches": d["transport_launches"], "avg_launch_ms": per_launch_ms}

    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = max(1, (os.cpu_count() or 2) - 1)
        from oracle import oracle as O
        o = abi.make_opts(seed=12345, mode=abi.MODE_COMPAT, precision=abi.PREC_FP32, compat_threads=threads)
        rate, n = cpu_reference_rate(prob, args.cpu_budget_s, threads)
        q = prob.with_(histories=n, generations=2, skip=1)
        t = time.perf_counter()
        O.monte_carlo(q, o, threads=threads, acc64=False, max_generations=1)
        dt = time.perf_counter() - t
        cpu = {"value": (n + threads) / dt, "unit": "histories/s", "cores": threads, "kind": "port",
               "sample": f"1 generation of {n}+{threads} histories of {args.workload}, COMPAT f32, "
                         f"CPU restatement of src/mc_code.rs (reference thread policy)"}

    small = (measure_plain_small(args.seed, local, max(1, (os.cpu_count() or 2) - 1))
             if args.plain_small and rank == 0 else None)
    bshape = tuple(int(x) for x in args.batched_shape.split(",")) if args.batched_shape else None
    batched = (measure_batched(args.seed, local, args.batched_steps, args.batched_warmup, args.batched_instances, bshape)
               if args.batched_steps > 0 and arm == "event" else None)
    scale = measure_scale_stress(args.seed, local) if args.scale_stress and arm == "event" else None
    serving = (measure_serving(args.seed, local, args.serve_seconds, args.serve_rate)
               if args.serve_seconds > 0 and arm == "event" else None)
    sweep = None
    if args.serve_seconds > 0 and arm == "event" and args.serve_sweep:
        # past the knee the queue grows without bound: the window's throughput
        # is the measure, and the drain after the window is capped at 10 s
        sweep = [measure_serving(args.seed, local, args.serve_sweep_seconds, float(r), drain_seconds=10.0)
                 for r in args.serve_sweep.split(",") if r]

    if rank == 0:
        line = {
            "metric": "histories/s", "value": value, "unit": "histories/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64" if arm == "event" else "f64", "data": "synthetic",
            "config": arm_config(args, prob, world),
            "form": "event Woodcock FP32 flights + FP64 tallies" if arm == "event"
            else "plain history-per-thread FP64",
            "sigma_k_pcm": d["k_sigma"] * 1e5, "k_mean": d["k_mean"],
            "collisions_per_s": world * d["collisions"] / (ms / 1000.0),
            "gpu_launches": d["launches"], "launch_shape": d["tuning"],
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "plain": plain, "clocks": clk,
            "fp32_vs_fp64": fp, "plain_small": small,
            "batched": batched, "serving": serving, "serving_sweep": sweep, "scale_stress": scale,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
