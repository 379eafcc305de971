"""ctypes loader for the CPU oracle library (test infrastructure only).

The oracle restates NRAPS's src/mc_code.rs and src/rand.rs on the CPU (see
oracle/nraps_oracle.cpp for the line-by-line citations).  The CUDA path is
checked against it, and it is the timed stand-in for the reference CPU solver.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from nraps_gb300 import abi
from oracle.build import build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build()
        L = C.CDLL(path)
        f32p, f64p, u32p, u64p = (C.POINTER(C.c_float), C.POINTER(C.c_double),
                                  C.POINTER(C.c_uint32), C.POINTER(C.c_uint64))
        L.oracle_hit_boundary.argtypes = [C.c_float] * 5 + [f32p]
        L.oracle_cross_mesh.argtypes = [C.c_uint64, C.c_float, C.c_float, C.c_float, C.c_float, f32p, u64p]
        L.oracle_direction.argtypes = [C.c_float]
        L.oracle_direction.restype = C.c_float
        L.oracle_scat_mat_calc.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_float, f32p, f32p]
        L.oracle_energy_cdf.argtypes = [f32p, C.c_uint32, C.c_float]
        L.oracle_energy_cdf.restype = C.c_uint32
        L.oracle_partition_fresh.argtypes = [f32p, C.c_uint32, C.c_uint64, C.c_uint64, u32p]
        L.oracle_partition_fresh.restype = C.c_uint32
        L.oracle_pcg32.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32, u32p]
        L.oracle_generation_seed.argtypes = [C.c_uint64, C.c_uint64]
        L.oracle_generation_seed.restype = C.c_uint64
        L.oracle_log.argtypes = [C.c_double]
        L.oracle_log.restype = C.c_double
        L.oracle_logf.argtypes = [C.c_float]
        L.oracle_logf.restype = C.c_float
        L.oracle_trace_generation.argtypes = [
            C.POINTER(abi.Problem), C.POINTER(abi.Opts), C.c_uint64, C.c_double,
            C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64, f64p, C.c_void_p, C.c_uint64,
            u64p, u64p]
        L.oracle_monte_carlo.argtypes = [C.POINTER(abi.Problem), C.POINTER(abi.Opts), C.c_uint32,
                                         C.c_int, C.c_uint64, C.POINTER(abi.Result)]
        L.oracle_hardware_threads.restype = C.c_uint
        L.oracle_trace_woodcock.argtypes = L.oracle_trace_generation.argtypes
        _lib = L
    return _lib


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def hit_boundary(mu, start_x, delta_s, bound, mesh_end):
    out = np.zeros(3, np.float32)
    lib().oracle_hit_boundary(mu, start_x, delta_s, bound, mesh_end, _fp(out))
    return tuple(out)


def cross_mesh(mesh_index, mu, start_x, mesh_end, delta_s):
    out = np.zeros(2, np.float32)
    idx = C.c_uint64()
    lib().oracle_cross_mesh(mesh_index, mu, start_x, mesh_end, delta_s, _fp(out), C.byref(idx))
    return float(out[0]), float(out[1]), int(idx.value)


def direction(r):
    return np.float32(lib().oracle_direction(r))


def scat_mat_calc(G, matid, g, inv_sigs, scat):
    scat = np.ascontiguousarray(scat, np.float32)
    out = np.zeros(G, np.float32)
    lib().oracle_scat_mat_calc(G, matid, g, np.float32(inv_sigs), _fp(scat), _fp(out))
    return out


def energy_cdf(cdf, chi):
    cdf = np.ascontiguousarray(cdf, np.float32)
    return int(lib().oracle_energy_cdf(_fp(cdf), cdf.size, np.float32(chi)))


def partition_fresh(cdf, seed, stream):
    cdf = np.ascontiguousarray(cdf, np.float32)
    d = C.c_uint32()
    i = lib().oracle_partition_fresh(_fp(cdf), cdf.size, seed, stream, C.byref(d))
    return int(i), int(d.value)


def pcg32(seed, stream, n):
    out = np.zeros(n, np.uint32)
    lib().oracle_pcg32(seed, stream, n, out.ctypes.data_as(C.POINTER(C.c_uint32)))
    return out


def generation_seed(base, gen):
    return int(lib().oracle_generation_seed(base, gen))


def log64(x):
    return lib().oracle_log(x)


def log32(x):
    return np.float32(lib().oracle_logf(np.float32(x)))


def trace_generation(prob: abi.ProblemArrays, opts: abi.Opts, gen: int, k: float,
                     sites_in=None, site_cap=None):
    """One generation, histories in id order: (records, tally, sites, kq)."""
    N = prob.histories + (opts.compat_threads if opts.mode == abi.MODE_COMPAT else 0)
    rec = np.zeros(N, abi.RECORD_DTYPE)
    tally = np.zeros(prob.energygroups * prob.n_cells, np.float64)
    cap = site_cap if site_cap is not None else 4 * prob.histories + 64
    sites = np.zeros(cap, abi.SITE_DTYPE)
    n_out = C.c_uint64()
    kq = C.c_uint64()
    pv = prob.view()
    sin = None
    n_in = 0
    if sites_in is not None and len(sites_in):
        sites_in = np.ascontiguousarray(sites_in, abi.SITE_DTYPE)
        sin = sites_in.ctypes.data_as(C.c_void_p)
        n_in = len(sites_in)
    st = lib().oracle_trace_generation(
        C.byref(pv), C.byref(opts), gen, k, sin, n_in,
        rec.ctypes.data_as(C.c_void_p), N, tally.ctypes.data_as(C.POINTER(C.c_double)),
        sites.ctypes.data_as(C.c_void_p), cap, C.byref(n_out), C.byref(kq))
    if st != 0:
        raise RuntimeError(f"oracle_trace_generation failed: {st}")
    return rec, tally, sites[: n_out.value].copy(), int(kq.value)


def monte_carlo(prob: abi.ProblemArrays, opts: abi.Opts, threads: int = 1, acc64: bool = True,
                max_generations: int = 0) -> abi.ResultArrays:
    res = abi.ResultArrays(prob.energygroups, prob.n_cells, prob.generations)
    pv = prob.view()
    rv = res.view()
    st = lib().oracle_monte_carlo(C.byref(pv), C.byref(opts), threads, int(acc64),
                                  max_generations, C.byref(rv))
    if st != 0:
        raise RuntimeError(f"oracle_monte_carlo failed: {st}")
    return res


def hardware_threads() -> int:
    return int(lib().oracle_hardware_threads())


def trace_woodcock(prob: abi.ProblemArrays, opts: abi.Opts, gen: int, k: float, sites_in=None, site_cap=None):
    """One event-form (Woodcock, exact_log) generation: (records, tally, sites, kq)."""
    N = prob.histories
    rec = np.zeros(N, abi.RECORD_DTYPE)
    tally = np.zeros(prob.energygroups * prob.n_cells, np.float64)
    cap = site_cap if site_cap is not None else 4 * prob.histories + 64
    sites = np.zeros(cap, abi.SITE_DTYPE)
    n_out = C.c_uint64()
    kq = C.c_uint64()
    pv = prob.view()
    sin, n_in = None, 0
    if sites_in is not None and len(sites_in):
        sites_in = np.ascontiguousarray(sites_in, abi.SITE_DTYPE)
        sin, n_in = sites_in.ctypes.data_as(C.c_void_p), len(sites_in)
    st = lib().oracle_trace_woodcock(
        C.byref(pv), C.byref(opts), gen, k, sin, n_in, rec.ctypes.data_as(C.c_void_p), N,
        tally.ctypes.data_as(C.POINTER(C.c_double)), sites.ctypes.data_as(C.c_void_p), cap,
        C.byref(n_out), C.byref(kq))
    if st != 0:
        raise RuntimeError(f"oracle_trace_woodcock failed: {st}")
    return rec, tally, sites[: n_out.value].copy(), int(kq.value)
