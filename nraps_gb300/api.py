"""Python mirror of NRAPS's Monte Carlo interface over the C ABI.

    process_input(path)              -> Input      (src/process_input.rs:85)
    mesh_gen(matid, variables, dx)   -> (mesh, fuel_indices)   (src/main.rs:85)
    monte_carlo(variables, xsdata, delta_x, meshid, fuel_indices, k_new)
                                     -> SolutionResults       (src/mc_code.rs:276)

Every call goes through libnraps_gb300.so; there is no CPU fallback.  If the
library cannot be loaded, or no CUDA device is present, the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from . import abi
from .abi import ProblemArrays, ResultArrays

_LIB = None


class NrapsError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"[{status}] {msg}")
        self.status = status


def lib_path() -> str:
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "libnraps_gb300.so")


def load(build_if_missing: bool = True):
    """Load (building first if needed) the CUDA library and declare its ABI."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not os.path.exists(path) and build_if_missing:
        from .build import build
        build()
    if not os.path.exists(path):
        raise NrapsError(abi.ERR_NO_DEVICE, f"libnraps_gb300.so not built at {path}")
    L = C.CDLL(path)
    P = C.POINTER
    vp = C.c_void_p
    L.nraps_opts_default.argtypes = [P(abi.Opts)]
    L.nraps_create.argtypes = [P(vp), P(abi.Opts)]
    L.nraps_destroy.argtypes = [vp]
    L.nraps_last_error.argtypes = [vp]
    L.nraps_last_error.restype = C.c_char_p
    L.nraps_set_opts.argtypes = [vp, P(abi.Opts)]
    L.nraps_get_opts.argtypes = [vp, P(abi.Opts)]
    L.nraps_launch_count.argtypes = [vp]
    L.nraps_launch_count.restype = C.c_uint64
    L.nraps_ctx_stream.argtypes = [vp]
    L.nraps_ctx_stream.restype = vp
    L.nraps_monte_carlo.argtypes = [vp, P(abi.Variables), P(abi.XSData), P(abi.DeltaX), P(abi.Mesh),
                                    P(C.c_uint64), C.c_uint64, C.c_float, P(abi.Result)]
    L.nraps_solve.argtypes = [vp, P(abi.Problem), P(abi.Result)]
    L.nraps_session_create.argtypes = [vp, P(abi.Problem), P(vp)]
    L.nraps_session_run.argtypes = [vp, C.c_uint64]
    L.nraps_session_sync.argtypes = [vp]
    L.nraps_session_flush.argtypes = [vp]
    L.nraps_session_results.argtypes = [vp, P(abi.Result)]
    L.nraps_session_generation.argtypes = [vp]
    L.nraps_session_generation.restype = C.c_uint64
    L.nraps_session_destroy.argtypes = [vp]
    L.nraps_session_set_profile.argtypes = [vp, C.c_int]
    L.nraps_session_timing.argtypes = [vp, P(C.c_double), P(C.c_double), P(C.c_uint64),
                                       P(C.c_uint64), P(C.c_uint64)]
    L.nraps_session_tuning.argtypes = [vp, P(C.c_uint32), P(C.c_uint32), P(C.c_uint32), P(C.c_uint32),
                                       P(C.c_uint32), P(C.c_uint32), P(C.c_uint32), P(C.c_float), C.c_uint32]
    L.nraps_trace_generation.argtypes = [vp, P(abi.Problem), C.c_uint64, C.c_double, vp, C.c_uint64,
                                         vp, C.c_uint64, P(C.c_double), vp, C.c_uint64,
                                         P(C.c_uint64), P(C.c_uint64)]
    L.nraps_pcg32_stream.argtypes = [vp, C.c_uint64, P(C.c_uint64), C.c_uint64, C.c_uint32, P(C.c_uint32)]
    L.nraps_log_eval.argtypes = [vp, P(C.c_double), C.c_uint64, P(C.c_double), P(C.c_float)]
    L.nraps_process_input.argtypes = [C.c_char_p, P(P(abi.Input))]
    L.nraps_process_input_text.argtypes = [C.c_char_p, C.c_uint64, P(P(abi.Input))]
    L.nraps_input_free.argtypes = [P(abi.Input)]
    L.nraps_mesh_gen.argtypes = [P(C.c_uint8), C.c_uint64, P(abi.Variables), P(abi.DeltaX),
                                 P(P(abi.MeshBuf))]
    L.nraps_meshbuf_free.argtypes = [P(abi.MeshBuf)]
    L.nraps_problem_view.argtypes = [P(abi.Input), P(abi.MeshBuf), P(abi.Problem)]
    L.nraps_batch_create.argtypes = [vp, P(abi.Problem), C.c_uint32, P(C.c_uint64), P(vp)]
    L.nraps_batch_run.argtypes = [vp, C.c_uint64]
    L.nraps_batch_sync.argtypes = [vp]
    L.nraps_batch_results.argtypes = [vp, C.c_uint32, P(abi.Result)]
    L.nraps_batch_timing.argtypes = [vp, P(C.c_double), P(C.c_uint64), P(C.c_uint64)]
    L.nraps_batch_tuning.argtypes = [vp, P(C.c_uint32), P(C.c_uint32), P(C.c_uint32), P(C.c_float), C.c_uint32]
    L.nraps_batch_size.argtypes = [vp]
    L.nraps_batch_size.restype = C.c_uint32
    L.nraps_batch_destroy.argtypes = [vp]
    L.nraps_server_opts_default.argtypes = [P(abi.ServerOpts)]
    L.nraps_server_create.argtypes = [vp, P(abi.ServerOpts), P(vp)]
    L.nraps_server_submit.argtypes = [vp, P(abi.Problem), C.c_uint64, P(C.c_uint64)]
    L.nraps_server_step.argtypes = [vp, P(C.c_uint32), P(C.c_uint32)]
    L.nraps_server_poll.argtypes = [vp, C.c_uint64, P(abi.Result), P(abi.RequestInfo)]
    L.nraps_server_release.argtypes = [vp, C.c_uint64]
    L.nraps_server_finished.argtypes = [vp, P(C.c_uint64), C.c_uint32, P(C.c_uint32)]
    L.nraps_server_stats.argtypes = [vp, P(C.c_uint64), P(C.c_uint64), P(C.c_uint32), P(C.c_uint32),
                                     P(C.c_double), P(C.c_uint64)]
    L.nraps_server_clock.argtypes = [vp]
    L.nraps_server_clock.restype = C.c_double
    L.nraps_server_destroy.argtypes = [vp]
    L.nraps_format_f32.argtypes = [C.c_float, C.c_char_p, C.c_uint64]
    L.nraps_format_f64.argtypes = [C.c_double, C.c_char_p, C.c_uint64]
    L.nraps_write_solution.argtypes = [C.c_char_p, P(abi.Result), C.c_uint32, C.c_uint64, C.c_uint64,
                                       C.c_double]
    L.nraps_run_input.argtypes = [vp, C.c_char_p, C.c_char_p, P(abi.Stats)]
    L.nraps_diffusion_solve.argtypes = [P(abi.Problem), C.c_uint64, P(C.c_float), P(C.c_float),
                                        P(abi.DiffusionInfo)]
    L.nraps_diffusion_source.argtypes = [P(abi.Problem), C.c_uint64, C.c_void_p, P(abi.DiffusionInfo)]
    L.nraps_status_string.argtypes = [C.c_int]
    L.nraps_status_string.restype = C.c_char_p
    _LIB = L
    return L


def _check(st: int, ctx=None):
    if st != abi.OK:
        L = load()
        msg = L.nraps_last_error(ctx).decode() if ctx is not None else L.nraps_last_error(None).decode()
        raise NrapsError(st, msg or L.nraps_status_string(st).decode())


# ---------------------------------------------------------------- front end --
@dataclass
class Input:
    """process_input's tuple: (Variables, XSData, matid, DeltaX, solution, solver)."""
    variables: abi.Variables
    delta_x: abi.DeltaX
    sigt: np.ndarray
    sigs: np.ndarray
    mu: np.ndarray
    siga: np.ndarray
    sigf: np.ndarray
    nut: np.ndarray
    chit: np.ndarray
    scat_matrix: np.ndarray
    inv_sigtr: np.ndarray
    matid: np.ndarray
    solution: bool
    solver: int


def _take(ptr, n, dtype):
    if n == 0:
        return np.zeros(0, dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


def _input_from(p) -> Input:
    s = p.contents
    v = abi.Variables.from_buffer_copy(s.variables)
    d = abi.DeltaX.from_buffer_copy(s.delta_x)
    return Input(v, d, _take(s.sigt, s.n_sigt, np.float32), _take(s.sigs, s.n_sigs, np.float32),
                 _take(s.mu, s.n_mu, np.float32), _take(s.siga, s.n_siga, np.float32),
                 _take(s.sigf, s.n_sigf, np.float32), _take(s.nut, s.n_nut, np.float32),
                 _take(s.chit, s.n_chit, np.float32), _take(s.scat_matrix, s.n_scat, np.float32),
                 _take(s.inv_sigtr, s.n_inv_sigtr, np.float32), _take(s.matid, s.n_matid, np.uint8),
                 bool(s.solution), int(s.solver))


def process_input(path: str = "./TestCaseC.txt") -> Input:
    """Parse an NRAPS input file exactly as src/process_input.rs does."""
    L = load()
    out = C.POINTER(abi.Input)()
    _check(L.nraps_process_input(path.encode(), C.byref(out)))
    try:
        return _input_from(out)
    finally:
        L.nraps_input_free(out)


def process_input_text(text: str | bytes) -> Input:
    L = load()
    b = text.encode() if isinstance(text, str) else text
    out = C.POINTER(abi.Input)()
    _check(L.nraps_process_input_text(b, len(b), C.byref(out)))
    try:
        return _input_from(out)
    finally:
        L.nraps_input_free(out)


@dataclass
class MeshArrays:
    matid: np.ndarray
    delta_x: np.ndarray
    mesh_left: np.ndarray
    mesh_right: np.ndarray

    def __len__(self):
        return int(self.matid.size)


def mesh_gen(matid, variables: abi.Variables, delta_x: abi.DeltaX):
    """src/main.rs:85-143: returns (MeshArrays, fuel_indices)."""
    L = load()
    m = np.ascontiguousarray(matid, np.uint8)
    out = C.POINTER(abi.MeshBuf)()
    _check(L.nraps_mesh_gen(m.ctypes.data_as(C.POINTER(C.c_uint8)), m.size, C.byref(variables),
                            C.byref(delta_x), C.byref(out)))
    try:
        s = out.contents
        mesh = MeshArrays(_take(s.matid, s.n_cells, np.uint8), _take(s.delta_x, s.n_cells, np.float32),
                          _take(s.mesh_left, s.n_cells, np.float32), _take(s.mesh_right, s.n_cells, np.float32))
        fuel = _take(s.fuel_indices, s.n_fuel, np.uint64)
        return mesh, fuel
    finally:
        L.nraps_meshbuf_free(out)


def problem_from_input(inp: Input, mesh: MeshArrays, fuel: np.ndarray, k_new: float = 1.0) -> ProblemArrays:
    v = inp.variables
    return ProblemArrays(
        mattypes=v.mattypes, energygroups=v.energygroups, generations=v.generations,
        histories=v.histories, skip=v.skip, sigt=inp.sigt, sigs=inp.sigs, mu=inp.mu, siga=inp.siga,
        sigf=inp.sigf, nut=inp.nut, chit=inp.chit, scat=inp.scat_matrix, matid=mesh.matid,
        delta_x=mesh.delta_x, mesh_left=mesh.mesh_left, mesh_right=mesh.mesh_right,
        fuel_indices=fuel, boundl=v.boundl, boundr=v.boundr, numass=v.numass, numrods=v.numrods,
        roddia=v.roddia, rodpitch=v.rodpitch, mpfr=v.mpfr, mpwr=v.mpwr,
        dx_fuel=inp.delta_x.fuel, dx_water=inp.delta_x.water, k_new=k_new, inv_sigtr=inp.inv_sigtr)


# ------------------------------------------------------------ output files --
def format_f32(v: float) -> str:
    """Rust `Display` text of an f32 (plot_solution's to_string())."""
    L = load()
    buf = C.create_string_buffer(64)
    n = L.nraps_format_f32(float(np.float32(v)), buf, 64)
    if n < 0:
        raise NrapsError(abi.ERR_INVALID, "format buffer too small")
    return buf.value.decode()


def format_f64(v: float) -> str:
    """Rust `Display` text of an f64."""
    L = load()
    buf = C.create_string_buffer(400)
    n = L.nraps_format_f64(float(v), buf, 400)
    if n < 0:
        raise NrapsError(abi.ERR_INVALID, "format buffer too small")
    return buf.value.decode()


def write_solution(res: ResultArrays, generations: int, assembly_length: float, out_dir: str = ".") -> None:
    """plot_solution (src/plot_solution.rs:7-58): vars.csv, interface.csv and
    k_eff.csv in out_dir."""
    L = load()
    rv = res.view()
    _check(L.nraps_write_solution(out_dir.encode(), C.byref(rv), res.G, res.cells, generations,
                                  float(assembly_length)))


def diffusion_solve(prob: ProblemArrays, max_iterations: int = 0):
    """nalgebra_method (src/discrete.rs:169-356) on the host: returns
    (flux[G, cells], assembly_average[G, cells], info dict)."""
    L = load()
    G, n = prob.energygroups, prob.n_cells
    flux = np.zeros(G * n, np.float32)
    avg = np.zeros(G * n, np.float32)
    info = abi.DiffusionInfo()
    pv = prob.view()
    _check(L.nraps_diffusion_solve(C.byref(pv), max_iterations, flux.ctypes.data_as(C.POINTER(C.c_float)),
                                   avg.ctypes.data_as(C.POINTER(C.c_float)), C.byref(info)))
    return (flux.reshape(G, n), avg.reshape(G, n),
            dict(k=info.k, iterations=info.iterations, converged=bool(info.converged),
                 delta_flux=info.delta_flux, delta_k=info.delta_k))


def diffusion_source(prob: ProblemArrays, n_sites: int) -> np.ndarray:
    """n_sites initial fission sites from the diffusion solution (SITE_DTYPE)."""
    L = load()
    out = np.zeros(n_sites, abi.SITE_DTYPE)
    pv = prob.view()
    _check(L.nraps_diffusion_source(C.byref(pv), n_sites, out.ctypes.data_as(C.c_void_p), None))
    return out


def run_input(input_path: str = "./TestCaseC.txt", out_dir: str = ".", ctx: "Context | None" = None):
    """The restored main dispatch without a context: only input files that
    select the deterministic solver run (Monte Carlo needs a Context)."""
    L = load()
    st = abi.Stats()
    h = ctx.h if ctx is not None else None
    _check(L.nraps_run_input(h, input_path.encode(), out_dir.encode(), C.byref(st)), h)
    return st


# ------------------------------------------------------------------ solver --
class Context:
    """One CUDA context handle (stream + options) of the engine."""

    def __init__(self, opts: abi.Opts | None = None, **kw):
        L = load()
        self._L = L
        self.opts = opts if opts is not None else abi.make_opts(**kw)
        h = C.c_void_p()
        _check(L.nraps_create(C.byref(h), C.byref(self.opts)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self._L.nraps_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_opts(self, opts: abi.Opts | None = None, **kw):
        self.opts = opts if opts is not None else abi.make_opts(**kw)
        _check(self._L.nraps_set_opts(self.h, C.byref(self.opts)), self.h)

    @property
    def launches(self) -> int:
        return int(self._L.nraps_launch_count(self.h))

    @property
    def stream_ptr(self) -> int:
        return int(self._L.nraps_ctx_stream(self.h) or 0)

    def solve(self, prob: ProblemArrays) -> ResultArrays:
        res = ResultArrays(prob.energygroups, prob.n_cells, prob.generations)
        pv, rv = prob.view(), res.view()
        _check(self._L.nraps_solve(self.h, C.byref(pv), C.byref(rv)), self.h)
        return res

    def monte_carlo(self, prob: ProblemArrays) -> ResultArrays:
        """The reference-shaped call (six arguments) through nraps_monte_carlo."""
        res = ResultArrays(prob.energygroups, prob.n_cells, prob.generations)
        pv, rv = prob.view(), res.view()
        _check(self._L.nraps_monte_carlo(self.h, C.byref(pv.variables), C.byref(pv.xsdata),
                                         C.byref(pv.delta_x), C.byref(pv.mesh), pv.fuel_indices,
                                         pv.n_fuel, pv.k_new, C.byref(rv)), self.h)
        return res

    def run_input(self, input_path: str = "./TestCaseC.txt", out_dir: str = ".") -> abi.Stats:
        """The restored main dispatch (src/main.rs:332-364): parse, mesh,
        Monte Carlo for Solution = 1, write the three CSV files."""
        st = abi.Stats()
        _check(self._L.nraps_run_input(self.h, input_path.encode(), out_dir.encode(), C.byref(st)), self.h)
        return st

    def session(self, prob: ProblemArrays) -> "Session":
        return Session(self, prob)

    def trace(self, prob: ProblemArrays, gen: int, k: float, sites_in=None, site_cap=None):
        """One generation with per-history records: (records, tally, sites, kq)."""
        N = prob.histories + (self.opts.compat_threads if self.opts.mode == abi.MODE_COMPAT else 0)
        rec = np.zeros(N, abi.RECORD_DTYPE)
        tally = np.zeros(prob.energygroups * prob.n_cells, np.float64)
        cap = site_cap if site_cap is not None else 4 * prob.histories + 64
        sites = np.zeros(cap, abi.SITE_DTYPE)
        n_out = C.c_uint64()
        kq = C.c_uint64()
        sin, n_in = None, 0
        if sites_in is not None and len(sites_in):
            sites_in = np.ascontiguousarray(sites_in, abi.SITE_DTYPE)
            sin, n_in = sites_in.ctypes.data_as(C.c_void_p), len(sites_in)
        pv = prob.view()
        _check(self._L.nraps_trace_generation(
            self.h, C.byref(pv), gen, k, sin, n_in, rec.ctypes.data_as(C.c_void_p), N,
            tally.ctypes.data_as(C.POINTER(C.c_double)), sites.ctypes.data_as(C.c_void_p), cap,
            C.byref(n_out), C.byref(kq)), self.h)
        return rec, tally, sites[: n_out.value].copy(), int(kq.value)

    def pcg32(self, seed: int, streams, per: int) -> np.ndarray:
        st = np.ascontiguousarray(streams, np.uint64)
        out = np.zeros(st.size * per, np.uint32)
        _check(self._L.nraps_pcg32_stream(self.h, seed, st.ctypes.data_as(C.POINTER(C.c_uint64)), st.size,
                                          per, out.ctypes.data_as(C.POINTER(C.c_uint32))), self.h)
        return out.reshape(st.size, per)

    def log_eval(self, x):
        x = np.ascontiguousarray(x, np.float64)
        o64 = np.zeros(x.size, np.float64)
        o32 = np.zeros(x.size, np.float32)
        _check(self._L.nraps_log_eval(self.h, x.ctypes.data_as(C.POINTER(C.c_double)), x.size,
                                      o64.ctypes.data_as(C.POINTER(C.c_double)),
                                      o32.ctypes.data_as(C.POINTER(C.c_float))), self.h)
        return o64, o32


class Session:
    """Device-resident problem: tables, tallies and banks stay in HBM."""

    def __init__(self, ctx: Context, prob: ProblemArrays):
        self.ctx, self.prob, self._L = ctx, prob, ctx._L
        self._pv = prob.view()
        h = C.c_void_p()
        _check(self._L.nraps_session_create(ctx.h, C.byref(self._pv), C.byref(h)), ctx.h)
        self.h = h

    def run(self, n: int):
        _check(self._L.nraps_session_run(self.h, n), self.ctx.h)

    def flush(self):
        """Enqueue a pending fold of the last generation (no wait)."""
        _check(self._L.nraps_session_flush(self.h), self.ctx.h)

    def sync(self):
        _check(self._L.nraps_session_sync(self.h), self.ctx.h)

    def set_profile(self, on: bool = True):
        _check(self._L.nraps_session_set_profile(self.h, int(on)), self.ctx.h)

    def timing(self):
        t, tot = C.c_double(), C.c_double()
        nl, coll, hist = C.c_uint64(), C.c_uint64(), C.c_uint64()
        _check(self._L.nraps_session_timing(self.h, C.byref(t), C.byref(tot), C.byref(nl), C.byref(coll),
                                            C.byref(hist)), self.ctx.h)
        return dict(transport_ms=t.value, total_ms=tot.value, transport_launches=nl.value,
                    collisions=coll.value, histories=hist.value)

    def tuning(self) -> dict:
        b, k, pa, t, po, rl, n = (C.c_uint32() for _ in range(7))
        ms = (C.c_float * 32)()
        _check(self._L.nraps_session_tuning(self.h, C.byref(b), C.byref(k), C.byref(pa), C.byref(t), C.byref(po),
                                            C.byref(rl), C.byref(n), ms, 32), self.ctx.h)
        return dict(block=b.value, events_per_pass=k.value, passes=pa.value, tail_lanes=t.value,
                    sort_rounds=po.value, range_len=rl.value, tried_ms=[ms[i] for i in range(min(n.value, 32))])

    @property
    def generation(self) -> int:
        return int(self._L.nraps_session_generation(self.h))

    def results(self) -> ResultArrays:
        p = self.prob
        res = ResultArrays(p.energygroups, p.n_cells, p.generations)
        rv = res.view()
        _check(self._L.nraps_session_results(self.h, C.byref(rv)), self.ctx.h)
        return res

    def close(self):
        if getattr(self, "h", None):
            self._L.nraps_session_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def monte_carlo(variables, xsdata, delta_x, meshid, fuel_indices, k_new=1.0, *, ctx: Context | None = None,
                **opts) -> ResultArrays:
    """Drop-in for monte_carlo(&variables, &xsdata, &deltax, &meshid, &fuel_indices, k_new).

    variables/delta_x are abi structures (as process_input returns them),
    xsdata is an `Input` (or any object with the XSData arrays), meshid a
    MeshArrays from mesh_gen.
    """
    inp = xsdata
    prob = ProblemArrays(
        mattypes=variables.mattypes, energygroups=variables.energygroups,
        generations=variables.generations, histories=variables.histories, skip=variables.skip,
        sigt=inp.sigt, sigs=inp.sigs, mu=inp.mu, siga=inp.siga, sigf=inp.sigf, nut=inp.nut,
        chit=inp.chit, scat=inp.scat_matrix, matid=meshid.matid, delta_x=meshid.delta_x,
        mesh_left=meshid.mesh_left, mesh_right=meshid.mesh_right, fuel_indices=fuel_indices,
        boundl=variables.boundl, boundr=variables.boundr, numass=variables.numass,
        numrods=variables.numrods, roddia=variables.roddia, rodpitch=variables.rodpitch,
        mpfr=variables.mpfr, mpwr=variables.mpwr, dx_fuel=delta_x.fuel, dx_water=delta_x.water,
        k_new=k_new, inv_sigtr=inp.inv_sigtr)
    own = ctx is None
    c = ctx or Context(**opts)
    try:
        return c.monte_carlo(prob)
    finally:
        if own:
            c.close()


class Batch:
    """Independent problems advancing together, one launch sequence per generation."""

    def __init__(self, ctx: Context, problems, seeds=None):
        self.ctx, self._L = ctx, ctx._L
        self.problems = list(problems)
        arr = (abi.Problem * len(self.problems))()
        for i, p in enumerate(self.problems):
            arr[i] = p.view()
        self._arr = arr
        sd = None
        if seeds is not None:
            self._seeds = np.ascontiguousarray(seeds, np.uint64)
            sd = self._seeds.ctypes.data_as(C.POINTER(C.c_uint64))
        h = C.c_void_p()
        _check(self._L.nraps_batch_create(ctx.h, arr, len(self.problems), sd, C.byref(h)), ctx.h)
        self.h = h

    def run(self, n: int):
        _check(self._L.nraps_batch_run(self.h, n), self.ctx.h)

    def sync(self):
        _check(self._L.nraps_batch_sync(self.h), self.ctx.h)

    def results(self, i: int) -> ResultArrays:
        p = self.problems[i]
        res = ResultArrays(p.energygroups, p.n_cells, p.generations)
        rv = res.view()
        _check(self._L.nraps_batch_results(self.h, i, C.byref(rv)), self.ctx.h)
        return res

    def tuning(self) -> dict:
        """Launch shape in use and the generation time of each tried shape."""
        b, rl, n = C.c_uint32(), C.c_uint32(), C.c_uint32()
        ms = (C.c_float * 32)()
        _check(self._L.nraps_batch_tuning(self.h, C.byref(b), C.byref(rl), C.byref(n), ms, 32), self.ctx.h)
        return dict(block=b.value, range_len=rl.value, tried_ms=[ms[i] for i in range(min(n.value, 32))])

    def timing(self) -> dict:
        ms, hist, coll = C.c_double(), C.c_uint64(), C.c_uint64()
        _check(self._L.nraps_batch_timing(self.h, C.byref(ms), C.byref(hist), C.byref(coll)), self.ctx.h)
        return dict(ms=ms.value, histories=hist.value, collisions=coll.value)

    def close(self):
        if getattr(self, "h", None):
            self._L.nraps_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching request loop for k-eigenvalue solves."""

    def __init__(self, ctx: Context, hbm_budget_bytes: int = 120 << 30, sigma_k_target: float = 50e-5,
                 min_active: int = 10, max_slots: int = 1024):
        self.ctx, self._L = ctx, ctx._L
        o = abi.ServerOpts()
        self._L.nraps_server_opts_default(C.byref(o))
        o.hbm_budget_bytes, o.sigma_k_target = hbm_budget_bytes, sigma_k_target
        o.min_active, o.max_slots = min_active, max_slots
        h = C.c_void_p()
        _check(self._L.nraps_server_create(ctx.h, C.byref(o), C.byref(h)), ctx.h)
        self.h = h
        self._problems = {}

    def submit(self, prob: ProblemArrays, seed: int) -> int:
        rid = C.c_uint64()
        pv = prob.view()
        _check(self._L.nraps_server_submit(self.h, C.byref(pv), seed, C.byref(rid)), self.ctx.h)
        self._problems[rid.value] = prob
        return rid.value

    def step(self):
        r, f = C.c_uint32(), C.c_uint32()
        _check(self._L.nraps_server_step(self.h, C.byref(r), C.byref(f)), self.ctx.h)
        return r.value, f.value

    def finished(self, cap: int = 4096) -> list:
        """Ids of requests retired since the last call, oldest first."""
        ids = (C.c_uint64 * cap)()
        n = C.c_uint32()
        _check(self._L.nraps_server_finished(self.h, ids, cap, C.byref(n)), self.ctx.h)
        return [ids[i] for i in range(n.value)]

    def poll(self, rid: int, results: bool = True):
        """(status, info dict, ResultArrays or None); status ERR_PENDING while running."""
        info = abi.RequestInfo()
        res = None
        rv_struct = None
        if results:
            p = self._problems[rid]
            res = ResultArrays(p.energygroups, p.n_cells, p.generations)
            rv_struct = res.view()
        st = self._L.nraps_server_poll(self.h, rid, C.byref(rv_struct) if rv_struct is not None else None,
                                       C.byref(info))
        d = {f: getattr(info, f) for f, _ in abi.RequestInfo._fields_}
        if st not in (abi.OK, abi.ERR_PENDING, abi.ERR_CAPPED):
            _check(st, self.ctx.h)
        return st, d, (res if st in (abi.OK, abi.ERR_CAPPED) else None)

    def release(self, rid: int):
        _check(self._L.nraps_server_release(self.h, rid), self.ctx.h)
        self._problems.pop(rid, None)

    def stats(self) -> dict:
        h, c, b = C.c_uint64(), C.c_uint64(), C.c_uint64()
        r, w = C.c_uint32(), C.c_uint32()
        ms = C.c_double()
        _check(self._L.nraps_server_stats(self.h, C.byref(h), C.byref(c), C.byref(r), C.byref(w), C.byref(ms),
                                          C.byref(b)), self.ctx.h)
        return dict(histories=h.value, completed=c.value, running=r.value, waiting=w.value, busy_ms=ms.value,
                    bytes_in_use=b.value)

    @property
    def clock(self) -> float:
        return float(self._L.nraps_server_clock(self.h))

    def close(self):
        if getattr(self, "h", None):
            self._L.nraps_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
