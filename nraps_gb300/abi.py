"""ctypes mirrors of the C ABI in include/nraps_gpu.h.

The structures here are the ABI itself (field order and widths match the
header); the product wrapper (nraps_gb300.api) and the CPU oracle loader both
use them.  `ProblemArrays` owns the numpy arrays behind an `nraps_problem`
view so the pointers stay valid for as long as the object lives.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

ABI_VERSION = 6

OK = 0
ERR_INVALID = 1
ERR_CUDA = 2
ERR_NOMEM = 3
ERR_NO_DEVICE = 4
ERR_IO = 5
ERR_PARSE = 6
ERR_CAPACITY = 7
ERR_EMPTY_BANK = 8
ERR_NOT_FOUND = 9
ERR_PENDING = 10
ERR_CAPPED = 11
ERR_REJECTED = 12
ERR_UNSUPPORTED = 13

ONE_PASS = 0xFFFFFFFF  # events_per_pass: a single transport pass

MODE_COMPAT, MODE_PHYSICS, MODE_BANK = 0, 1, 2
PREC_FP64, PREC_FP32 = 0, 1
TRACK_SURFACE, TRACK_WOODCOCK = 0, 1
FATE_ABSORBED, FATE_LEAKED, FATE_CAPPED = 0, 1, 2

_f32p = C.POINTER(C.c_float)
_f64p = C.POINTER(C.c_double)
_u8p = C.POINTER(C.c_uint8)
_u64p = C.POINTER(C.c_uint64)


class Opts(C.Structure):
    _fields_ = [
        ("abi_version", C.c_uint32), ("device", C.c_int32), ("seed", C.c_uint64),
        ("mode", C.c_int32), ("precision", C.c_int32), ("tracking", C.c_int32),
        ("compat_threads", C.c_uint32), ("max_events", C.c_uint64),
        ("block_size", C.c_uint32), ("events_per_pass", C.c_uint32),
        ("passes", C.c_uint32), ("use_graphs", C.c_uint32),
        ("bank_factor", C.c_double), ("entropy_bins", C.c_uint32),
        ("exact_log", C.c_uint32), ("tail_lanes", C.c_uint32), ("sort_rounds", C.c_uint32),
        ("initial_source", C.c_uint32), ("range_len", C.c_uint32), ("reserved", C.c_uint32 * 2),
    ]


def make_opts(*, seed=1, mode=MODE_COMPAT, precision=PREC_FP64, tracking=TRACK_SURFACE,
              compat_threads=0, max_events=0, block_size=0, events_per_pass=0, passes=0,
              use_graphs=0, bank_factor=0.0, entropy_bins=0, exact_log=0, device=-1, tail_lanes=0,
              sort_rounds=0, initial_source=0, range_len=0) -> Opts:
    o = Opts()
    o.abi_version = ABI_VERSION
    o.device = device
    o.seed = seed
    o.mode = mode
    o.precision = precision
    o.tracking = tracking
    o.compat_threads = compat_threads
    o.max_events = max_events
    o.block_size = block_size
    o.events_per_pass = events_per_pass
    o.passes = passes
    o.use_graphs = use_graphs
    o.bank_factor = bank_factor
    o.entropy_bins = entropy_bins
    o.exact_log = exact_log
    o.tail_lanes = tail_lanes
    o.sort_rounds = sort_rounds
    o.initial_source = initial_source
    o.range_len = range_len
    return o


class Variables(C.Structure):
    _fields_ = [
        ("analk", C.c_uint32), ("mattypes", C.c_uint32), ("energygroups", C.c_uint32),
        ("generations", C.c_uint64), ("histories", C.c_uint64), ("skip", C.c_uint64),
        ("numass", C.c_uint32), ("numrods", C.c_uint32),
        ("roddia", C.c_float), ("rodpitch", C.c_float),
        ("mpfr", C.c_uint64), ("mpwr", C.c_uint64),
        ("boundl", C.c_float), ("boundr", C.c_float),
    ]


class DeltaX(C.Structure):
    _fields_ = [("fuel", C.c_float), ("water", C.c_float)]


class XSData(C.Structure):
    _fields_ = [
        ("sigt", _f32p), ("sigs", _f32p), ("mu", _f32p), ("siga", _f32p),
        ("sigf", _f32p), ("nut", _f32p), ("chit", _f32p),
        ("scat_matrix", _f32p), ("inv_sigtr", _f32p),
        ("n_xs", C.c_uint64), ("n_scat", C.c_uint64),
    ]


class Mesh(C.Structure):
    _fields_ = [("matid", _u8p), ("delta_x", _f32p), ("mesh_left", _f32p),
                ("mesh_right", _f32p), ("n_cells", C.c_uint64)]


class Problem(C.Structure):
    _fields_ = [("variables", Variables), ("xsdata", XSData), ("delta_x", DeltaX),
                ("mesh", Mesh), ("fuel_indices", _u64p), ("n_fuel", C.c_uint64),
                ("k_new", C.c_float)]


class DiffusionInfo(C.Structure):
    _fields_ = [("k", C.c_double), ("iterations", C.c_uint64), ("converged", C.c_int32), ("pad", C.c_int32),
                ("delta_flux", C.c_double), ("delta_k", C.c_double)]


class Stats(C.Structure):
    _fields_ = [
        ("k_mean", C.c_double), ("k_sigma", C.c_double),
        ("histories", C.c_uint64), ("collisions", C.c_uint64),
        ("virtual_collisions", C.c_uint64), ("crossings", C.c_uint64),
        ("absorbed", C.c_uint64), ("leaked", C.c_uint64), ("capped", C.c_uint64),
        ("sites", C.c_uint64),
        ("transport_ms", C.c_double), ("total_ms", C.c_double),
        ("transport_launches", C.c_uint64), ("gpu_launches", C.c_uint64),
    ]


class Result(C.Structure):
    _fields_ = [
        ("flux", _f32p), ("assembly_average", _f32p), ("fission_source", _f32p),
        ("k", _f32p), ("k_fund", _f32p),
        ("k64", _f64p), ("entropy", _f64p), ("flux_mean", _f64p), ("flux_sem", _f64p),
        ("stats", C.POINTER(Stats)),
    ]


class HistoryRecord(C.Structure):
    _fields_ = [
        ("collisions", C.c_uint32), ("crossings", C.c_uint32), ("reflections", C.c_uint32),
        ("segments", C.c_uint32), ("fate", C.c_int32), ("final_cell", C.c_uint32),
        ("final_group", C.c_uint32), ("n_sites", C.c_uint32),
        ("final_x", C.c_double), ("track", C.c_double), ("nsf_track", C.c_double),
        ("draws", C.c_uint64),
    ]


RECORD_DTYPE = np.dtype([
    ("collisions", "<u4"), ("crossings", "<u4"), ("reflections", "<u4"), ("segments", "<u4"),
    ("fate", "<i4"), ("final_cell", "<u4"), ("final_group", "<u4"), ("n_sites", "<u4"),
    ("final_x", "<f8"), ("track", "<f8"), ("nsf_track", "<f8"), ("draws", "<u8"),
])
assert RECORD_DTYPE.itemsize == C.sizeof(HistoryRecord) == 64


class Site(C.Structure):
    _fields_ = [("x", C.c_float), ("cell", C.c_uint32), ("group", C.c_uint32), ("pad", C.c_uint32)]


SITE_DTYPE = np.dtype([("x", "<f4"), ("cell", "<u4"), ("group", "<u4"), ("pad", "<u4")])


class Input(C.Structure):
    _fields_ = [
        ("variables", Variables), ("delta_x", DeltaX),
        ("sigt", _f32p), ("sigs", _f32p), ("mu", _f32p), ("siga", _f32p), ("sigf", _f32p),
        ("nut", _f32p), ("chit", _f32p), ("scat_matrix", _f32p), ("inv_sigtr", _f32p),
        ("n_sigt", C.c_uint64), ("n_sigs", C.c_uint64), ("n_mu", C.c_uint64),
        ("n_siga", C.c_uint64), ("n_sigf", C.c_uint64), ("n_nut", C.c_uint64),
        ("n_chit", C.c_uint64), ("n_scat", C.c_uint64), ("n_inv_sigtr", C.c_uint64),
        ("matid", _u8p), ("n_matid", C.c_uint64),
        ("solution", C.c_int32), ("solver", C.c_int32),
    ]


class MeshBuf(C.Structure):
    _fields_ = [("matid", _u8p), ("delta_x", _f32p), ("mesh_left", _f32p),
                ("mesh_right", _f32p), ("n_cells", C.c_uint64),
                ("fuel_indices", _u64p), ("n_fuel", C.c_uint64)]


def _ptr(a: np.ndarray, ct):
    return a.ctypes.data_as(C.POINTER(ct))


@dataclass
class ProblemArrays:
    """Owner of one slab problem in the reference's layout.

    xs arrays are flat [m + M*g]; scat is [G*G*m + G*g + g']; the mesh is the
    Vec<Mesh> of mesh_gen as four arrays.
    """
    mattypes: int
    energygroups: int
    generations: int
    histories: int
    skip: int
    sigt: np.ndarray
    sigs: np.ndarray
    mu: np.ndarray
    siga: np.ndarray
    sigf: np.ndarray
    nut: np.ndarray
    chit: np.ndarray
    scat: np.ndarray
    matid: np.ndarray
    delta_x: np.ndarray
    mesh_left: np.ndarray
    mesh_right: np.ndarray
    fuel_indices: np.ndarray
    boundl: float = 0.0
    boundr: float = 0.0
    numass: int = 1
    numrods: int = 0
    roddia: float = 1.0
    rodpitch: float = 1.5
    mpfr: int = 1
    mpwr: int = 1
    dx_fuel: float = 0.05
    dx_water: float = 0.05
    k_new: float = 1.0
    inv_sigtr: np.ndarray | None = None
    name: str = ""
    k_deterministic: float | None = None
    input_matid: np.ndarray | None = None
    _keep: list = field(default_factory=list, repr=False)

    def __post_init__(self):
        f32 = lambda a: np.ascontiguousarray(a, dtype=np.float32)
        for n in ("sigt", "sigs", "mu", "siga", "sigf", "nut", "chit", "scat",
                  "delta_x", "mesh_left", "mesh_right"):
            setattr(self, n, f32(getattr(self, n)))
        self.matid = np.ascontiguousarray(self.matid, dtype=np.uint8)
        self.fuel_indices = np.ascontiguousarray(self.fuel_indices, dtype=np.uint64)
        if self.inv_sigtr is None:
            # 1/(sigt - mu*sigs) in f32, as process_input.rs:152-156
            self.inv_sigtr = (np.float32(1.0) / (self.sigt - self.mu * self.sigs)).astype(np.float32)
        self.inv_sigtr = f32(self.inv_sigtr)
        M, G = self.mattypes, self.energygroups
        assert self.sigt.size == M * G and self.scat.size == M * G * G
        assert self.matid.size == self.delta_x.size == self.mesh_left.size == self.mesh_right.size

    @property
    def n_cells(self) -> int:
        return int(self.matid.size)

    def view(self) -> Problem:
        p = Problem()
        v = p.variables
        v.analk = 1
        v.mattypes = self.mattypes
        v.energygroups = self.energygroups
        v.generations = self.generations
        v.histories = self.histories
        v.skip = self.skip
        v.numass = self.numass
        v.numrods = self.numrods
        v.roddia = self.roddia
        v.rodpitch = self.rodpitch
        v.mpfr = self.mpfr
        v.mpwr = self.mpwr
        v.boundl = self.boundl
        v.boundr = self.boundr
        x = p.xsdata
        x.sigt, x.sigs, x.mu = _ptr(self.sigt, C.c_float), _ptr(self.sigs, C.c_float), _ptr(self.mu, C.c_float)
        x.siga, x.sigf, x.nut = _ptr(self.siga, C.c_float), _ptr(self.sigf, C.c_float), _ptr(self.nut, C.c_float)
        x.chit, x.scat_matrix = _ptr(self.chit, C.c_float), _ptr(self.scat, C.c_float)
        x.inv_sigtr = _ptr(self.inv_sigtr, C.c_float)
        x.n_xs = self.sigt.size
        x.n_scat = self.scat.size
        p.delta_x.fuel = self.dx_fuel
        p.delta_x.water = self.dx_water
        m = p.mesh
        m.matid = _ptr(self.matid, C.c_uint8)
        m.delta_x = _ptr(self.delta_x, C.c_float)
        m.mesh_left = _ptr(self.mesh_left, C.c_float)
        m.mesh_right = _ptr(self.mesh_right, C.c_float)
        m.n_cells = self.n_cells
        p.fuel_indices = _ptr(self.fuel_indices, C.c_uint64)
        p.n_fuel = self.fuel_indices.size
        p.k_new = self.k_new
        return p

    def with_(self, **kw) -> "ProblemArrays":
        d = {f: getattr(self, f) for f in self.__dataclass_fields__ if f != "_keep"}
        d.update(kw)
        return ProblemArrays(**d)


class ResultArrays:
    """Caller-allocated SolutionResults buffers plus the FP64 extras."""

    def __init__(self, G: int, cells: int, generations: int):
        self.flux = np.zeros(G * cells, np.float32)
        self.assembly_average = np.zeros(G * cells, np.float32)
        self.fission_source = np.zeros(cells, np.float32)
        self.k = np.zeros(generations, np.float32)
        self.k_fund = np.zeros(generations, np.float32)
        self.k64 = np.zeros(generations, np.float64)
        self.entropy = np.zeros(generations, np.float64)
        self.flux_mean = np.zeros(G * cells, np.float64)
        self.flux_sem = np.zeros(G * cells, np.float64)
        self.stats = Stats()
        self.G, self.cells = G, cells

    def view(self) -> Result:
        r = Result()
        r.flux = _ptr(self.flux, C.c_float)
        r.assembly_average = _ptr(self.assembly_average, C.c_float)
        r.fission_source = _ptr(self.fission_source, C.c_float)
        r.k = _ptr(self.k, C.c_float)
        r.k_fund = _ptr(self.k_fund, C.c_float)
        r.k64 = _ptr(self.k64, C.c_double)
        r.entropy = _ptr(self.entropy, C.c_double)
        r.flux_mean = _ptr(self.flux_mean, C.c_double)
        r.flux_sem = _ptr(self.flux_sem, C.c_double)
        r.stats = C.pointer(self.stats)
        return r

    def flux2d(self):
        return self.flux.reshape(self.G, self.cells)


REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_REJECTED = 0, 1, 2, 3


class ServerOpts(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("sigma_k_target", C.c_double),
                ("min_active", C.c_uint32), ("max_slots", C.c_uint32), ("reserved", C.c_uint32 * 4)]


class RequestInfo(C.Structure):
    _fields_ = [("id", C.c_uint64), ("state", C.c_int32), ("status", C.c_int32),
                ("generations_run", C.c_uint64), ("histories_per_generation", C.c_uint64),
                ("k_mean", C.c_double), ("k_sigma", C.c_double),
                ("t_submit", C.c_double), ("t_admit", C.c_double), ("t_done", C.c_double)]
