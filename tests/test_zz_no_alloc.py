"""The entry point that allocates nothing, against the existing entry point.

Callers that cannot allocate device memory at call time (their device memory
is all handed out by their own pool, or laid out in advance) pass the problem
already on the device and receive the tally and k in their own buffers; the
library keeps its working state in a fixed array.  This file is collected
last so that a run stopping at the first failure has run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from nraps_gb300 import abi, api, synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu


class DeviceProblem(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("sigt", "sigs", "mu", "siga", "sigf", "nut", "chit",
                                           "scat_matrix", "inv_sigtr", "matid", "delta_x",
                                           "mesh_left", "mesh_right", "fuel_indices")] + [
        ("mattypes", C.c_uint32), ("energygroups", C.c_uint32), ("n_cells", C.c_uint64),
        ("n_fuel", C.c_uint64), ("histories", C.c_uint64), ("boundl", C.c_float), ("boundr", C.c_float)]


def _entry():
    L = api.load()
    f = L.nraps_physics_generation_noalloc
    f.argtypes = [C.POINTER(DeviceProblem), C.c_uint64, C.c_uint64, C.c_uint64, C.c_void_p, C.c_void_p,
                  C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return L, f


def _device_problem(p, torch, dev):
    keep = {}
    for name, arr in (("sigt", p.sigt), ("sigs", p.sigs), ("mu", p.mu), ("siga", p.siga), ("sigf", p.sigf),
                      ("nut", p.nut), ("chit", p.chit), ("scat_matrix", p.scat), ("inv_sigtr", p.inv_sigtr),
                      ("matid", p.matid), ("delta_x", p.delta_x), ("mesh_left", p.mesh_left),
                      ("mesh_right", p.mesh_right), ("fuel_indices", p.fuel_indices.astype(np.int64))):
        keep[name] = torch.from_numpy(np.ascontiguousarray(arr)).to(dev)
    dp = DeviceProblem(**{k: v.data_ptr() for k, v in keep.items()})
    dp.mattypes, dp.energygroups = p.mattypes, p.energygroups
    dp.n_cells, dp.n_fuel, dp.histories = p.n_cells, p.fuel_indices.size, p.histories
    dp.boundl, dp.boundr = p.boundl, p.boundr
    return dp, keep


def _anisotropic(p):
    """The same slab with mu-bar = 0.1 in the fuel and 0.2 in the water:
    inv_sigtr and the within-group scatter change (mu*sigs correction)."""
    M, G = p.mattypes, p.energygroups
    mu = np.zeros(M * G, np.float32)
    for g in range(G):
        mu[0 + M * g], mu[1 + M * g], mu[2 + M * g] = 0.1, 0.1, 0.2
    return p.with_(mu=mu, inv_sigtr=None)


@pytest.mark.parametrize("aniso", [False, True], ids=["isotropic", "mu_bar"])
def test_no_alloc_generation_matches_existing_entry_point(ctx_factory, aniso):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    torch.cuda.set_device(0)
    L, fn = _entry()
    p = synth.plain_small(5).with_(histories=6000, generations=8, skip=2)
    if aniso:
        p = _anisotropic(p)
    dp, keep = _device_problem(p, torch, dev)
    tally = torch.zeros(p.energygroups * p.n_cells, dtype=torch.float64, device=dev)
    k = torch.zeros(1, dtype=torch.float64, device=dev)
    err = torch.full((1,), -1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    seed = 2024
    ref = ctx_factory(seed=seed, mode=abi.MODE_PHYSICS, precision=abi.PREC_FP32)
    for gen in (3, 4):                      # two calls in a row share the fixed array
        st = fn(C.byref(dp), seed, gen, 0, tally.data_ptr(), k.data_ptr(), err.data_ptr(), stream)
        assert st == 0, L.nraps_last_error(None).decode()
        torch.cuda.synchronize(dev)
        _, want_tally, _, kq = ref.trace(p, gen, 1.0)
        np.testing.assert_allclose(tally.cpu().numpy(), want_tally, rtol=1e-12, atol=0)
        assert float(k.item()) == (kq * 2.0 ** -32) / p.histories
        assert int(err.item()) == 0
        # and against the CPU oracle directly (FP64 tally sums differ only in order)
        _, o_tally, _, o_kq = O.trace_generation(p, ref.opts, gen, 1.0)
        np.testing.assert_allclose(tally.cpu().numpy(), o_tally, rtol=1e-12, atol=0)
        assert o_kq == kq


def test_no_alloc_device_input_checks(ctx_factory):
    """Inputs that would index out of range are caught on the device before
    any transport kernel runs; a valid call afterwards still matches (the
    check's flags start from zero on every call)."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    torch.cuda.set_device(0)
    L, fn = _entry()
    p = synth.plain_small(6).with_(histories=3000)
    seed, gen = 77, 2
    out = torch.zeros(p.energygroups * p.n_cells, dtype=torch.float64, device=dev)
    k = torch.zeros(1, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    bad_mat = p.matid.copy()
    bad_mat[7] = p.mattypes                     # one material index equal to MatTypes
    bad_fuel = p.fuel_indices.copy()
    bad_fuel[3] = p.n_cells                     # one fuel index equal to n_cells
    for q, text in ((p.with_(matid=bad_mat), "matid"), (p.with_(fuel_indices=bad_fuel), "fuel index")):
        dq, keep = _device_problem(q, torch, dev)
        st = fn(C.byref(dq), seed, gen, 0, out.data_ptr(), k.data_ptr(), None, stream)
        assert st == abi.ERR_INVALID
        assert text in L.nraps_last_error(None).decode()
    dp, keep = _device_problem(p, torch, dev)
    st = fn(C.byref(dp), seed, gen, 0, out.data_ptr(), k.data_ptr(), None, stream)
    assert st == 0, L.nraps_last_error(None).decode()
    torch.cuda.synchronize(dev)
    ref = ctx_factory(seed=seed, mode=abi.MODE_PHYSICS, precision=abi.PREC_FP32)
    _, want_tally, _, kq = ref.trace(p, gen, 1.0)
    np.testing.assert_allclose(out.cpu().numpy(), want_tally, rtol=1e-12, atol=0)
    assert float(k.item()) == (kq * 2.0 ** -32) / p.histories


def test_no_alloc_rejects_sizes_beyond_its_array(ctx_factory):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    L, fn = _entry()
    p = synth.plain_small(5).with_(histories=100)
    dp, keep = _device_problem(p, torch, dev)
    dp.mattypes = 300                       # 300 * 4 (material, group) pairs > 1024
    out = torch.zeros(p.energygroups * p.n_cells, dtype=torch.float64, device=dev)
    k = torch.zeros(1, dtype=torch.float64, device=dev)
    st = fn(C.byref(dp), 1, 0, 0, out.data_ptr(), k.data_ptr(), None,
            torch.cuda.current_stream(dev).cuda_stream)
    assert st == abi.ERR_INVALID
    assert "1024" in L.nraps_last_error(None).decode()
