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


def test_no_alloc_generation_matches_existing_entry_point(ctx_factory):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    torch.cuda.set_device(0)
    L, fn = _entry()
    p = synth.plain_small(5).with_(histories=6000, generations=8, skip=2)
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
