"""The deterministic diffusion solver (nalgebra_method, src/discrete.rs:169-356)
against an independent numpy restatement of the reference's procedure (dense
matrices and an explicit inverse read back the way the reference reads
nalgebra's column-major storage), on the reference's own input files; and the
input-file dispatch for `Solution != 1` files, which needs no GPU."""
from __future__ import annotations

import os

import numpy as np
import pytest

from nraps_gb300 import abi, api

from .conftest import GOLDEN

INPUTS = os.path.join(GOLDEN, "inputs")


def reference_procedure(prob):
    """src/discrete.rs restated step by step in float64 numpy."""
    G, M, n = prob.energygroups, prob.mattypes, prob.n_cells
    mat = prob.matid.astype(np.int64)
    dx = prob.delta_x.astype(np.float64)
    f = lambda a: np.asarray(a, np.float64)
    sigt, inv, nut, sigf, chit, scat = f(prob.sigt), f(prob.inv_sigtr), f(prob.nut), f(prob.sigf), f(prob.chit), f(prob.scat)
    ix = lambda m, g: m + M * g
    D = lambda i, g: (1.0 / 3.0) * inv[ix(mat[i], g)] / dx[i]
    harm = lambda a, b: (2.0 * a * b) / (a + b)
    sgg = lambda m, g: scat[G * G * m + G * g + g]

    def beta(bound, da, db):
        if bound == 1.0:
            return 1.0
        if bound == 0.0:
            return 0.25
        r = (1.0 - bound) / (1.0 + bound)
        return (1.0 - 0.25 * (r * (1.0 / da))) / (1.0 + 0.25 * (r * (1.0 / db)))

    a_inv_rows = []
    for g in range(G):
        A = np.zeros((n, n))
        dc0, dn0 = D(0, g), D(1, g)
        dnc0 = harm(dc0, dn0)
        A[0, 0] = 2 * dc0 * (1 - beta(float(prob.boundl), dn0, dc0)) + dx[0] * (sigt[ix(mat[0], g)] - sgg(mat[0], g)) + dnc0
        A[0, 1] = -dnc0
        for x in range(1, n - 1):
            dc = D(x, g)
            dpc, dnc = harm(dc, D(x - 1, g)), harm(dc, D(x + 1, g))
            A[x, x - 1] = -dpc
            A[x, x] = dpc + dx[x] * (sigt[ix(mat[x], g)] - sgg(mat[x], g)) + dnc
            A[x, x + 1] = -dnc
        dc = D(n - 1, g)
        dpc = harm(dc, D(n - 2, g))
        A[n - 1, n - 2] = -dpc
        A[n - 1, n - 1] = (2 * dc * (1 - beta(float(prob.boundr), dn0, dc))
                           + dx[n - 1] * (sigt[ix(mat[n - 1], g)] - sgg(mat[n - 1], g)) + dnc0)
        inv_a = np.linalg.inv(A)
        # nalgebra stores column-major; chunks(n) of that storage are columns
        a_inv_rows.append(inv_a.T.copy())

    def q_gen(phi):
        q = np.zeros((G, n))
        for g in range(G):
            for i in range(n):
                s = sum(nut[ix(mat[i], e)] * sigf[ix(mat[i], e)] * phi[e, i] for e in range(G))
                q[g, i] = s * dx[i] * chit[ix(mat[i], g)]
        return q

    phi = np.ones((G, n))
    q = q_gen(phi)
    k, dfl, dk, it = 1.0, 1.0, 1.0, 0
    while dfl >= 1e-5 and dk >= 1e-6:
        q_old = q.copy()
        for g in range(G):
            sc = np.zeros(n)
            for i in range(n):
                sc[i] = sum(scat[G * G * mat[i] + G * e + g] * phi[e, i] * dx[i] for e in range(G) if e != g)
            tf = q[g] * (1.0 / k) + sc
            y = a_inv_rows[g] @ tf
            dfl = max(abs((phi[g, 0] - y[0]) / phi[g, 0]), dfl)
            phi[g, 0] = y[0]
            for i in range(1, n - 1):
                dfl = abs((phi[g, i] - y[i]) / phi[g, 0])
                phi[g, i] = y[i]
            dfl = max(abs((phi[g, n - 1] - y[n - 1]) / phi[g, 0]), dfl)
            phi[g, n - 1] = y[n - 1]
        q = q_gen(phi)
        k_old = k
        k = k_old * (q.sum() / q_old.sum())
        dk = abs((k - k_old) / k_old)
        it += 1
    flat = np.array([phi[e, i] * nut[ix(mat[i], e)] * sigf[ix(mat[i], e)] for e in range(G) for i in range(n)])
    chunks = flat.reshape(n, G).sum(axis=1)          # chunks of G consecutive group-major values
    pc = 3565e6 / (1.6022e-13 * 200.0 * float((chunks * dx).sum()))
    return k, it, phi * pc


@pytest.fixture(scope="module")
def lib():
    return api.load()


@pytest.mark.parametrize("case", ["TestCaseA.txt", "TestCaseB.txt", "TestCaseC.txt"])
def test_matches_reference_procedure(lib, case):
    inp = api.process_input(os.path.join(INPUTS, case))
    mesh, fuel = api.mesh_gen(inp.matid, inp.variables, inp.delta_x)
    prob = api.problem_from_input(inp, mesh, fuel)
    flux, avg, info = api.diffusion_solve(prob)
    k, it, phi = reference_procedure(prob)
    assert info["converged"] and info["iterations"] == it
    assert info["k"] == pytest.approx(k, rel=1e-9)
    np.testing.assert_allclose(flux, phi.astype(np.float32), rtol=1e-5)
    # average_assembly: the per-assembly mean written to each of its cells
    na = max(1, prob.numass)
    ma = prob.n_cells // na
    for a in range(na):
        np.testing.assert_allclose(avg[:, a * ma:(a + 1) * ma],
                                   phi[:, a * ma:(a + 1) * ma].mean(axis=1, keepdims=True).repeat(ma, 1),
                                   rtol=1e-5)


def test_vacuum_and_albedo_boundaries(lib):
    """The three boundary rows: vacuum (beta 0.25), reflective (1) and the
    albedo formula, on a modified TestCaseC."""
    inp = api.process_input(os.path.join(INPUTS, "TestCaseC.txt"))
    mesh, fuel = api.mesh_gen(inp.matid, inp.variables, inp.delta_x)
    base = api.problem_from_input(inp, mesh, fuel)
    ks = []
    for bl, br in ((0.0, 0.0), (1.0, 1.0), (0.5, 0.25)):
        prob = base.with_(boundl=bl, boundr=br)
        _, _, info = api.diffusion_solve(prob)
        k, it, _ = reference_procedure(prob)
        assert info["k"] == pytest.approx(k, rel=1e-9) and info["iterations"] == it
        ks.append(info["k"])
    assert ks[0] < ks[2] < ks[1]          # leakage lowers k


def test_dispatch_deterministic_files(lib, tmp_path):
    """Solution = 0 with the LinAlg solver runs the diffusion solver with no
    context; one k, and empty k_fund and fission-source rows."""
    api.run_input(os.path.join(INPUTS, "TestCaseB.txt"), str(tmp_path))
    vars_ = open(tmp_path / "vars.csv").read().split("\n")
    assert vars_[1:] == ["400", "100", ""]
    rows = open(tmp_path / "interface.csv").read().split("\n")
    assert len(rows) == 2 * 2 + 2 and rows[-2] == "" and rows[-1] == ""
    assert all(len(r.split(",")) == 400 for r in rows[:4])
    k_rows = open(tmp_path / "k_eff.csv").read().split("\n")
    assert len(k_rows[0].split(",")) == 1 and k_rows[1] == "" and k_rows[2] == ""
    inp = api.process_input(os.path.join(INPUTS, "TestCaseB.txt"))
    mesh, fuel = api.mesh_gen(inp.matid, inp.variables, inp.delta_x)
    _, _, info = api.diffusion_solve(api.problem_from_input(inp, mesh, fuel))
    assert k_rows[0] == api.format_f32(info["k"])


def test_dispatch_errors_without_gpu(lib, tmp_path):
    # Solution = 1 runs Monte Carlo and needs a context
    with pytest.raises(api.NrapsError) as e:
        api.run_input(os.path.join(INPUTS, "TestCaseC.txt"), str(tmp_path))
    assert e.value.status == abi.ERR_INVALID
    # the Gaussian/Jacobian/SR solvers are not implemented by the reference
    text = open(os.path.join(INPUTS, "TestCaseA.txt")).read().replace("solver = 0", "solver = 2")
    (tmp_path / "jac.txt").write_text(text)
    with pytest.raises(api.NrapsError) as e:
        api.run_input(str(tmp_path / "jac.txt"), str(tmp_path))
    assert e.value.status == abi.ERR_UNSUPPORTED


def test_diffusion_source_sites(lib):
    """The initial source: deterministic, sorted, each site inside its cell,
    cell counts proportional to the diffusion fission density, groups from
    the cell material's chi."""
    inp = api.process_input(os.path.join(INPUTS, "TestCaseC.txt"))
    mesh, fuel = api.mesh_gen(inp.matid, inp.variables, inp.delta_x)
    prob = api.problem_from_input(inp, mesh, fuel)
    n = 50000
    a = api.diffusion_source(prob, n)
    b = api.diffusion_source(prob, n)
    assert np.array_equal(a, b)
    assert np.all(np.diff(a["x"]) >= 0)
    left, right = prob.mesh_left[a["cell"]], prob.mesh_right[a["cell"]]
    assert np.all(a["x"] >= left - 1e-5) and np.all(a["x"] <= right + 1e-5)
    flux, _, _ = api.diffusion_solve(prob)
    G, M = prob.energygroups, prob.mattypes
    m = prob.matid.astype(np.int64)
    dens = sum(prob.nut[m + M * g].astype(np.float64) * prob.sigf[m + M * g] * flux[g] for g in range(G)) * prob.delta_x
    want = n * dens / dens.sum()
    got = np.bincount(a["cell"], minlength=prob.n_cells)
    assert np.all(np.abs(got - want) <= 1.0 + 1e-9)
    assert np.all(dens[a["cell"]] > 0)
    # groups: chi of the site's material, within sampling resolution
    for mat in np.unique(m[a["cell"]]):
        sel = m[a["cell"]] == mat
        chi = np.array([prob.chit[mat + M * g] for g in range(G)], np.float64)
        frac = np.bincount(a["group"][sel], minlength=G) / sel.sum()
        np.testing.assert_allclose(frac, chi / chi.sum(), atol=2e-3)
