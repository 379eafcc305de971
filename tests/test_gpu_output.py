"""The restored main dispatch (src/main.rs:332-364) end to end on the GPU:
input file -> process_input -> mesh_gen -> Monte Carlo -> the three CSV files
of plot_solution (src/plot_solution.rs:36-58), through the C-ABI call and
through the `nraps` program."""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

from nraps_gb300 import abi, api
from nraps_gb300.build import CLI

from .conftest import GOLDEN

pytestmark = pytest.mark.gpu

INPUTS = os.path.join(GOLDEN, "inputs")


def _read_rows(path):
    text = open(path).read()
    assert text.endswith("\n")
    return [np.array(r.split(","), dtype=np.float64) for r in text[:-1].split("\n")]


def test_run_input_matches_solve(ctx_factory, tmp_path):
    """TestCaseC (Solution = 1; 408 cells, 4 groups, 100 generations of 1M
    histories) through nraps_run_input equals solve() + write_solution."""
    path = os.path.join(INPUTS, "TestCaseC.txt")
    ctx = ctx_factory(seed=11, mode=abi.MODE_BANK, precision=abi.PREC_FP32, tracking=abi.TRACK_WOODCOCK)
    d1, d2 = tmp_path / "a", tmp_path / "b"
    d1.mkdir()
    d2.mkdir()
    st = ctx.run_input(path, str(d1))
    inp = api.process_input(path)
    mesh, fuel = api.mesh_gen(inp.matid, inp.variables, inp.delta_x)
    prob = api.problem_from_input(inp, mesh, fuel, k_new=1.0)
    res = ctx.solve(prob)
    api.write_solution(res, prob.generations, float(mesh.mesh_right[-1]), str(d2))
    assert open(d1 / "vars.csv").read() == open(d2 / "vars.csv").read()
    assert open(d1 / "vars.csv").read().split("\n")[1:] == ["408", "100", ""]
    # k is accumulated in fixed point: identical text
    assert open(d1 / "k_eff.csv").read() == open(d2 / "k_eff.csv").read()
    a, b = _read_rows(d1 / "interface.csv"), _read_rows(d2 / "interface.csv")
    assert len(a) == len(b) == 2 * 4 + 1
    for ra, rb in zip(a, b):
        assert ra.size == 408
        # FP64 atomics sum in any order; after rounding to f32 the results
        # agree to a few ulp
        np.testing.assert_allclose(ra, rb, rtol=1e-6, atol=0)
    k = _read_rows(d1 / "k_eff.csv")[0]
    assert np.all(np.isfinite(k)) and 0.5 < k[-1] < 2.0
    assert abs(st.k_mean - res.stats.k_mean) < 1e-12


def test_run_input_compat_default(ctx_factory, tmp_path):
    """Default options: the reference's algorithm (COMPAT, FP64 plain kernel)
    on a smaller copy of TestCaseC."""
    text = open(os.path.join(INPUTS, "TestCaseC.txt")).read()
    text = text.replace("Histories = 1000000", "Histories = 20000").replace("Generations = 100", "Generations = 12")
    src = tmp_path / "small.txt"
    src.write_text(text)
    ctx = ctx_factory(seed=5)
    ctx.run_input(str(src), str(tmp_path))
    rows = _read_rows(tmp_path / "interface.csv")
    assert len(rows) == 9 and all(r.size == 408 for r in rows)
    k = _read_rows(tmp_path / "k_eff.csv")
    assert k[0].size == 12 and k[1].size == 12


def test_run_input_dispatch_errors(ctx_factory, tmp_path):
    ctx = ctx_factory(seed=1)
    # Solution = 0 with the LinAlg solver: the deterministic solver, one k
    det = tmp_path / "det"
    det.mkdir()
    ctx.run_input(os.path.join(INPUTS, "TestCaseA.txt"), str(det))
    assert len(open(det / "k_eff.csv").read().split("\n")[0].split(",")) == 1
    with pytest.raises(api.NrapsError) as e:
        ctx.run_input(str(tmp_path / "missing.txt"), str(tmp_path))
    assert e.value.status == abi.ERR_IO
    assert not (tmp_path / "k_eff.csv").exists()


def test_cli_program(tmp_path):
    assert os.path.exists(CLI)
    text = open(os.path.join(INPUTS, "TestCaseC.txt")).read().replace("Histories = 1000000", "Histories = 100000")
    (tmp_path / "TestCaseC.txt").write_text(text)
    r = subprocess.run([CLI, "--mode", "bank", "--form", "event", "-o", str(tmp_path)], cwd=tmp_path,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "Run was completed in" in r.stdout
    for name in ("vars.csv", "interface.csv", "k_eff.csv"):
        assert (tmp_path / name).exists()
    text = open(os.path.join(INPUTS, "TestCaseB.txt")).read().replace("solver   = 0", "solver   = 3")
    (tmp_path / "sr.txt").write_text(text)
    r = subprocess.run([CLI, str(tmp_path / "sr.txt"), "-o", str(tmp_path)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 1 and "LinAlg" in r.stderr
