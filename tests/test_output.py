"""Output files of plot_solution (src/plot_solution.rs:7-63) and the float
text they hold (Rust `Display`), checked on the CPU.

Pins:
  * the reference's committed vars.csv / k_eff.csv / interface.csv (written by
    an older revision in f64): every field re-formatted from its parsed value
    must give back the same bytes;
  * numpy's shortest round-trip positional formatting (Dragon4, unique=True,
    trim='-') for f32 and f64 values over the whole exponent range;
  * the written files parse the way plot.py reads them.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from nraps_gb300 import abi, api

HERE = os.path.dirname(os.path.abspath(__file__))
PO = os.path.join(HERE, "golden", "plot_output")


@pytest.fixture(scope="module")
def L():
    return api.load()


def np_shortest(v) -> str:
    if np.isnan(v):
        return "NaN"
    if np.isinf(v):
        return "-inf" if v < 0 else "inf"
    return np.format_float_positional(v, unique=True, trim="-")


def test_known_texts(L):
    cases32 = {1.0: "1", 0.1: "0.1", -2.5: "-2.5", 1e20: "100000000000000000000",
               1e-7: "0.0000001", 0.0: "0", 123456.0: "123456", 16777216.0: "16777216",
               3.4028234663852886e38: "340282350000000000000000000000000000000",
               1.401298464324817e-45: "0.000000000000000000000000000000000000000000001"}
    for v, want in cases32.items():
        assert api.format_f32(v) == want, v
    assert api.format_f32(-0.0) == "-0"
    assert api.format_f32(float("nan")) == "NaN"
    assert api.format_f32(float("inf")) == "inf"
    assert api.format_f32(float("-inf")) == "-inf"
    assert api.format_f64(42.90800000000001) == "42.90800000000001"
    assert api.format_f64(1.0) == "1"
    assert api.format_f64(5e-324) == "0." + "0" * 323 + "5"
    assert api.format_f64(1.7976931348623157e308) == "17976931348623157" + "0" * 292


def test_reference_fixture_bytes(L):
    """Each field of the reference's own files re-formats to the same text."""
    for name in ("k_eff.csv", "interface_head.csv"):
        raw = open(os.path.join(PO, name), "rb").read().decode()
        rows = raw.split("\n")
        assert rows[-1] == ""
        n = 0
        for row in rows[:-1]:
            for field in row.split(","):
                assert api.format_f64(float(field)) == field, (name, field)
                n += 1
        assert n > 100
    lines = open(os.path.join(PO, "vars.csv")).read().split("\n")
    assert api.format_f64(float(lines[0])) == lines[0]
    assert lines[1:] == ["408", "100", ""]


def test_matches_numpy_shortest(L):
    rng = np.random.default_rng(7)
    bits32 = rng.integers(0, 2**32, 20000, dtype=np.uint64).astype(np.uint32)
    f32 = bits32.view(np.float32)
    for v in f32:
        assert api.format_f32(float(v)) == np_shortest(v), hex(int(np.float32(v).view(np.uint32)))
    bits64 = rng.integers(0, 2**63, 5000, dtype=np.uint64) | (rng.integers(0, 2, 5000, dtype=np.uint64) << 63)
    for v in bits64.view(np.float64):
        assert api.format_f64(float(v)) == np_shortest(v)
    # values a solver writes: fluxes, k, averages
    for v in rng.uniform(0.5, 1.5, 2000).astype(np.float32):
        assert api.format_f32(float(v)) == np_shortest(v)
    for v in (rng.lognormal(0, 8, 2000)).astype(np.float32):
        assert api.format_f32(float(v)) == np_shortest(v)


def test_format_buffer_too_small(L):
    import ctypes as C
    buf = C.create_string_buffer(4)
    assert L.nraps_format_f32(123456.0, buf, 4) == -1
    assert L.nraps_format_f32(12.0, buf, 4) == 2
    assert buf.value == b"12"


def _result(G, cells, gens, rng):
    r = abi.ResultArrays(G, cells, gens)
    r.flux[:] = rng.lognormal(0, 3, G * cells).astype(np.float32)
    r.assembly_average[:] = rng.lognormal(0, 3, G * cells).astype(np.float32)
    r.fission_source[:] = rng.uniform(0, 2, cells).astype(np.float32)
    r.fission_source[::7] = 0.0
    r.k[:] = rng.uniform(0.9, 1.1, gens).astype(np.float32)
    r.k_fund[:] = rng.uniform(0.9, 1.1, gens).astype(np.float32)
    return r


def test_write_solution_layout(L, tmp_path):
    rng = np.random.default_rng(3)
    G, cells, gens = 4, 37, 11
    r = _result(G, cells, gens, rng)
    length = float(np.float32(42.908))
    api.write_solution(r, gens, length, str(tmp_path))
    vars_ = open(tmp_path / "vars.csv").read()
    assert vars_ == f"{api.format_f64(length)}\n{cells}\n{gens}\n"
    assert vars_.startswith("42.90800094604492\n")
    rows = open(tmp_path / "interface.csv").read().split("\n")
    assert rows[-1] == "" and len(rows) == 2 * G + 2
    want = ([r.flux[g * cells:(g + 1) * cells] for g in range(G)]
            + [r.assembly_average[g * cells:(g + 1) * cells] for g in range(G)] + [r.fission_source])
    for row, w in zip(rows[:-1], want):
        fields = row.split(",")
        assert len(fields) == cells
        assert fields == [np_shortest(v) for v in w]
        # plot.py: np.array(line.strip().split(',')).astype(float)
        got = np.array(row.strip().split(",")).astype(float).astype(np.float32)
        assert np.array_equal(got, w)
    k_rows = open(tmp_path / "k_eff.csv").read().split("\n")
    assert len(k_rows) == 3 and k_rows[2] == ""
    assert np.array_equal(np.array(k_rows[0].split(",")).astype(float).astype(np.float32), r.k)
    assert np.array_equal(np.array(k_rows[1].split(",")).astype(float).astype(np.float32), r.k_fund)


def test_write_solution_errors(L, tmp_path):
    r = _result(2, 5, 3, np.random.default_rng(1))
    with pytest.raises(api.NrapsError) as e:
        api.write_solution(r, 3, 1.0, str(tmp_path / "no" / "such" / "dir"))
    assert e.value.status == abi.ERR_IO
    r.G = 0
    with pytest.raises(api.NrapsError) as e:
        api.write_solution(r, 3, 1.0, str(tmp_path))
    assert e.value.status == abi.ERR_INVALID
