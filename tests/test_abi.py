"""The C-ABI library: loads, exports every declared symbol, fails loudly."""
import os
import re

import pytest

from nraps_gb300 import abi, api

from .conftest import ROOT


def declared_functions():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(nraps_\w+)\s*\(", txt))
    return sorted(names)


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) > 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_sizes_match_header(lib):
    import ctypes as C
    assert C.sizeof(abi.HistoryRecord) == 64
    assert C.sizeof(abi.Site) == 16


def test_opts_default(lib):
    o = abi.Opts()
    lib.nraps_opts_default(o)
    assert o.abi_version == abi.ABI_VERSION and o.seed == 1 and o.device == -1


def test_no_device_fails_loudly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(api.NrapsError) as e:
        api.Context()
    assert e.value.status == abi.ERR_NO_DEVICE
