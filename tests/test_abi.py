"""The C-ABI library loads and exports every entry point include/nnet_gb300.h declares;
host-only calls work without a GPU (no compute is attempted here)."""
import ctypes
import os
import re

import pytest

from conftest import REPO

HEADER = os.path.join(REPO, "include", "nnet_gb300.h")


def declared():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(nnet_\w+)\s*\(", src, re.M)))


@pytest.fixture(scope="module")
def lib():
    import nnet_build
    nnet_build.build()
    import nnet_gb300
    return nnet_gb300.load_library()


def test_every_declared_symbol_is_exported(lib):
    names = declared()
    assert "nnet_burn" in names and len(names) >= 9
    for n in names:
        assert hasattr(lib, n), n


def test_network_info(lib):
    s, r = ctypes.c_int(), ctypes.c_int()
    for net, nr in [(14, 29), (86, 309), (87, 311)]:
        assert lib.nnet_network_info(net, ctypes.byref(s), ctypes.byref(r)) == 0
        assert (s.value, r.value) == (net, nr)
    assert lib.nnet_network_info(15, ctypes.byref(s), ctypes.byref(r)) == -1
    assert b"unknown network" in lib.nnet_last_error_message()


def test_invalid_arguments_rejected_on_host(lib):
    assert lib.nnet_burn(None, None, None) == -1
    assert lib.nnet_create(0, None) == -1


def test_library_is_sm103a_only():
    """The shared library carries sm_103a SASS (one -gencode)."""
    import nnet_build
    assert nnet_build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
