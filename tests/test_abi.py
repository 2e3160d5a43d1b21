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


def test_ctypes_structs_match_the_header(tmp_path):
    """The Python mirror's nnet_burn_args / nnet_stats have the C header's field offsets and sizes."""
    import subprocess
    import nnet_gb300 as nn
    structs = {"nnet_burn_args": nn._BurnArgs, "nnet_stats": nn._Stats}
    lines = []
    for cname, py in structs.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'printf("{cname}.{f} %zu\\n", offsetof({cname}, {f}));')
    src = tmp_path / "layout.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "nnet_gb300.h"\nint main(void){\n'
                   + "\n".join(lines) + "\nreturn 0;}\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)], check=True)
    c = dict(l.split() for l in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines())
    for cname, py in structs.items():
        assert int(c[cname]) == ctypes.sizeof(py), cname
        for f, _ in py._fields_:
            assert int(c[f"{cname}.{f}"]) == getattr(py, f).offset, (cname, f)
