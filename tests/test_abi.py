"""The C-ABI library builds, loads on a host without a GPU and exports every
entry point that include/pespace_gb300.h declares; the ctypes structs match the
header's layout (checked by compiling the header with the host C compiler)."""

import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "pespace_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pes_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def built_lib():
    import pespace_gb300

    path = pespace_gb300.build.build()
    return ctypes.CDLL(path)


def test_exports_every_declared_symbol(built_lib):
    names = declared_functions()
    assert len(names) >= 14
    for n in names:
        assert hasattr(built_lib, n), n


def test_ctypes_signatures_cover_header():
    from pespace_gb300 import _lib

    assert set(declared_functions()) == set(_lib.SIGNATURES)


def test_struct_layout_matches_header(tmp_path):
    from pespace_gb300 import _lib

    src = tmp_path / "layout.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "pespace_gb300.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu %zu\\n\", sizeof(PesOrbit), sizeof(PesDetectorDesc),"
        " sizeof(PesPlanDesc), offsetof(PesPlanDesc, det), offsetof(PesOrbit, ck)); return 0;}\n"
    )
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    want = [ctypes.sizeof(_lib.PesOrbit), ctypes.sizeof(_lib.PesDetectorDesc), ctypes.sizeof(_lib.PesPlanDesc),
            _lib.PesPlanDesc.det.offset, _lib.PesOrbit.ck.offset]
    assert got == want


def test_host_only_calls_without_gpu(built_lib):
    """Argument validation and host-side entry points need no device."""
    from pespace_gb300 import _lib

    lib = _lib.load()
    assert lib.pes_version() >= 1
    assert lib.pes_whittle_workspace_len(0) == 1
    assert lib.pes_whittle_workspace_len(10 ** 9) == 1024
    # invalid generation is rejected before any launch
    rc = lib.pes_tdi_combination(None, 10, 8.3, 17, 1, None, None, None)
    assert rc == _lib.PES_EINVAL
    assert b"generation" in lib.pes_last_error()
    # plan with bad sizes
    desc = _lib.PesPlanDesc()
    desc.nbins = 0
    handle = ctypes.c_void_p()
    assert lib.pes_plan_create(ctypes.byref(desc), ctypes.byref(handle)) == _lib.PES_EINVAL
    assert not handle.value
