"""The C-ABI library builds, loads and exports every symbol include/sf_align.h declares, with
struct layouts that match the Python mirror.  No compute call is made here (no GPU)."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "sf_align.h")


@pytest.fixture(scope="module")
def lib():
    from spearfish_gb300 import build, _abi
    build.build()
    return _abi.load()


def declared() -> set[str]:
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"\b(sf_[a-z0-9_]+)\s*\(", text))


def test_header_symbols_exported(lib):
    names = declared()
    assert len(names) >= 29
    for n in sorted(names):
        assert hasattr(lib, n), n


def test_python_binding_covers_header():
    from spearfish_gb300 import _abi
    assert declared() == set(_abi.SIGNATURES)


def test_struct_layouts(lib):
    from spearfish_gb300 import _abi, batch
    assert C.sizeof(_abi.JobT) == 80
    assert C.sizeof(_abi.ResultT) == 64
    assert C.sizeof(_abi.ExtendT) == 32
    assert C.sizeof(_abi.CutT) == 16
    assert C.sizeof(_abi.CigarT) == 40
    assert C.sizeof(_abi.SpanT) == 16
    assert C.sizeof(_abi.BandedReadT) == 40
    assert C.sizeof(_abi.EndsT) == 40
    assert C.sizeof(_abi.HitT) == 40
    assert C.sizeof(_abi.SortedCallT) == 80
    assert batch.JOB_DTYPE.itemsize == 80 and batch.RESULT_DTYPE.itemsize == 64


def test_version_and_errors(lib):
    assert b"sm_103a" in lib.sf_version()
    # An invalid argument is rejected before any device work.
    out = C.c_uint32()
    rc = lib.sf_distance(None, 0, None, 0, 7, 0, C.byref(out))
    assert rc == -1
    assert b"bad argument" in lib.sf_last_error()


def test_no_cpu_fallback_in_product():
    """The product package never reaches the oracle."""
    pkg = os.path.join(ROOT, "spearfish_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".cpp")):
                src = open(os.path.join(dirpath, f)).read()
                assert "oracle" not in src.replace("oracle)", ""), f
