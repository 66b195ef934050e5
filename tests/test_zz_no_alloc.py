"""sf_affine_noalloc: the `affine` entry point for callers that must not allocate device
memory -- a latency-bound serving path (cudaMalloc and cudaFree synchronize the device and
stall every request in flight) or an application that lends this library device memory from
its own pool.  Its scratch is a fixed device array inside the library; the caller hands device
buffers for the sequences and the score.

Checked through the C ABI, bit-exact, against both the existing entry point (sf_affine) and
the oracle (align.rs:699-701 `affine`), on calls in a row that share the array: every mode,
banded and unbanded, empty pattern or text, a pattern far longer than its text under a band,
and an unbanded pass at SF_NOALLOC_MAX_LEN (the largest use of the array).  The file sorts
last so that a run stopping at its first failure has run every other test before it; it
passes alone in a fresh process as well.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

MAX_LEN = 16384  # SF_NOALLOC_MAX_LEN


@pytest.fixture(scope="module")
def lib():
    from spearfish_gb300 import _abi, build
    build.build()
    return _abi.load()


def _noalloc(lib, p, t, mode, sc, band):
    import torch
    from spearfish_gb300 import _abi
    # Length-0 inputs still get a valid device buffer (never read).
    def dev(a):
        a = np.asarray(a, dtype=np.uint8)
        return torch.tensor(a if a.size else np.zeros(1, np.uint8), device="cuda")

    dp, dt = dev(p), dev(t)
    out = torch.full((1,), -12345, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    rc = lib.sf_affine_noalloc(dp.data_ptr(), len(p), dt.data_ptr(), len(t), mode,
                               C.byref(_abi.Affine(*sc)),
                               _abi.SF_NOLIMIT if band is None else band, out.data_ptr(),
                               stream.cuda_stream)
    assert rc == 0, lib.sf_last_error()
    stream.synchronize()
    return int(out.item())


def _cases():
    rng = np.random.default_rng(9001)
    ont, hifi = (2, 4, 4, 2), (1, 4, 6, 2)
    # Unbanded Infix over a text wider than the register rows hold.
    t1 = rng.integers(0, 4, 5000, dtype=np.uint8)
    p1 = t1[1200:2400].copy()
    p1[::37] = (p1[::37] + 1) & 3
    # A banded Global pass of other lengths; the array still holds the last call's bytes.
    p2 = rng.integers(0, 4, 1500, dtype=np.uint8)
    t2 = np.delete(p2, np.arange(0, 1500, 53))
    # Prefix, banded and unbanded.
    p3 = rng.integers(0, 4, 900, dtype=np.uint8)
    t3 = np.concatenate([np.delete(p3, np.arange(5, 900, 41)), rng.integers(0, 4, 300,
                                                                            dtype=np.uint8)])
    # A pattern far longer than its text, under a band (rows past the text's end).
    p4 = rng.integers(0, 4, 3000, dtype=np.uint8)
    t4 = p4[:400].copy()
    e = np.zeros(0, np.uint8)
    return [(p1, t1, 0, ont, None), (p2, t2, 2, hifi, 40), (p3, t3, 1, ont, 30),
            (p3, t3, 1, hifi, None), (p4, t4, 2, ont, 64), (p4, t4, 1, ont, 64),
            (e, t2, 0, ont, None), (e, t2, 2, ont, 16), (e, t2, 1, ont, None),
            (p2, e, 2, ont, 16), (p2, e, 1, ont, None), (p2, e, 0, ont, None),
            (e, e, 2, ont, 8)]


def test_noalloc_matches_affine_and_oracle(lib):
    from spearfish_gb300 import align as A
    for (p, t, mode, sc, band) in _cases():
        want = O.affine(p, t, mode, sc, band)
        assert A.affine(p, t, A.Mode(mode), sc, band) == want
        got = _noalloc(lib, p, t, mode, sc, band)
        assert got == want, (mode, len(p), len(t), band, got, want)


def test_noalloc_twice_in_a_row(lib):
    """Two calls in a row on one stream: the second reads nothing the first left behind."""
    cases = _cases()
    for (p, t, mode, sc, band) in (cases[0], cases[1], cases[1], cases[0]):
        assert _noalloc(lib, p, t, mode, sc, band) == O.affine(p, t, mode, sc, band)


def test_noalloc_at_max_len(lib):
    """Unbanded Global and Infix passes with pattern and text at SF_NOALLOC_MAX_LEN: the wide
    kernel's row buffers take the most of the array there."""
    from spearfish_gb300 import align as A
    rng = np.random.default_rng(9002)
    p = rng.integers(0, 4, MAX_LEN, dtype=np.uint8)
    t = p.copy()
    t[::29] = (t[::29] + 1) & 3
    for mode in (2, 0):
        want = O.affine(p, t, mode, (2, 4, 4, 2), None)
        assert A.affine(p, t, A.Mode(mode), (2, 4, 4, 2), None) == want
        assert _noalloc(lib, p, t, mode, (2, 4, 4, 2), None) == want


def test_noalloc_rejects_oversize(lib):
    from spearfish_gb300 import _abi
    big = MAX_LEN + 1
    rc = lib.sf_affine_noalloc(None, big, None, 10, 2, C.byref(_abi.Affine(2, 4, 4, 2)), 16,
                               None, None)
    assert rc == -1  # null buffers are rejected first
    import torch
    dp = torch.zeros(big, dtype=torch.uint8, device="cuda")
    out = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = lib.sf_affine_noalloc(dp.data_ptr(), big, dp.data_ptr(), 10, 2,
                               C.byref(_abi.Affine(2, 4, 4, 2)), 16, out.data_ptr(), None)
    assert rc == -4 and b"SF_NOALLOC_MAX_LEN" in lib.sf_last_error()
    # The library still answers after the refusal.
    p = np.arange(50, dtype=np.uint8) & 3
    assert _noalloc(lib, p, p, 2, (2, 4, 4, 2), 8) == O.affine(p, p, 2, (2, 4, 4, 2), 8)
