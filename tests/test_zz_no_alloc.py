"""sf_affine_noalloc: the `affine` entry point for callers that must not allocate device
memory -- a latency-bound serving path (cudaMalloc and cudaFree synchronize the device and
stall every request in flight) or an application that lends this library device memory from
its own pool.  Its scratch is a fixed device array inside the library; the caller hands device
buffers for the sequences and the score.

Checked through the C ABI against the existing entry point (sf_affine), bit-exact, on two
calls in a row that share the array.  The file sorts last so that a run stopping at its first
failure has run every other test before it; it passes alone in a fresh process as well.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from spearfish_gb300 import _abi, build
    build.build()
    return _abi.load()


def _noalloc(lib, p, t, mode, sc, band):
    import torch
    from spearfish_gb300 import _abi
    dp = torch.tensor(np.asarray(p, dtype=np.uint8), device="cuda")
    dt = torch.tensor(np.asarray(t, dtype=np.uint8), device="cuda")
    out = torch.full((1,), -12345, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    rc = lib.sf_affine_noalloc(dp.data_ptr(), len(p), dt.data_ptr(), len(t), mode,
                               C.byref(_abi.Affine(*sc)),
                               _abi.SF_NOLIMIT if band is None else band, out.data_ptr(),
                               stream.cuda_stream)
    assert rc == 0, lib.sf_last_error()
    stream.synchronize()
    return int(out.item())


def test_noalloc_matches_affine_twice(lib):
    from spearfish_gb300 import align as A
    rng = np.random.default_rng(9001)
    ont, hifi = (2, 4, 4, 2), (1, 4, 6, 2)
    # Call 1: unbanded Infix over a text wider than the register rows hold.
    t1 = rng.integers(0, 4, 5000, dtype=np.uint8)
    p1 = t1[1200:2400].copy()
    p1[::37] = (p1[::37] + 1) & 3
    # Call 2: a banded Global pass of other lengths; the array still holds call 1's bytes.
    p2 = rng.integers(0, 4, 1500, dtype=np.uint8)
    t2 = np.delete(p2, np.arange(0, 1500, 53))
    for (p, t, mode, sc, band) in ((p1, t1, A.Mode.Infix, ont, None),
                                   (p2, t2, A.Mode.Global, hifi, 40)):
        want = A.affine(p, t, mode, sc, band)
        got = _noalloc(lib, p, t, int(mode), sc, band)
        assert got == want, (int(mode), got, want)


def test_noalloc_rejects_oversize(lib):
    from spearfish_gb300 import _abi
    big = 16384 + 1
    rc = lib.sf_affine_noalloc(None, big, None, 10, 2, C.byref(_abi.Affine(2, 4, 4, 2)), 16,
                               None, None)
    assert rc == -1  # null buffers are rejected first
    import torch
    dp = torch.zeros(big, dtype=torch.uint8, device="cuda")
    out = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = lib.sf_affine_noalloc(dp.data_ptr(), big, dp.data_ptr(), 10, 2,
                               C.byref(_abi.Affine(2, 4, 4, 2)), 16, out.data_ptr(), None)
    assert rc == -4 and b"SF_NOALLOC_MAX_LEN" in lib.sf_last_error()
