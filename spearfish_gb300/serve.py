"""Serving loop: continuous batching of alignment requests on one GPU (sf_server_*).

Each request is the jobs of one read batch over a byte pool.  Requests are admitted in
arrival order as soon as a slot is free and the device memory they need fits the HBM budget;
requests on different slots run on the device at the same time.  ``wait`` returns the
request's results and its latency (queue, run, total).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import _abi
from .align import Affine, _aff
from .batch import JOB_DTYPE, RESULT_DTYPE, Output

TIMEOUT = -5


@dataclass
class Stats:
    queue_ms: float
    run_ms: float
    total_ms: float
    cells: int
    slot: int


class Server:
    def __init__(self, device: int = 0, slots: int = 8, hbm_budget: int = 0,
                 scores: Sequence = (Affine.ONT,), store=None):
        self._lib = _abi.load()
        self._scores = (_abi.Affine * max(1, len(scores)))(*[_aff(s) for s in scores])
        self._store = store  # jobs may name texts as windows of it (text_src = TEXT_STORE)
        opts = _abi.ServerOpts(int(device), int(slots), int(hbm_budget), self._scores,
                               len(scores), store.handle if store is not None else None)
        h = C.c_void_p()
        _abi.check(self._lib.sf_server_create(C.byref(opts), C.byref(h)))
        self.handle = h
        self._keep: dict[int, tuple] = {}

    def submit(self, pool: np.ndarray, jobs: np.ndarray) -> int:
        pool = np.ascontiguousarray(pool, dtype=np.uint8)
        jobs = np.ascontiguousarray(jobs, dtype=JOB_DTYPE)
        t = C.c_uint64()
        _abi.check(self._lib.sf_server_submit(
            self.handle, pool.ctypes.data_as(C.POINTER(C.c_uint8)), pool.size,
            jobs.ctypes.data_as(C.POINTER(_abi.JobT)), len(jobs), C.byref(t)))
        self._keep[t.value] = (pool, jobs)  # the pool must outlive the request
        return t.value

    def wait(self, ticket: int, timeout_ms: int = 60_000) -> tuple[Output, Stats]:
        if ticket not in self._keep:  # not submitted here: the library reports it
            _abi.check(self._lib.sf_server_wait(self.handle, ticket, 0, None, None, 0, None,
                                                None))
        pool, jobs = self._keep[ticket]
        res = np.zeros(len(jobs), dtype=RESULT_DTYPE)
        want = jobs["want_cigar"] != 0
        cap = int((jobs["m"][want].astype(np.uint64) + jobs["n"][want] + 2).sum()) if want.any() \
            else 0
        ops = np.zeros(max(1, cap), dtype=np.uint32)
        used = C.c_uint64()
        st = _abi.RequestStats()
        rc = self._lib.sf_server_wait(self.handle, ticket, int(timeout_ms),
                                      res.ctypes.data_as(C.POINTER(_abi.ResultT)),
                                      ops.ctypes.data_as(C.POINTER(C.c_uint32)), cap,
                                      C.byref(used), C.byref(st))
        if rc != TIMEOUT:
            self._keep.pop(ticket, None)
        _abi.check(rc)
        return Output(res, ops[:used.value]), Stats(st.queue_ms, st.run_ms, st.total_ms,
                                                    int(st.cells), int(st.slot))

    def try_wait(self, ticket: int) -> Optional[tuple[Output, Stats]]:
        try:
            return self.wait(ticket, 0)
        except _abi.SfError as e:
            if e.code == TIMEOUT:
                return None
            raise

    def query(self) -> dict:
        s = _abi.ServerStats()
        _abi.check(self._lib.sf_server_query(self.handle, C.byref(s)))
        return {f: getattr(s, f) for f, _ in _abi.ServerStats._fields_ if f != "pad_"}

    def close(self):
        if self.handle:
            self._lib.sf_server_destroy(self.handle)
            self.handle = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass
