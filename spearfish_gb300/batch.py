"""Batched alignment: thousands of (pattern, text) jobs in one plan -- length-bucketed,
persistent launches captured in a CUDA graph (include/sf_align.h, "batched form").

Jobs are numpy structured arrays laid out as ``sf_job_t``; results come back as
``sf_result_t`` records plus a pool of CIGAR ops.  The reference's callers build the same
pairs per read (map/src/lib.rs:851-911 `banded`, 1294-1884 `segmented`, 2100-2114
`extend_dp`); here a whole read batch goes to the device at once.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import _abi
from .align import Affine, Mode, _aff

JOB_MYERS, JOB_AFFINE, JOB_EXTEND_WINDOW, JOB_LOCAL = 0, 1, 2, 3

JOB_DTYPE = np.dtype([("p_off", "<u8"), ("t_off", "<u8"), ("m", "<u4"), ("n", "<u4"),
                      ("kind", "u1"), ("mode", "u1"), ("want_cigar", "u1"), ("text_src", "u1"),
                      ("k", "<u4"), ("band", "<u8"), ("window", "<u8"), ("dlo", "<i8"),
                      ("dhi", "<i8"), ("end_bonus", "<i4"), ("end_bonus2", "<i4"),
                      ("xdrop", "<i4"), ("sc_index", "<u4")], align=True)
RESULT_DTYPE = np.dtype([("score", "<i4"), ("distance", "<u4"), ("pattern_end", "<u8"),
                         ("text_start", "<u8"), ("text_end", "<u8"), ("text_read", "<u8"),
                         ("cells", "<u8"), ("cigar_off", "<u8"), ("n_ops", "<u4"),
                         ("status", "<i4")], align=True)
assert JOB_DTYPE.itemsize == C.sizeof(_abi.JobT)
assert RESULT_DTYPE.itemsize == C.sizeof(_abi.ResultT)


def new_jobs(count: int) -> np.ndarray:
    j = np.zeros(count, dtype=JOB_DTYPE)
    j["k"] = 0xFFFFFFFF
    j["band"] = _abi.SF_NOLIMIT
    j["xdrop"] = 2 ** 31 - 1
    return j


class Context:
    """A device context: one CUDA stream (plus fan-out streams) on one GPU."""

    def __init__(self, device: int = 0):
        self._lib = _abi.load()
        h = C.c_void_p()
        _abi.check(self._lib.sf_context_create(int(device), C.byref(h)))
        self.handle = h

    def use_store(self, store: Optional["Store"]) -> None:
        """Later plans resolve TEXT_STORE texts in `store` (None: no store)."""
        _abi.check(self._lib.sf_context_use_store(self.handle, store.handle if store else None))

    def untune(self) -> None:
        """Drops the autotuner's choices: later plans use the default kernel classes."""
        _abi.check(self._lib.sf_context_untune(self.handle))

    def close(self):
        if self.handle:
            self._lib.sf_context_destroy(self.handle)
            self.handle = None

    def __del__(self):  # pragma: no cover - interpreter teardown
        try:
            self.close()
        except Exception:
            pass


TEXT_POOL, TEXT_STORE = 0, 1


class Store:
    """The index's transcripts packed once in HBM (sf_store_*): jobs of plans built in a
    context that uses it name texts as windows (text_src = TEXT_STORE, t_off = the first
    base in the transcripts' concatenation, n = the window's length)."""

    def __init__(self, ctx: "Context", transcripts=None, packed=None, bases: int = 0):
        self._lib = _abi.load()
        h = C.c_void_p()
        if packed is not None:
            w = np.ascontiguousarray(packed, dtype=np.uint64)
            _abi.check(self._lib.sf_store_create_packed(
                ctx.handle, w.ctypes.data_as(C.POINTER(C.c_uint64)), int(bases), C.byref(h)))
            self.starts = None
        else:
            parts = [np.ascontiguousarray(np.asarray(t, dtype=np.uint8)) for t in transcripts]
            lens = np.array([p.size for p in parts], dtype=np.uint64)
            codes = np.concatenate(parts) if parts else np.zeros(1, np.uint8)
            _abi.check(self._lib.sf_store_create(
                ctx.handle, codes.ctypes.data_as(C.POINTER(C.c_uint8)),
                lens.ctypes.data_as(C.POINTER(C.c_uint64)), len(parts), C.byref(h)))
            self.starts = np.concatenate([[0], np.cumsum(lens)[:-1]]).astype(np.uint64) \
                if len(parts) else np.zeros(0, np.uint64)
        self.handle = h

    @property
    def bases(self) -> int:
        return int(self._lib.sf_store_bases(self.handle))

    def close(self):
        if self.handle:
            self._lib.sf_store_destroy(self.handle)
            self.handle = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass


@dataclass
class Output:
    results: np.ndarray  # RESULT_DTYPE
    ops: np.ndarray      # uint32 CIGAR ops, per job at results["cigar_off"]

    def cigar(self, q: int) -> list[int]:
        r = self.results[q]
        o = int(r["cigar_off"])
        return [int(v) for v in self.ops[o:o + int(r["n_ops"])]]


class Plan:
    """Jobs prepared once: device descriptors, buckets and buffers; run many times."""

    def __init__(self, ctx: Context, jobs: np.ndarray, pool_bytes: int,
                 scores: Sequence = (Affine.ONT,)):
        self._lib = _abi.load()
        self.ctx = ctx
        self.jobs = np.ascontiguousarray(jobs, dtype=JOB_DTYPE)
        self._scores = (_abi.Affine * max(1, len(scores)))(*[_aff(s) for s in scores])
        h = C.c_void_p()
        _abi.check(self._lib.sf_plan_create(
            ctx.handle, self.jobs.ctypes.data_as(C.POINTER(_abi.JobT)), len(self.jobs),
            self._scores, len(scores), int(pool_bytes), C.byref(h)))
        self.handle = h
        self.pool_bytes = int(pool_bytes)

    def upload(self, pool: np.ndarray) -> None:
        pool = np.ascontiguousarray(pool, dtype=np.uint8)
        if pool.size < self.pool_bytes:
            raise ValueError("pool smaller than the plan's pool_bytes")
        _abi.check(self._lib.sf_plan_upload(self.handle,
                                            pool.ctypes.data_as(C.POINTER(C.c_uint8))))

    def execute(self) -> None:
        _abi.check(self._lib.sf_plan_execute(self.handle))

    def sync(self) -> None:
        _abi.check(self._lib.sf_plan_sync(self.handle))

    def stream(self) -> int:
        return int(self._lib.sf_plan_stream(self.handle) or 0)

    def launches(self) -> int:
        return int(self._lib.sf_plan_launches(self.handle))

    def profile(self) -> list[float]:
        """One execute in order with events between stages: ms of pack, each bucket (in
        `describe()` order, walks included), then the CIGAR compaction."""
        ms = (C.c_float * 256)()
        n = C.c_uint32()
        _abi.check(self._lib.sf_plan_profile(self.handle, ms, 256, C.byref(n)))
        return [float(ms[i]) for i in range(n.value)]

    def describe(self) -> str:
        return self._lib.sf_plan_describe(self.handle).decode()

    def job_buckets(self) -> np.ndarray:
        """Each job's bucket: its index in `describe()`'s bucket list (sf_plan_job_buckets;
        0xFFFFFFFF for a job a row-sharing chain runs)."""
        out = np.zeros(max(1, len(self.jobs)), dtype=np.uint32)
        _abi.check(self._lib.sf_plan_job_buckets(self.handle,
                                                 out.ctypes.data_as(C.POINTER(C.c_uint32)),
                                                 len(self.jobs)))
        return out[:len(self.jobs)]

    def tune(self, pool: np.ndarray, reps: int = 3) -> dict:
        """Autotunes the kernel classes of this plan's length buckets (sf_plan_tune): the
        choices stay in the context for later plans; the plan is rebuilt and its pool
        uploaded again.  Returns the tuner's report."""
        import json
        pool = np.ascontiguousarray(pool, dtype=np.uint8)
        buf = C.create_string_buffer(1 << 20)
        _abi.check(self._lib.sf_plan_tune(self.handle, pool.ctypes.data_as(C.POINTER(C.c_uint8)),
                                          int(reps), buf, len(buf)))
        return json.loads(buf.value.decode())

    def download(self, ops_cap: Optional[int] = None) -> Output:
        res = np.zeros(len(self.jobs), dtype=RESULT_DTYPE)
        if ops_cap is None:
            want = self.jobs["want_cigar"] != 0
            ops_cap = int((self.jobs["m"][want].astype(np.uint64) +
                           self.jobs["n"][want] + 2).sum()) if want.any() else 0
        ops = np.zeros(max(1, ops_cap), dtype=np.uint32)
        used = C.c_uint64()
        _abi.check(self._lib.sf_plan_download(
            self.handle, res.ctypes.data_as(C.POINTER(_abi.ResultT)),
            ops.ctypes.data_as(C.POINTER(C.c_uint32)), ops_cap, C.byref(used)))
        return Output(res, ops[:used.value])

    def close(self):
        if self.handle:
            self._lib.sf_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass


def run(ctx: Context, pool: np.ndarray, jobs: np.ndarray,
        scores: Sequence = (Affine.ONT,)) -> Output:
    """One call: plan, upload, execute, download (sf_batch_run)."""
    lib = _abi.load()
    pool = np.ascontiguousarray(pool, dtype=np.uint8)
    jobs = np.ascontiguousarray(jobs, dtype=JOB_DTYPE)
    sc = (_abi.Affine * max(1, len(scores)))(*[_aff(s) for s in scores])
    res = np.zeros(len(jobs), dtype=RESULT_DTYPE)
    want = jobs["want_cigar"] != 0
    cap = int((jobs["m"][want].astype(np.uint64) + jobs["n"][want] + 2).sum()) if want.any() else 0
    ops = np.zeros(max(1, cap), dtype=np.uint32)
    used = C.c_uint64()
    _abi.check(lib.sf_batch_run(ctx.handle, pool.ctypes.data_as(C.POINTER(C.c_uint8)), pool.size,
                                jobs.ctypes.data_as(C.POINTER(_abi.JobT)), len(jobs), sc,
                                len(scores), res.ctypes.data_as(C.POINTER(_abi.ResultT)),
                                ops.ctypes.data_as(C.POINTER(C.c_uint32)), cap, C.byref(used)))
    return Output(res, ops[:used.value])


class PoolBuilder:
    """Concatenates byte-code sequences into one pool, returning each one's offset."""

    def __init__(self):
        self.parts: list[np.ndarray] = []
        self.size = 0

    def add(self, codes) -> int:
        a = np.ascontiguousarray(np.asarray(codes, dtype=np.uint8))
        off = self.size
        self.parts.append(a)
        self.size += a.size
        return off

    def build(self) -> np.ndarray:
        if not self.parts:
            return np.zeros(1, dtype=np.uint8)
        return np.concatenate(self.parts)


__all__ = ["Context", "Plan", "Output", "run", "new_jobs", "PoolBuilder", "JOB_DTYPE",
           "RESULT_DTYPE", "JOB_MYERS", "JOB_AFFINE", "JOB_EXTEND_WINDOW", "JOB_LOCAL", "Mode"]
