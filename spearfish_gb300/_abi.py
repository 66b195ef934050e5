"""ctypes binding of libsf_align.so (include/sf_align.h).

The library is the product: every entry point computes on the GPU.  Loading fails loudly
when the library has not been built; no call has a CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libsf_align.so")

SF_OK = 0
ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "out of memory", -4: "too long",
          -5: "timeout", -6: "capacity", -7: "busy"}
SF_NONE = 0xFFFFFFFF
SF_NOLIMIT = (1 << 64) - 1
SF_NEG = -(2 ** 31) // 4


class SfError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"sf_align error {code} ({ERRORS.get(code, '?')}): {msg}")
        self.code = code


class Affine(C.Structure):
    _fields_ = [("mat", C.c_int32), ("mis", C.c_int32), ("open", C.c_int32), ("ext", C.c_int32)]


class ExtendT(C.Structure):
    _fields_ = [("score", C.c_int32), ("pad_", C.c_int32), ("pattern_bases", C.c_uint64),
                ("text_bases", C.c_uint64), ("text_read", C.c_uint64)]


class CutT(C.Structure):
    _fields_ = [("whole", C.c_int32), ("cut", C.c_int32), ("cols", C.c_uint64)]


class CigarT(C.Structure):
    _fields_ = [("score", C.c_int32), ("status", C.c_int32), ("pattern_end", C.c_uint64),
                ("text_start", C.c_uint64), ("text_end", C.c_uint64), ("n_ops", C.c_uint64)]


class JobT(C.Structure):
    _fields_ = [("p_off", C.c_uint64), ("t_off", C.c_uint64), ("m", C.c_uint32),
                ("n", C.c_uint32), ("kind", C.c_uint8), ("mode", C.c_uint8),
                ("want_cigar", C.c_uint8), ("text_src", C.c_uint8), ("k", C.c_uint32),
                ("band", C.c_uint64), ("window", C.c_uint64), ("dlo", C.c_int64),
                ("dhi", C.c_int64), ("end_bonus", C.c_int32), ("end_bonus2", C.c_int32),
                ("xdrop", C.c_int32), ("sc_index", C.c_uint32)]


class SpanT(C.Structure):
    _fields_ = [("off", C.c_uint64), ("len", C.c_uint64)]


class BandedReadT(C.Structure):
    _fields_ = [("p_off", C.c_uint64), ("first", C.c_uint64), ("m", C.c_uint32),
                ("count", C.c_uint32), ("mode", C.c_uint32), ("cap", C.c_uint32),
                ("distinct", C.c_uint32), ("pad_", C.c_uint32)]


class EndsT(C.Structure):
    _fields_ = [("sc", Affine), ("band", C.c_uint64), ("end_bonus", C.c_int32),
                ("xdrop", C.c_int32), ("pad", C.c_uint32), ("pad_div", C.c_uint32)]


class HitT(C.Structure):
    _fields_ = [("read_off", C.c_uint64), ("tx_start", C.c_uint64), ("read_len", C.c_uint32),
                ("tx_len", C.c_uint32), ("qstart", C.c_uint32), ("qend", C.c_uint32),
                ("tstart", C.c_uint32), ("tend", C.c_uint32)]


class SortedCallT(C.Structure):
    _fields_ = [("p_off", C.c_uint64), ("first", C.c_uint64), ("band", C.c_uint64),
                ("window", C.c_uint64), ("cut", C.c_uint64), ("m", C.c_uint32),
                ("count", C.c_uint32), ("kind", C.c_uint32), ("mode", C.c_uint32),
                ("end_bonus", C.c_int32), ("xdrop", C.c_int32), ("diagonal", C.c_uint32),
                ("track_cut", C.c_uint32), ("bonus_within_cut", C.c_uint32),
                ("sc_index", C.c_uint32)]


class ResultT(C.Structure):
    _fields_ = [("score", C.c_int32), ("distance", C.c_uint32), ("pattern_end", C.c_uint64),
                ("text_start", C.c_uint64), ("text_end", C.c_uint64), ("text_read", C.c_uint64),
                ("cells", C.c_uint64), ("cigar_off", C.c_uint64), ("n_ops", C.c_uint32),
                ("status", C.c_int32)]


class ServerOpts(C.Structure):
    _fields_ = [("device", C.c_int), ("slots", C.c_uint32), ("hbm_budget", C.c_uint64),
                ("scores", C.POINTER(Affine)), ("n_scores", C.c_uint32), ("store", C.c_void_p)]


class RequestStats(C.Structure):
    _fields_ = [("queue_ms", C.c_double), ("run_ms", C.c_double), ("total_ms", C.c_double),
                ("cells", C.c_uint64), ("slot", C.c_uint32), ("status", C.c_int32)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("failed", C.c_uint64),
                ("cells", C.c_uint64), ("hbm_budget", C.c_uint64), ("hbm_held", C.c_uint64),
                ("slots", C.c_uint32), ("busy_slots", C.c_uint32), ("pending", C.c_uint32),
                ("pad_", C.c_uint32)]


# Every symbol include/sf_align.h declares, with (restype, argtypes).
_u8p = C.POINTER(C.c_uint8)
_u8pp = C.POINTER(_u8p)
_u64p = C.POINTER(C.c_uint64)
_u32p = C.POINTER(C.c_uint32)
_i32p = C.POINTER(C.c_int32)
_aff = C.POINTER(Affine)
_vp = C.c_void_p

SIGNATURES = {
    "sf_last_error": (C.c_char_p, []),
    "sf_version": (C.c_char_p, []),
    "sf_set_device": (C.c_int, [C.c_int]),
    "sf_distance": (C.c_int, [_u8p, C.c_uint64, _u8p, C.c_uint64, C.c_int, C.c_uint32, _u32p]),
    "sf_batch_distances": (C.c_int, [_u8p, C.c_uint64, _u8pp, _u64p, C.c_uint64, C.c_int,
                                     C.c_uint32, _u32p]),
    "sf_store_create": (C.c_int, [_vp, _u8p, _u64p, C.c_uint64, C.POINTER(_vp)]),
    "sf_store_create_packed": (C.c_int, [_vp, _u64p, C.c_uint64, C.POINTER(_vp)]),
    "sf_store_destroy": (None, [_vp]),
    "sf_store_bases": (C.c_uint64, [_vp]),
    "sf_context_use_store": (C.c_int, [_vp, _vp]),
    "sf_extend_ends_batch": (C.c_int, [_vp, _u8p, C.c_uint64, C.POINTER(EndsT), C.POINTER(HitT),
                                       C.c_uint64]),
    "sf_sorted_batch": (C.c_int, [_vp, _u8p, C.c_uint64, _aff, C.c_uint32, C.POINTER(SortedCallT),
                                  C.c_uint64, C.POINTER(SpanT), C.c_uint64, C.POINTER(CutT)]),
    "sf_banded": (C.c_int, [_u8p, C.c_uint64, _u8pp, _u64p, C.c_uint64, C.c_int, C.c_uint32,
                            C.c_int, _u32p]),
    "sf_banded_batch": (C.c_int, [_vp, _u8p, C.c_uint64, C.POINTER(BandedReadT), C.c_uint64,
                                  C.POINTER(SpanT), C.c_uint64, _u32p]),
    "sf_infix_distance": (C.c_int, [_u8p, C.c_uint64, _u8p, C.c_uint64, _u32p]),
    "sf_affine": (C.c_int, [_u8p, C.c_uint64, _u8p, C.c_uint64, C.c_int, _aff, C.c_uint64,
                            _i32p]),
    "sf_affine_extend": (C.c_int, [_u8p, C.c_uint64, _u8p, C.c_uint64, _aff, C.c_uint64,
                                   C.c_int32, C.c_int32, _i32p]),
    "sf_affine_extend_window": (C.c_int, [_u8p, C.c_uint64, _u8p, C.c_uint64, C.c_uint64, _aff,
                                          C.c_uint64, C.c_int32, C.c_int32, C.POINTER(ExtendT)]),
    "sf_affine_sorted": (C.c_int, [_u8p, C.c_uint64, _u8pp, _u64p, C.c_uint64, C.c_int, _aff,
                                   C.c_uint64, _i32p]),
    "sf_affine_extend_sorted_cut": (C.c_int, [_u8p, C.c_uint64, _u8pp, _u64p, C.c_uint64, _aff,
                                              C.c_uint64, C.c_int32, C.c_int32, C.c_int,
                                              C.c_uint64, C.c_uint64, C.POINTER(CutT)]),
    "sf_affine_extend_sorted_cut_bonus": (C.c_int, [_u8p, C.c_uint64, _u8pp, _u64p, C.c_uint64,
                                                    _aff, C.c_uint64, C.c_int32, C.c_int32,
                                                    C.c_int, C.c_uint64, C.c_uint64, C.c_int,
                                                    C.c_int, C.POINTER(CutT)]),
    "sf_local_band": (C.c_int, [_u8p, C.c_uint64, _u8p, C.c_uint64, _aff, C.c_int64, C.c_int64,
                                C.c_int32, _i32p]),
    "sf_local_band_ends": (C.c_int, [_u8p, C.c_uint64, _u8p, C.c_uint64, _aff, C.c_int64,
                                     C.c_int64, C.c_int32, C.c_int32, _i32p]),
    "sf_dp_work": (None, [_u64p, _u64p]),
    "sf_affine_cigar": (C.c_int, [_u8p, C.c_uint64, _u8p, C.c_uint64, C.c_int, _aff, C.c_uint64,
                                  _u32p, C.c_uint64, C.POINTER(CigarT)]),
    "sf_affine_extend_window_cigar": (C.c_int, [_u8p, C.c_uint64, _u8p, C.c_uint64, C.c_uint64,
                                                _aff, C.c_uint64, C.c_int32, C.c_int32, _u32p,
                                                C.c_uint64, C.POINTER(CigarT)]),
    "sf_context_create": (C.c_int, [C.c_int, C.POINTER(_vp)]),
    "sf_context_destroy": (None, [_vp]),
    "sf_plan_create": (C.c_int, [_vp, C.POINTER(JobT), C.c_uint64, _aff, C.c_uint32, C.c_uint64,
                                 C.POINTER(_vp)]),
    "sf_plan_destroy": (None, [_vp]),
    "sf_plan_upload": (C.c_int, [_vp, _u8p]),
    "sf_plan_execute": (C.c_int, [_vp]),
    "sf_plan_download": (C.c_int, [_vp, C.POINTER(ResultT), _u32p, C.c_uint64, _u64p]),
    "sf_plan_sync": (C.c_int, [_vp]),
    "sf_plan_stream": (_vp, [_vp]),
    "sf_plan_launches": (C.c_uint64, [_vp]),
    "sf_plan_describe": (C.c_char_p, [_vp]),
    "sf_plan_job_buckets": (C.c_int, [_vp, _u32p, C.c_uint64]),
    "sf_plan_profile": (C.c_int, [_vp, C.POINTER(C.c_float), C.c_uint32, _u32p]),
    "sf_plan_tune": (C.c_int, [_vp, C.POINTER(C.c_uint8), C.c_uint32, C.c_char_p, C.c_uint64]),
    "sf_context_untune": (C.c_int, [_vp]),
    "sf_server_create": (C.c_int, [C.POINTER(ServerOpts), C.POINTER(_vp)]),
    "sf_server_destroy": (None, [_vp]),
    "sf_server_submit": (C.c_int, [_vp, _u8p, C.c_uint64, C.POINTER(JobT), C.c_uint64, _u64p]),
    "sf_server_wait": (C.c_int, [_vp, C.c_uint64, C.c_int32, C.POINTER(ResultT), _u32p,
                                 C.c_uint64, _u64p, C.POINTER(RequestStats)]),
    "sf_server_query": (C.c_int, [_vp, C.POINTER(ServerStats)]),
    "sf_affine_noalloc": (C.c_int, [C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64, C.c_int, _aff,
                                    C.c_uint64, C.c_void_p, C.c_void_p]),
    "sf_int_peak": (C.c_int, [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "sf_batch_run": (C.c_int, [_vp, _u8p, C.c_uint64, C.POINTER(JobT), C.c_uint64, _aff,
                               C.c_uint32, C.POINTER(ResultT), _u32p, C.c_uint64, _u64p]),
}

_lib = None


def load(path: str = LIB_PATH):
    """Loads the library and declares every symbol; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build it with `python -m spearfish_gb300.build` (nvcc, sm_103a). "
            "There is no CPU fallback.")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int) -> None:
    if rc != SF_OK:
        msg = load().sf_last_error()
        raise SfError(rc, msg.decode() if msg else "")
