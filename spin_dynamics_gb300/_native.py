"""ctypes binding of libspinchem_gpu.so (the C ABI in include/spinchem_gpu.h).

The library is built in-tree by `spin_dynamics_gb300.build`. There is no CPU
fallback: if the library is missing or cannot be loaded, `lib()` raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

SPC_OK = 0
SPC_ERR_ARG = 1
SPC_ERR_CUDA = 2
SPC_ERR_ALLOC = 3
SPC_ERR_UNSUPPORTED = 4
SPC_ERR_NUMERIC = 5
SPC_ERR_STATE = 6
SPC_H_REFERENCE = 0
SPC_H_GENERAL = 1
SPC_GRAD_ALL = 0
SPC_GRAD_FIELD = 1
SPC_KRYLOV_MGS = 0
SPC_KRYLOV_LANCZOS = 1
SPC_KRYLOV_AUTO = 2


class SpcError(RuntimeError):
    """A libspinchem_gpu call returned a nonzero status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[spc error {code}] {msg}")
        self.code = code


class spc_system(C.Structure):
    _fields_ = [("n_nuc1", C.c_int), ("n_nuc2", C.c_int),
                ("mult1", C.POINTER(C.c_int)), ("mult2", C.POINTER(C.c_int)),
                ("A1", C.POINTER(C.c_double)), ("A2", C.POINTER(C.c_double)),
                ("gamma1", C.POINTER(C.c_double)), ("gamma2", C.POINTER(C.c_double)),
                ("B", C.c_double * 3), ("J", C.c_double), ("D", C.c_double * 9),
                ("kS", C.c_double), ("kT", C.c_double)]


class spc_csr(C.Structure):
    _fields_ = [("n", C.c_int32), ("nnz", C.c_int64), ("rowptr", C.POINTER(C.c_int32)),
                ("col", C.POINTER(C.c_int32)), ("val", C.POINTER(C.c_double)),
                ("index_base", C.c_int32)]


class spc_stats(C.Structure):
    _fields_ = [("krylov_builds", C.c_int64), ("lanczos_fallbacks", C.c_int64),
                ("rounds", C.c_int64), ("sample_steps", C.c_int64),
                ("kernel_launches", C.c_int64), ("seconds", C.c_double)]


# every symbol the header declares, with (restype, argtypes)
_P = C.c_void_p
_D = C.c_double
_I = C.c_int
SIGNATURES = {
    "spc_last_error": (C.c_char_p, []),
    "spc_create": (_I, [_I, C.POINTER(_P)]),
    "spc_destroy": (_I, [_P]),
    "spc_set_stream": (_I, [_P, _P]),
    "spc_build_h": (_I, [_P, C.POINTER(spc_system), _I]),
    "spc_set_h": (_I, [_P, C.POINTER(spc_csr)]),
    "spc_build_h_noalloc": (_I, [C.POINTER(spc_system), _I, _P, _P, _P, C.c_int64,
                                 C.POINTER(C.c_int32), C.POINTER(C.c_int64), _P]),
    "spc_h_size": (_I, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int64)]),
    "spc_get_h": (_I, [_P, _P, _P, _P]),
    "spc_num_time_points": (_I, [_D, _D]),
    "spc_trace_sampling": (_I, [_P, _P, _P, _P, _I, _D, _D, _I, _D, _P, _P, _P, _P, _I]),
    "spc_trace_sampling_device": (_I, [_P, _P, _P, _P, _I, _D, _D, _I, _D, _P, _I]),
    "spc_get_stats": (_I, [_P, C.POINTER(spc_stats)]),
    "spc_seeded_samples": (_I, [C.c_int64, C.c_int64, _I, _I, _I, _P]),
    "spc_init_el_state": (_I, [_I, _P, _P]),
    "spc_rng_stream": (_I, [C.c_int64, C.c_int64, _I, _P]),
    "spc_kinetics": (_I, [_I, _P, _P, _P, _P, _D, _D, _D, _P, _P, _P]),
    "spc_set_krylov": (_I, [_P, _I]),
    "spc_build_h_batch": (_I, [_P, _I, _P, _I]),
    "spc_trace_sampling_batch": (_I, [_P, _I, _P, _P, _P, _P, _P, _D, _D, _I, _D, _P, _I]),
    "spc_trace_sampling_batch_device": (_I, [_P, _I, _P, _P, _P, _P, _P, _D, _D, _I, _D, _P, _I]),
    "spc_yield_gradient_size": (_I, [C.POINTER(spc_system)]),
    "spc_gradient_nodes": (_I, [C.POINTER(spc_system), _D, C.POINTER(_I)]),
    "spc_yield_gradient": (_I, [_P, C.POINTER(spc_system), _P, _P, _I, _D, _D, _I, _I, _I, _D, _D, _P,
                                _P]),
    "spc_yield_gradient_batch": (_I, [_P, _I, _P, _P, _P, _P, _D, _D, _I, _I, _I, _D, _D, _I, _P, _P]),
    "spc_autotune_krylov": (_I, [_P, _I, _P, _P, _P, _P, _P, _D, _D, _D, _P, _I, _P, _P]),
    "spc_set_graphs": (_I, [_P, _I]),
    "spc_set_memory_limit": (_I, [_P, C.c_int64]),
    "spc_set_sample_path": (_I, [_P, _I]),
    "spc_mem_info": (_I, [_I, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "spc_set_profiling": (_I, [_P, _I]),
    "spc_get_profile": (_I, [_P, _I, C.POINTER(_D), C.POINTER(C.c_int64), C.POINTER(_D),
                             C.POINTER(_D)]),
    "spc_kernel_kind_name": (C.c_char_p, [_I]),
    "spc_fp64_peak": (_I, [_I, C.POINTER(_D)]),
}
SPC_KERNEL_KINDS = 14
SPC_SAMPLE_AUTO, SPC_SAMPLE_OFF, SPC_SAMPLE_ON, SPC_SAMPLE_SINGLE = 0, 1, 2, 3

_LIB: C.CDLL | None = None


def lib_path() -> str:
    return _build.LIB


def lib(build_if_missing: bool = True) -> C.CDLL:
    """Load libspinchem_gpu.so (building it with nvcc if absent)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise OSError(f"{path} is missing: run `python -m spin_dynamics_gb300.build`")
        _build.build()
    L = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _LIB = L
    return L


def check(rc: int) -> None:
    if rc != SPC_OK:
        msg = lib().spc_last_error()
        raise SpcError(rc, msg.decode() if msg else "")
