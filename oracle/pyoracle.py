"""ORACLE — test infrastructure only.

ctypes wrapper around oracle/_build/liboracle.so, the C++ restatement of the
reference trace-sampling path (see spinchem_oracle.cpp for the per-function
citations). Only tests/, __graft_entry__.smoke() and bench.py's CPU legs use
this module; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIBS: dict[bool, C.CDLL] = {}

_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")


def build() -> None:
    """Compile both oracle builds (parity and timed baseline) with make."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib(fast: bool = False) -> C.CDLL:
    if fast in _LIBS:
        return _LIBS[fast]
    path = os.path.join(HERE, "_build", "liboracle_fast.so" if fast else "liboracle.so")
    if not os.path.exists(path):
        build()
    L = C.CDLL(path)
    L.orc_set_threads.argtypes = [C.c_int]
    L.orc_set_threads.restype = C.c_int
    L.orc_rng_stream.argtypes = [C.c_uint64, C.c_uint64, C.c_int, C.c_int, _u64p]
    L.orc_rng_normals.argtypes = [C.c_uint64, C.c_uint64, C.c_int, _f64p]
    L.orc_seeded_samples.argtypes = [C.c_uint64, C.c_uint64, C.c_int, C.c_int, C.c_int, _f64p]
    hargs = [C.c_int, _i32p, _f64p, C.c_int, _i32p, _f64p, C.c_double, C.c_double, _f64p,
             C.c_double, C.c_double, C.c_long, C.c_void_p, C.c_void_p, C.c_void_p]
    L.orc_build_h_iso.argtypes = hargs
    L.orc_build_h_iso.restype = C.c_long
    L.orc_build_h_iso_coo.argtypes = hargs
    L.orc_build_h_iso_coo.restype = C.c_long
    L.orc_build_h_general.argtypes = [C.c_int, _i32p, _f64p, _f64p, C.c_int, _i32p, _f64p, _f64p,
                                      _f64p, C.c_double, _f64p, C.c_double, C.c_double, C.c_long,
                                      C.c_void_p, C.c_void_p, C.c_void_p]
    L.orc_build_h_general.restype = C.c_long
    L.orc_expm.argtypes = [C.c_int, _f64p, _f64p]
    L.orc_num_time_points.argtypes = [C.c_double, C.c_double]
    L.orc_num_time_points.restype = C.c_int
    L.orc_init_el_state.argtypes = [C.c_int, _f64p, _f64p]
    L.orc_trace_sampling.argtypes = [C.c_int, _i32p, _i32p, _f64p, _f64p, _f64p, _f64p, C.c_int,
                                     C.c_double, C.c_double, C.c_int, C.c_double, _f64p, _f64p,
                                     _f64p, _f64p, C.c_int, C.c_void_p, C.c_void_p]
    L.orc_kinetics.argtypes = [C.c_int, _f64p, _f64p, _f64p, _f64p, C.c_double, C.c_double,
                               C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]
    _LIBS[fast] = L
    return L


def set_threads(n: int, fast: bool = False) -> int:
    return lib(fast).orc_set_threads(n)


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def rng_stream(seed, n, do_seed=True):
    out = np.zeros(n, np.uint64)
    lib().orc_rng_stream(int(seed[0]) & (2**64 - 1), int(seed[1]) & (2**64 - 1), int(do_seed), n, out)
    return out


def rng_normals(seed, n):
    out = np.zeros(n, np.float64)
    lib().orc_rng_normals(int(seed[0]) & (2**64 - 1), int(seed[1]) & (2**64 - 1), n, out)
    return out


def seeded_samples(seed, Z, M, mode=0):
    """M x Z complex samples exactly as trace_sampling_para draws them."""
    out = np.zeros(2 * Z * M, np.float64)
    lib().orc_seeded_samples(int(seed[0]) & (2**64 - 1), int(seed[1]) & (2**64 - 1), Z, M, mode, out)
    return out.view(np.complex128).reshape(M, Z)


def _iso_args(g1, a1, g2, a2, B, J, D, kS, kT):
    g1 = np.ascontiguousarray(g1, np.int32)
    g2 = np.ascontiguousarray(g2, np.int32)
    a1 = np.ascontiguousarray(a1, np.float64)
    a2 = np.ascontiguousarray(a2, np.float64)
    D9 = np.ascontiguousarray(np.asarray(D, np.float64).reshape(3, 3).T.reshape(9))  # column-major
    return [len(g1), g1, a1 if a1.size else np.zeros(1), len(g2), g2, a2 if a2.size else np.zeros(1),
            float(B), float(J), D9, float(kS), float(kT)]


def build_h_iso(g1, a1, g2, a2, B, J, D, kS, kT):
    """getHiso_sp + coo_to_csr. D is a 3x3 (row, col) array. Returns (rowptr, col, val) 0-based."""
    args = _iso_args(g1, a1, g2, a2, B, J, D, kS, kT)
    L = lib()
    nnz = L.orc_build_h_iso(*args, 0, None, None, None)
    if nnz < 0:
        raise ValueError("getHiso_sp refused the system (code %d)" % nnz)
    N = 4 * int(np.prod(args[1])) * int(np.prod(args[4]))
    rp = np.zeros(N + 1, np.int32)
    col = np.zeros(nnz, np.int32)
    val = np.zeros(2 * nnz, np.float64)
    L.orc_build_h_iso(*args, nnz, _ptr(rp), _ptr(col), _ptr(val))
    return rp, col, val.view(np.complex128)


def build_h_iso_coo(g1, a1, g2, a2, B, J, D, kS, kT):
    args = _iso_args(g1, a1, g2, a2, B, J, D, kS, kT)
    L = lib()
    nnz = L.orc_build_h_iso_coo(*args, 0, None, None, None)
    if nnz < 0:
        raise ValueError("getHiso_sp refused the system (code %d)" % nnz)
    r = np.zeros(nnz, np.int32)
    c = np.zeros(nnz, np.int32)
    v = np.zeros(2 * nnz, np.float64)
    L.orc_build_h_iso_coo(*args, nnz, _ptr(r), _ptr(c), _ptr(v))
    return r, c, v.view(np.complex128)


def build_h_general(g1, A1, gam1, g2, A2, gam2, Bvec, J, D, kS, kT):
    """General anisotropic H. A1/A2: (n,3,3) row/col tensors. Returns (rowptr, col, val)."""
    g1 = np.ascontiguousarray(g1, np.int32)
    g2 = np.ascontiguousarray(g2, np.int32)
    # column-major 3x3 per nucleus, as input.ini stores them
    A1c = np.ascontiguousarray(np.asarray(A1, np.float64).reshape(-1, 3, 3).transpose(0, 2, 1).reshape(-1))
    A2c = np.ascontiguousarray(np.asarray(A2, np.float64).reshape(-1, 3, 3).transpose(0, 2, 1).reshape(-1))
    gam1 = np.ascontiguousarray(gam1, np.float64)
    gam2 = np.ascontiguousarray(gam2, np.float64)
    D9 = np.ascontiguousarray(np.asarray(D, np.float64).reshape(3, 3).T.reshape(9))
    Bv = np.ascontiguousarray(Bvec, np.float64)
    one = np.zeros(1)
    args = [len(g1), g1, A1c if A1c.size else one, gam1 if gam1.size else one,
            len(g2), g2, A2c if A2c.size else one, gam2 if gam2.size else one,
            Bv, float(J), D9, float(kS), float(kT)]
    L = lib()
    nnz = L.orc_build_h_general(*args, 0, None, None, None)
    N = 4 * int(np.prod(g1)) * int(np.prod(g2))
    rp = np.zeros(N + 1, np.int32)
    col = np.zeros(nnz, np.int32)
    val = np.zeros(2 * nnz, np.float64)
    L.orc_build_h_general(*args, nnz, _ptr(rp), _ptr(col), _ptr(val))
    return rp, col, val.view(np.complex128)


def expm(A):
    A = np.asarray(A, np.complex128)
    n = A.shape[0]
    a = np.ascontiguousarray(A.T).view(np.float64).reshape(-1)  # column-major
    e = np.zeros(2 * n * n, np.float64)
    if lib().orc_expm(n, np.ascontiguousarray(a), e) != 0:
        raise FloatingPointError("singular Pade denominator")
    return e.view(np.complex128).reshape(n, n).T.copy()


def num_time_points(dt, t_end):
    return lib().orc_num_time_points(float(dt), float(t_end))


def init_el_state(which):
    idx = {"singlet": 0, "T0": 1, "Tp": 2, "Tm": 3}[which]
    th = np.zeros(8)
    pop = np.zeros(4)
    lib().orc_init_el_state(idx, th, pop)
    return th.view(np.complex128), pop


def trace_sampling(rowptr, col, val, zkets, dt, t_end, m, tol, init_state="singlet",
                   per_sample=False, fast=False, threads=0):
    """trace_sampling_para on caller-supplied samples (M x Z complex).

    Returns dict with P_S, P_T0, P_Tp, P_Tm (length T), n_builds (M,) and
    optionally per_sample (M, 4, T)."""
    L = lib(fast)
    if threads:
        L.orc_set_threads(threads)
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    v = np.ascontiguousarray(np.asarray(val, np.complex128)).view(np.float64)
    zk = np.ascontiguousarray(np.asarray(zkets, np.complex128))
    M, Z = zk.shape
    N = len(rowptr) - 1
    assert N == 4 * Z
    th, pop = init_el_state(init_state)
    T = num_time_points(dt, t_end)
    outs = [np.zeros(T) for _ in range(4)]
    ps = np.zeros(M * 4 * T) if per_sample else None
    nb = np.zeros(M, np.int64)
    rc = L.orc_trace_sampling(N, rowptr, col, v, np.ascontiguousarray(th.view(np.float64)), pop,
                              zk.view(np.float64).reshape(-1), M, float(dt), float(t_end), int(m),
                              float(tol), *outs, T, _ptr(ps), _ptr(nb))
    if rc != 0:
        raise RuntimeError("oracle trace_sampling failed")
    res = dict(P_S=outs[0], P_T0=outs[1], P_Tp=outs[2], P_Tm=outs[3], n_builds=nb, T=T)
    if per_sample:
        res["per_sample"] = ps.reshape(M, 4, T)
    return res


def kinetics(P_S, P_T0, P_Tp, P_Tm, dt, kS, kT):
    T = len(P_S)
    nh = T // 2
    phis = np.zeros(nh)
    phit = np.zeros(nh)
    iden = np.zeros(T)
    lib().orc_kinetics(T, *(np.ascontiguousarray(x, np.float64) for x in (P_S, P_T0, P_Tp, P_Tm)),
                       float(dt), float(kS), float(kT), _ptr(phis), _ptr(phit), _ptr(iden))
    return phis, phit, iden
