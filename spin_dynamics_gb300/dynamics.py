"""Host-side mirror of module `dynamics` (src/qm_dynamics.f90) over the C ABI.

`TraceSampler` owns one libspinchem_gpu handle (one GPU, one stream). The
module-level functions keep the reference's names and argument meaning:

  trace_sampling_para(sys, sim, out=None)   src/qm_dynamics.f90:257-384
  trace_sampling(sys, sim, out=None)        src/qm_dynamics.f90:139-255
  exact_dynamics(sys, sim, out=None)        src/qm_dynamics.f90:24-137

`sys.e1.w` / `sys.e2.w` carry the Larmor frequency w = -B that the driver
sets per field (app/main.f90:53-54), exactly as in the reference.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import _native as nat
from .observables import Observables
from .spinsys import SimParam, SpinchemError, SysParam

INIT_STATES = {"singlet": 0, "T0": 1, "Tp": 2, "Tm": 3}


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _system_template(sys: SysParam) -> tuple:
    """The field-independent part of an spc_system: (struct, keepalive
    arrays) with nuclei, couplings and rates filled and B = 0."""
    keep = []

    def arr(x, dt):
        a = np.ascontiguousarray(x, dtype=dt)
        if a.size == 0:
            a = np.zeros(1, dtype=dt)
        keep.append(a)
        return a

    s = nat.spc_system()
    s.n_nuc1 = len(sys.e1.g_I)
    s.n_nuc2 = len(sys.e2.g_I)
    m1 = arr(sys.e1.g_I, np.int32)
    m2 = arr(sys.e2.g_I, np.int32)
    # 9 values per nucleus in column-major (input.ini) order
    A1 = arr([a.reshape(3, 3).T.reshape(9) for a in sys.e1.A] or np.zeros(9), np.float64)
    A2 = arr([a.reshape(3, 3).T.reshape(9) for a in sys.e2.A] or np.zeros(9), np.float64)
    s.mult1 = m1.ctypes.data_as(C.POINTER(C.c_int))
    s.mult2 = m2.ctypes.data_as(C.POINTER(C.c_int))
    s.A1 = A1.ctypes.data_as(C.POINTER(C.c_double))
    s.A2 = A2.ctypes.data_as(C.POINTER(C.c_double))
    if sys.e1.gamma_I is not None:
        g1 = arr(sys.e1.gamma_I, np.float64)
        s.gamma1 = g1.ctypes.data_as(C.POINTER(C.c_double))
    if sys.e2.gamma_I is not None:
        g2 = arr(sys.e2.gamma_I, np.float64)
        s.gamma2 = g2.ctypes.data_as(C.POINTER(C.c_double))
    s.J = float(sys.J)
    Dc = np.asarray(sys.D, np.float64).reshape(3, 3).T.reshape(9)
    for i in range(9):
        s.D[i] = float(Dc[i])
    s.kS = float(sys.kS)
    s.kT = float(sys.kT)
    return s, keep


def _with_field(template: tuple, B) -> tuple:
    s0, keep = template
    s = nat.spc_system.from_buffer_copy(s0)
    if np.isscalar(B):
        s.B[0], s.B[1], s.B[2] = 0.0, 0.0, float(B)
    else:
        Bv = np.asarray(B, np.float64).reshape(3)
        s.B[0], s.B[1], s.B[2] = float(Bv[0]), float(Bv[1]), float(Bv[2])
    return s, keep


def make_system(sys: SysParam, B) -> tuple:
    """Fill an spc_system from a SysParam and a field (scalar along z, or a
    3-vector). Returns (struct, keepalive arrays)."""
    return _with_field(_system_template(sys), B)


def make_systems(systems, fields) -> tuple:
    """spc_system array for (system, field) pairs; a system object that
    appears with several fields is converted once. Returns (ctypes array,
    keepalive)."""
    cache, structs, keep = {}, [], []
    for sy, B in zip(systems, fields):
        t = cache.get(id(sy))
        if t is None:
            t = cache[id(sy)] = _system_template(sy)
            keep.append(t)
        structs.append(_with_field(t, B)[0])
    arr = (nat.spc_system * len(structs))(*structs)
    return arr, (keep, systems)


def num_time_points(dt: float, t_end: float) -> int:
    return nat.lib().spc_num_time_points(float(dt), float(t_end))


def init_el_state(which: str):
    """init_el_state (src/qm_dynamics.f90:386-414): (theta[4] complex, init_pop[4])."""
    if which not in INIT_STATES:
        raise SpinchemError("Error: Invalid initial radical pair state entered.")
    th = np.zeros(8)
    pop = np.zeros(4)
    nat.check(nat.lib().spc_init_el_state(INIT_STATES[which], _dptr(th), _dptr(pop)))
    return th.view(np.complex128), pop


def seeded_samples(seed: Sequence[int], Z: int, M: int, serial: bool = False) -> np.ndarray:
    """Sample vectors as the reference draws them (M x Z complex)."""
    out = np.zeros(2 * Z * M)
    s0 = int(seed[0])
    s1 = int(seed[1])
    s0 = s0 - 2**64 if s0 >= 2**63 else s0
    s1 = s1 - 2**64 if s1 >= 2**63 else s1
    nat.check(nat.lib().spc_seeded_samples(s0, s1, Z, M, 1 if serial else 0, _dptr(out)))
    return out.view(np.complex128).reshape(M, Z)


def device_memory(device: int = 0) -> tuple:
    """(free, total) bytes of a CUDA device (spc_mem_info)."""
    f, t = C.c_int64(), C.c_int64()
    nat.check(nat.lib().spc_mem_info(int(device), C.byref(f), C.byref(t)))
    return f.value, t.value


def padded_samples(M: int) -> int:
    """Sample columns a job occupies on the device (tiles of 32)."""
    return (M + 31) // 32 * 32


def batch_groups(entries, budget: float) -> list:
    """Consecutive groups of jobs (given their vector entries, rows x padded
    samples) whose sum stays under `budget` entries; a job larger than the
    budget forms a group of its own."""
    groups, cur, tot = [], [], 0
    for i, x in enumerate(entries):
        if cur and tot + x > budget:
            groups.append(cur)
            cur, tot = [], 0
        cur.append(i)
        tot += x
    if cur:
        groups.append(cur)
    return groups


@dataclass
class YieldGradient:
    """Yields and gradient of spc_yield_gradient. Tensors are (row, col)
    matrices; `raw` is the C layout (column-major tensors)."""
    Phi_S: float
    Phi_T: float
    B: np.ndarray
    J: float
    D: np.ndarray
    kS: float
    kT: float
    A1: list
    A2: list
    raw: np.ndarray

    def symmetric_A(self) -> list:
        """Derivatives with respect to the 6 independent elements (xx, xy, xz,
        yy, yz, zz) of each hyperfine tensor taken as symmetric."""
        out = []
        for a in self.A1 + self.A2:
            out.append(np.array([a[0, 0], a[0, 1] + a[1, 0], a[0, 2] + a[2, 0], a[1, 1],
                                 a[1, 2] + a[2, 1], a[2, 2]]))
        return out

    def axial_D(self) -> float:
        """Derivative with respect to the scalar D of the axial tensor
        2/3 D diag(-1, -1, 2)."""
        return float(np.sum(self.D * (2.0 / 3.0) * np.diag([-1.0, -1.0, 2.0])))

    @staticmethod
    def unpack(y, g, n1: int, n2: int) -> "YieldGradient":
        mat = lambda v: np.asarray(v).reshape(3, 3).T.copy()
        A = [mat(g[15 + 9 * j:24 + 9 * j]) for j in range(n1 + n2)]
        return YieldGradient(float(y[0]), float(y[1]), g[0:3].copy(), float(g[3]), mat(g[4:13]),
                             float(g[13]), float(g[14]), A[:n1], A[n1:], g.copy())


class TraceSampler:
    """One GPU handle: a device Hamiltonian plus the batched propagator."""

    def __init__(self, device: int = 0):
        L = nat.lib()
        h = C.c_void_p()
        nat.check(L.spc_create(int(device), C.byref(h)))
        self._h = h
        self.device = device

    def close(self) -> None:
        if getattr(self, "_h", None):
            nat.lib().spc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_ptr: int) -> None:
        nat.check(nat.lib().spc_set_stream(self._h, C.c_void_p(stream_ptr)))

    def set_graphs(self, enable: bool) -> None:
        """Replay each build round as a captured CUDA graph (default) or
        launch its kernels one by one; results are identical."""
        nat.check(nat.lib().spc_set_graphs(self._h, 1 if enable else 0))

    def set_sample_path(self, mode: str) -> None:
        """Small systems with one CTA per sample ('auto' when it pays, 'off',
        'on' whenever the call fits it, with a cluster of two CTAs per sample
        when the samples fill at most half the SMs; 'single': 'on' with one
        CTA per sample always); results agree to rounding."""
        code = {"auto": nat.SPC_SAMPLE_AUTO, "off": nat.SPC_SAMPLE_OFF, "on": nat.SPC_SAMPLE_ON,
                "single": nat.SPC_SAMPLE_SINGLE}[mode]
        nat.check(nat.lib().spc_set_sample_path(self._h, code))

    def set_memory_limit(self, nbytes: int) -> None:
        """Cap the device memory of one propagation call (0: the device's
        free memory). Samples beyond it run in chunks of 32-sample tiles
        within each build round."""
        nat.check(nat.lib().spc_set_memory_limit(self._h, int(nbytes)))

    def set_krylov(self, method: str) -> None:
        """'mgs' (full modified Gram-Schmidt, the reference's get_krylov),
        'lanczos' (kS == kT only) or 'auto' (Lanczos when it applies)."""
        code = {"mgs": nat.SPC_KRYLOV_MGS, "lanczos": nat.SPC_KRYLOV_LANCZOS,
                "auto": nat.SPC_KRYLOV_AUTO}[method]
        nat.check(nat.lib().spc_set_krylov(self._h, code))

    # ---- Hamiltonian ----
    def build_h(self, sys: SysParam, B, mode: str = "reference") -> tuple:
        """getHiso_sp + coo_to_csr on the device (mode 'reference'), or the
        anisotropic general builder (mode 'general'). Returns (n, nnz)."""
        m = {"reference": nat.SPC_H_REFERENCE, "general": nat.SPC_H_GENERAL}[mode]
        s, keep = make_system(sys, B)
        nat.check(nat.lib().spc_build_h(self._h, C.byref(s), m))
        return self.h_size()

    def set_h(self, rowptr, col, val, index_base: int = 0) -> None:
        rp = np.ascontiguousarray(rowptr, np.int32)
        cl = np.ascontiguousarray(col, np.int32)
        vv = np.ascontiguousarray(np.asarray(val, np.complex128)).view(np.float64)
        csr = nat.spc_csr(len(rp) - 1, len(cl), rp.ctypes.data_as(C.POINTER(C.c_int32)),
                          cl.ctypes.data_as(C.POINTER(C.c_int32)),
                          vv.ctypes.data_as(C.POINTER(C.c_double)), index_base)
        nat.check(nat.lib().spc_set_h(self._h, C.byref(csr)))

    def h_size(self) -> tuple:
        n = C.c_int32()
        nnz = C.c_int64()
        nat.check(nat.lib().spc_h_size(self._h, C.byref(n), C.byref(nnz)))
        return n.value, nnz.value

    def get_h(self):
        n, nnz = self.h_size()
        rp = np.zeros(n + 1, np.int32)
        cl = np.zeros(max(nnz, 1), np.int32)
        vv = np.zeros(2 * max(nnz, 1))
        nat.check(nat.lib().spc_get_h(self._h, _dptr(rp), _dptr(cl), _dptr(vv)))
        return rp, cl[:nnz], vv.view(np.complex128)[:nnz]

    # ---- propagation ----
    def trace_sampling(self, zkets: np.ndarray, dt: float, t_end: float, m: int, tol: float,
                       init_state: str = "singlet") -> Observables:
        """Propagate the M x Z sample vectors (host memory) and return the
        sample-averaged populations."""
        zk = np.ascontiguousarray(np.asarray(zkets, np.complex128))
        if zk.ndim != 2:
            raise ValueError("zkets must be M x Z")
        M = zk.shape[0]
        th, pop = init_el_state(init_state)
        th = np.ascontiguousarray(th).view(np.float64)
        # an invalid dt gives T = -1; the C ABI reports the argument error
        T = max(num_time_points(dt, t_end), 1)
        outs = [np.zeros(T) for _ in range(4)]
        nat.check(nat.lib().spc_trace_sampling(
            self._h, _dptr(th), _dptr(pop), _dptr(zk.view(np.float64)), M, float(dt), float(t_end),
            int(m), float(tol), *(_dptr(o) for o in outs), T))
        return Observables(*outs)

    def trace_sampling_device(self, zkets_ptr: int, M: int, dt: float, t_end: float, m: int,
                              tol: float, out_ptr: int, init_state: str = "singlet") -> None:
        """Same on device-resident buffers: zkets_ptr -> M x Z complex128,
        out_ptr -> 4*T float64 (P_S | P_T0 | P_Tp | P_Tm)."""
        th, pop = init_el_state(init_state)
        th = np.ascontiguousarray(th).view(np.float64)
        T = num_time_points(dt, t_end)
        nat.check(nat.lib().spc_trace_sampling_device(
            self._h, _dptr(th), _dptr(pop), C.c_void_p(zkets_ptr), int(M), float(dt),
            float(t_end), int(m), float(tol), C.c_void_p(out_ptr), T))

    # ---- batches ----
    def build_h_batch(self, systems, fields, mode: str = "reference") -> list:
        """Build one Hamiltonian per (system, field) pair and keep them as
        the handle's batch. Returns the dimensions."""
        m = {"reference": nat.SPC_H_REFERENCE, "general": nat.SPC_H_GENERAL}[mode]
        arr, keep = make_systems(systems, fields)
        nat.check(nat.lib().spc_build_h_batch(self._h, len(arr), C.cast(arr, C.c_void_p), m))
        return [4 * s.Z for s in systems]

    def trace_sampling_batch(self, zkets_list, dt: float, t_end: float, m: int, tol: float,
                             init_state: str = "singlet", job_sys=None) -> list:
        """Propagate job k's M_k x Z_k vectors under batch system job_sys[k]
        (default k) together; returns one Observables per job."""
        M = np.array([z.shape[0] for z in zkets_list], np.int32)
        flat = np.ascontiguousarray(np.concatenate([np.asarray(z, np.complex128).reshape(-1)
                                                    for z in zkets_list]))
        th, pop = init_el_state(init_state)
        th = np.ascontiguousarray(th).view(np.float64)
        T = max(num_time_points(dt, t_end), 1)
        out = np.zeros(len(zkets_list) * 4 * T)
        js = None if job_sys is None else np.ascontiguousarray(job_sys, np.int32)
        nat.check(nat.lib().spc_trace_sampling_batch(
            self._h, len(zkets_list), _dptr(js) if js is not None else None, _dptr(M), _dptr(th),
            _dptr(pop), _dptr(flat.view(np.float64)), float(dt), float(t_end), int(m), float(tol),
            _dptr(out), T))
        out = out.reshape(len(zkets_list), 4, T)
        return [Observables(o[0].copy(), o[1].copy(), o[2].copy(), o[3].copy()) for o in out]

    def trace_sampling_many(self, systems, fields, zkets_list, dt: float, t_end: float, m: int, tol: float,
                            mode: str = "general", init_state: str = "singlet", memory_fraction: float = 0.5,
                            device: int = 0) -> list:
        """Any number of jobs (system, field, samples): split into batches whose
        Krylov bases and states use at most `memory_fraction` of the device's
        free memory, each batch one spc_build_h_batch + spc_trace_sampling_batch
        call. Returns one Observables per job, in job order."""
        free, _ = device_memory(device)
        budget = free * memory_fraction / (16.0 * (m + 4))
        entries = [4 * s.Z * padded_samples(z.shape[0]) for s, z in zip(systems, zkets_list)]
        out = [None] * len(systems)
        for grp in batch_groups(entries, budget):
            self.build_h_batch([systems[i] for i in grp], [fields[i] for i in grp], mode)
            res = self.trace_sampling_batch([zkets_list[i] for i in grp], dt, t_end, m, tol, init_state)
            for i, r in zip(grp, res):
                out[i] = r
        return out

    def trace_sampling_batch_device(self, zk_ptr: int, M, dt: float, t_end: float, m: int,
                                    tol: float, out_ptr: int, init_state: str = "singlet",
                                    job_sys=None) -> None:
        """Device-resident batch: zk_ptr -> the jobs' sample blocks back to
        back, out_ptr -> n_jobs x 4 x T float64."""
        M = np.ascontiguousarray(M, np.int32)
        th, pop = init_el_state(init_state)
        th = np.ascontiguousarray(th).view(np.float64)
        T = num_time_points(dt, t_end)
        js = None if job_sys is None else np.ascontiguousarray(job_sys, np.int32)
        nat.check(nat.lib().spc_trace_sampling_batch_device(
            self._h, len(M), _dptr(js) if js is not None else None, _dptr(M), _dptr(th), _dptr(pop),
            C.c_void_p(zk_ptr), float(dt), float(t_end), int(m), float(tol), C.c_void_p(out_ptr), T))

    def yield_gradient(self, sys: SysParam, B, zkets, dt: float, t_end: float, m: int,
                       n_quad: int = 0, checkpoint_every: int = 0, wS: float = 1.0, wT: float = 0.0,
                       init_state: str = "singlet") -> "YieldGradient":
        """Yields (Phi_S, Phi_T) of the stepwise propagation and the gradient
        of wS*Phi_S + wT*Phi_T with respect to every parameter of the system
        (internal units: mT for B, J, D, A; kS, kT as stored), by the discrete
        adjoint; the general Hamiltonian (anisotropic A, field vector).
        n_quad = 0 takes the Gauss-Legendre node count gradient_nodes gives."""
        st, keep = make_system(sys, B)
        npar = nat.lib().spc_yield_gradient_size(C.byref(st))
        zk = np.ascontiguousarray(zkets, np.complex128)
        th, _ = init_el_state(init_state)
        th = np.ascontiguousarray(th).view(np.float64)
        y = np.zeros(2)
        g = np.zeros(npar)
        nat.check(nat.lib().spc_yield_gradient(
            self._h, C.byref(st), _dptr(th), _dptr(zk.view(np.float64)), zk.shape[0], float(dt),
            float(t_end), int(m), int(n_quad), int(checkpoint_every), float(wS), float(wT), _dptr(y),
            _dptr(g)))
        return YieldGradient.unpack(y, g, len(sys.e1.g_I), len(sys.e2.g_I))

    def yield_gradient_batch(self, systems, fields, zkets_list, dt: float, t_end: float, m: int,
                             n_quad: int = 0, checkpoint_every: int = 0, wS: float = 1.0,
                             wT: float = 0.0, hyperfine: bool = True, init_state: str = "singlet",
                             gradient: bool = True) -> list:
        """spc_yield_gradient_batch: job k = (systems[k], fields[k],
        zkets_list[k]); all jobs share every launch. hyperfine=False computes
        the B, J, D, kS, kT entries only (nuclei up to multiplicity 6).
        gradient=False returns the yields only. Returns one YieldGradient per
        job."""
        arr, keep = make_systems(systems, fields)
        structs = list(arr)
        sizes = [15 + 9 * (len(s.e1.g_I) + len(s.e2.g_I)) for s in systems]
        M = np.array([z.shape[0] for z in zkets_list], np.int32)
        flat = np.ascontiguousarray(np.concatenate([np.asarray(z, np.complex128).reshape(-1)
                                                    for z in zkets_list]))
        th, _ = init_el_state(init_state)
        th = np.ascontiguousarray(th).view(np.float64)
        y = np.zeros(2 * len(structs))
        g = np.zeros(int(sum(sizes)))
        which = nat.SPC_GRAD_ALL if hyperfine else nat.SPC_GRAD_FIELD
        nat.check(nat.lib().spc_yield_gradient_batch(
            self._h, len(structs), C.cast(arr, C.c_void_p), _dptr(M), _dptr(th),
            _dptr(flat.view(np.float64)), float(dt), float(t_end), int(m), int(n_quad),
            int(checkpoint_every), float(wS), float(wT), which, _dptr(y),
            _dptr(g) if gradient else None))
        out, off = [], 0
        for k, s in enumerate(systems):
            out.append(YieldGradient.unpack(y[2 * k:2 * k + 2], g[off:off + sizes[k]], len(s.e1.g_I),
                                            len(s.e2.g_I)))
            off += sizes[k]
        return out

    def stepwise_yields(self, sys: SysParam, B, zkets, dt: float, t_end: float, m: int,
                        init_state: str = "singlet") -> tuple:
        """(Phi_S, Phi_T) of the stepwise propagation spc_yield_gradient
        differentiates: its forward sweep alone."""
        st, keep = make_system(sys, B)
        zk = np.ascontiguousarray(zkets, np.complex128)
        th, _ = init_el_state(init_state)
        th = np.ascontiguousarray(th).view(np.float64)
        y = np.zeros(2)
        nat.check(nat.lib().spc_yield_gradient(
            self._h, C.byref(st), _dptr(th), _dptr(zk.view(np.float64)), zk.shape[0], float(dt),
            float(t_end), int(m), 1, 0, 1.0, 0.0, _dptr(y), None))
        return float(y[0]), float(y[1])

    def autotune_krylov(self, zkets_list, dt: float, t_window: float, tol: float,
                        candidates=(12, 16, 20, 24, 30, 40), init_state: str = "singlet",
                        job_sys=None) -> tuple:
        """spc_autotune_krylov over the batch store: the Krylov dimension with
        the most sample-steps/s on one tile of every job. Returns (best_m,
        {m: rate})."""
        M = np.array([z.shape[0] for z in zkets_list], np.int32)
        flat = np.ascontiguousarray(np.concatenate([np.asarray(z, np.complex128).reshape(-1)
                                                    for z in zkets_list]))
        th, pop = init_el_state(init_state)
        th = np.ascontiguousarray(th).view(np.float64)
        cand = np.ascontiguousarray(candidates, np.int32)
        rates = np.zeros(cand.size)
        best = C.c_int(0)
        js = None if job_sys is None else np.ascontiguousarray(job_sys, np.int32)
        nat.check(nat.lib().spc_autotune_krylov(
            self._h, len(zkets_list), _dptr(js) if js is not None else None, _dptr(M), _dptr(th), _dptr(pop),
            _dptr(flat.view(np.float64)), float(dt), float(t_window), float(tol), _dptr(cand), int(cand.size),
            C.byref(best), _dptr(rates)))
        return int(best.value), {int(m): float(r) for m, r in zip(cand, rates)}

    def stats(self) -> dict:
        s = nat.spc_stats()
        nat.check(nat.lib().spc_get_stats(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in nat.spc_stats._fields_}


def gradient_nodes(sys: SysParam, B, dt: float) -> int:
    """Gauss-Legendre nodes per step the yield gradient takes with n_quad = 0
    (spc_gradient_nodes: the smallest count whose remainder bound at the
    norm bound of H_eff is below 1e-8). Host only."""
    st, keep = make_system(sys, B)
    n = C.c_int()
    nat.check(nat.lib().spc_gradient_nodes(C.byref(st), float(dt), C.byref(n)))
    return n.value


# ---------------------------------------------------------------------------
# reference-named drivers
_DEFAULT: Optional[TraceSampler] = None


def default_sampler() -> TraceSampler:
    global _DEFAULT
    if _DEFAULT is None:
        _DEFAULT = TraceSampler(0)
    return _DEFAULT


def _field(sys: SysParam) -> float:
    # main sets sys%e1%w = sys%e2%w = -B (app/main.f90:53-54)
    return -float(sys.e1.w)


def _require_isotropic(sys: SysParam) -> None:
    if not (sys.e1.isotropic and sys.e2.isotropic):
        raise SpinchemError("Anisotropic Hamiltoninans have not been implemented yet")


def trace_sampling_para(sys: SysParam, sim: SimParam, out: Optional[str] = None,
                        sampler: Optional[TraceSampler] = None) -> Observables:
    """trace_sampling_para (src/qm_dynamics.f90:257-384): H from getHiso_sp on
    the device, per-sample seeds drawn from sim.seed, the batched Krylov
    propagation, the sample average; writes the output files when `out` is
    given (without yields, as the reference)."""
    _require_isotropic(sys)
    sp = sampler or default_sampler()
    sp.build_h(sys, _field(sys), "reference")
    zk = seeded_samples(sim.seed, sys.Z, sim.N_samples)
    res = sp.trace_sampling(zk, sim.dt, sim.t_end, sim.N_krylov, sim.tol, sim.init_state)
    if out is not None:
        res.output(out)
    return res


def trace_sampling(sys: SysParam, sim: SimParam, out: Optional[str] = None,
                   sampler: Optional[TraceSampler] = None) -> Observables:
    """trace_sampling (serial variant, src/qm_dynamics.f90:139-255): one RNG
    stream across samples; propagation as trace_sampling_para."""
    _require_isotropic(sys)
    sp = sampler or default_sampler()
    sp.build_h(sys, _field(sys), "reference")
    zk = seeded_samples(sim.seed, sys.Z, sim.N_samples, serial=True)
    res = sp.trace_sampling(zk, sim.dt, sim.t_end, sim.N_krylov, sim.tol, sim.init_state)
    if out is not None:
        res.output(out)
    return res


def field_dynamics(sys: SysParam, sim: SimParam, folders=None,
                   sampler: Optional[TraceSampler] = None) -> list:
    """The field loop of app/main.f90:48-79 for trace_sampling (parallel and
    serial) and exact_dynamics, every field value of sim.B together: main
    re-seeds the generator with sim.seed before each field (app/main.f90:50),
    so every field propagates the same vectors. Each field's Hamiltonian
    (getHiso_sp with w = -B) is one system of the batch store; groups of
    fields bounded by device memory (a third of the free memory at m + 4
    states per vector entry) share one build and one propagation. Writes
    field k's files into folders[k] when given; returns one Observables per
    field."""
    _require_isotropic(sys)
    sp = sampler or default_sampler()
    if sim.type == "exact_dynamics":
        zk = np.eye(sys.Z, dtype=np.complex128)
    else:
        zk = seeded_samples(sim.seed, sys.Z, sim.N_samples, serial=sim.type == "trace_sampling_serial")
    free, _ = device_memory()
    budget = max(1.0, free / 3.0 / (16.0 * (sim.N_krylov + 4)))
    res = [None] * len(sim.B)
    for grp in batch_groups([4 * sys.Z * padded_samples(zk.shape[0])] * len(sim.B), budget):
        sp.build_h_batch([sys] * len(grp), [sim.B[k] for k in grp], "reference")
        for k, r in zip(grp, sp.trace_sampling_batch([zk] * len(grp), sim.dt, sim.t_end, sim.N_krylov, sim.tol,
                                                     sim.init_state)):
            res[k] = r
    if folders is not None:
        for r, f in zip(res, folders):
            r.output(f)
    return res


def exact_dynamics(sys: SysParam, sim: SimParam, out: Optional[str] = None,
                   sampler: Optional[TraceSampler] = None) -> Observables:
    """exact_dynamics (src/qm_dynamics.f90:24-137): the same propagator over
    all Z nuclear basis states, averaged with weight 1/Z."""
    _require_isotropic(sys)
    sp = sampler or default_sampler()
    sp.build_h(sys, _field(sys), "reference")
    zk = np.eye(sys.Z, dtype=np.complex128)
    res = sp.trace_sampling(zk, sim.dt, sim.t_end, sim.N_krylov, sim.tol, sim.init_state)
    if out is not None:
        res.output(out)
    return res
