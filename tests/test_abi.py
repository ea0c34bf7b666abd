"""The C ABI without a GPU: the library builds, loads, exports every symbol the
header declares, and its host-side helpers agree with the oracle."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT, gpu_available
from spin_dynamics_gb300 import _native as nat
from spin_dynamics_gb300.dynamics import init_el_state, num_time_points, seeded_samples

HEADER = os.path.join(ROOT, "include", "spinchem_gpu.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(spc_\w+)\s*\(", src, flags=re.M)))


def test_header_declares_expected_entry_points():
    names = declared_functions()
    for n in ("spc_create", "spc_destroy", "spc_build_h", "spc_set_h", "spc_get_h",
              "spc_trace_sampling", "spc_trace_sampling_device", "spc_seeded_samples",
              "spc_kinetics", "spc_last_error"):
        assert n in names


def test_header_constants_match_the_binding():
    """Every #define SPC_* of the header has the same value in _native."""
    defs = dict(re.findall(r"^#define (SPC_\w+) (\d+)", open(HEADER).read(), flags=re.M))
    assert "SPC_SAMPLE_SINGLE" in defs
    for name, value in defs.items():
        if hasattr(nat, name):
            assert getattr(nat, name) == int(value), name
    for name in ("SPC_SAMPLE_AUTO", "SPC_SAMPLE_OFF", "SPC_SAMPLE_ON", "SPC_SAMPLE_SINGLE",
                 "SPC_KRYLOV_MGS", "SPC_KRYLOV_LANCZOS", "SPC_KRYLOV_AUTO"):
        assert getattr(nat, name) == int(defs[name]), name


def test_library_exports_every_declared_symbol():
    L = nat.lib()
    for name in declared_functions():
        assert hasattr(L, name), f"{name} declared in spinchem_gpu.h but not exported"
        assert name in nat.SIGNATURES, f"{name} has no ctypes signature"


def test_create_without_gpu_fails_cleanly():
    if gpu_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    rc = nat.lib().spc_create(0, C.byref(h))
    assert rc == nat.SPC_ERR_CUDA
    assert b"CUDA" in nat.lib().spc_last_error()


@pytest.mark.parametrize("seed,serial", [((42, 99), False), ((1436699015287340820, 6992165104747523623), False),
                                         ((42, 99), True), ((-5, 2**63 + 7), False)])
def test_seeded_samples_match_oracle_bitwise(oracle, seed, serial):
    a = seeded_samples(seed, 72, 9, serial=serial)
    b = oracle.seeded_samples(seed, 72, 9, mode=1 if serial else 0)
    assert np.array_equal(a, b)
    assert np.allclose(np.linalg.norm(a, axis=1), 1.0, atol=1e-14)


def test_kinetics_matches_oracle(oracle):
    rng = np.random.default_rng(0)
    T = 101
    P = [rng.random(T) for _ in range(4)]
    ph, pt, iden = oracle.kinetics(*P, 0.176, 0.0056, 0.0011)
    out = [np.zeros(T // 2), np.zeros(T // 2), np.zeros(T)]
    ptr = lambda a: a.ctypes.data_as(C.c_void_p)
    nat.check(nat.lib().spc_kinetics(T, *(ptr(np.ascontiguousarray(x)) for x in P), 0.176, 0.0056,
                                     0.0011, *(ptr(o) for o in out)))
    assert np.array_equal(out[0], ph) and np.array_equal(out[1], pt) and np.array_equal(out[2], iden)


def test_time_points_and_initial_states(oracle):
    for dt, te in ((0.17608596, 880.4298), (0.08804298, 17.5), (1.0, 0.0), (0.3, 0.29999)):
        assert num_time_points(dt, te) == oracle.num_time_points(dt, te)
    for s in ("singlet", "T0", "Tp", "Tm"):
        th, pop = init_el_state(s)
        th2, pop2 = oracle.init_el_state(s)
        assert np.array_equal(th, th2) and np.array_equal(pop, pop2)
    assert nat.lib().spc_num_time_points(0.0, 1.0) == -1


def test_yield_gradient_size_is_host_only():
    from spin_dynamics_gb300 import workloads as W
    from spin_dynamics_gb300.dynamics import make_system
    s = W.small_pair()
    st, keep = make_system(s, 0.05)
    assert nat.lib().spc_yield_gradient_size(C.byref(st)) == 15 + 9 * 5
    assert nat.lib().spc_yield_gradient_size(None) == -1


def _gl_integral(H, lam, V, psi, dt, n):
    """n-node Gauss-Legendre value of int_0^dt <exp(iH^H(dt-s)) lam| V |exp(-iHs) psi> ds."""
    from scipy.linalg import expm
    x, w = np.polynomial.legendre.leggauss(n)
    s = 0.5 * dt * (x + 1.0)
    tot = 0.0j
    for sk, wk in zip(s, w):
        u = expm(1j * H.conj().T * (dt - sk)) @ lam
        v = expm(-1j * H * sk) @ psi
        tot += 0.5 * dt * wk * np.vdot(u, V @ v)
    return tot


@pytest.mark.parametrize("scale,dt", [(1.0, 0.17608596), (3.0, 0.17608596), (0.2, 0.5)])
def test_gradient_node_rule_bounds_the_quadrature_error(scale, dt):
    """spc_gradient_nodes (the count n_quad = 0 takes): its norm bound is at
    least ||H_eff||_2, and n nodes integrate the derivative integrand of a
    step to 1e-8 of the integrand's scale (a 20-node rule as reference)."""
    import dense
    from spin_dynamics_gb300 import workloads as W
    from spin_dynamics_gb300.dynamics import gradient_nodes
    s = W.notebook_pair()
    rng = np.random.default_rng(3)
    s.e1.A = [scale * (a + 0.3 * rng.standard_normal((3, 3))) for a in s.e1.A]
    s.e2.A = [scale * (a + 0.3 * rng.standard_normal((3, 3))) for a in s.e2.A]
    s.e1.A = [0.5 * (a + a.T) for a in s.e1.A]
    s.e2.A = [0.5 * (a + a.T) for a in s.e2.A]
    s.kS, s.kT = 0.011, 0.004
    B = np.array([0.03, -0.02, 0.05])
    n = gradient_nodes(s, B, dt)
    assert 1 <= n <= 16
    H = dense.hamiltonian(s.e1.g_I, s.e1.A, s.e2.g_I, s.e2.A, B, s.J, s.D, s.kS, s.kT,
                          s.e1.gammas, s.e2.gammas)
    psi = rng.standard_normal(H.shape[0]) + 1j * rng.standard_normal(H.shape[0])
    lam = rng.standard_normal(H.shape[0]) + 1j * rng.standard_normal(H.shape[0])
    psi /= np.linalg.norm(psi)
    lam /= np.linalg.norm(lam)
    V = dense.hamiltonian(s.e1.g_I, s.e1.A, s.e2.g_I, s.e2.A, B + [1e-3, 0, 0], s.J, s.D, s.kS, s.kT,
                          s.e1.gammas, s.e2.gammas) - H  # a field-derivative direction
    V /= np.linalg.norm(V, 2)
    ref = _gl_integral(H, lam, V, psi, dt, 20)
    got = _gl_integral(H, lam, V, psi, dt, n)
    assert abs(got - ref) <= 1e-8 * dt
    if n > 1:  # one node fewer is not always enough for the bound: the rule is not over-generous
        assert abs(_gl_integral(H, lam, V, psi, dt, n - 1) - ref) <= 1.0 * dt
