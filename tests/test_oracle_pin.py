"""Pins the CPU oracle (C++ restatement of the reference) without the
reference itself: against an independently assembled dense Hamiltonian with
exact eigendecomposition propagation, analytic known answers, SciPy's expm,
and an independent pure-Python xoroshiro128+."""
import numpy as np
import pytest
import scipy.linalg as sl
import scipy.sparse as sp

import dense
from conftest import general_csr, iso_csr
from spin_dynamics_gb300 import workloads as W
from spin_dynamics_gb300.spinsys import GAMMA_E, Electron, SysParam

DT = 0.5 * GAMMA_E / 1000


def to_dense(rp, col, val):
    n = len(rp) - 1
    return sp.csr_matrix((val, col, rp), shape=(n, n)).toarray()


def dense_of(sysp, B):
    Bv = [0.0, 0.0, B] if np.isscalar(B) else B
    return dense.hamiltonian(sysp.e1.g_I, sysp.e1.A, sysp.e2.g_I, sysp.e2.A, Bv, sysp.J, sysp.D,
                             sysp.kS, sysp.kT, sysp.e1.gammas, sysp.e2.gammas)


# ------------------------------------------------------------------ Hamiltonian
@pytest.mark.parametrize("which", ["notebook", "small", "small_rates"])
def test_reference_hamiltonian_equals_dense(oracle, which):
    sysp = {"notebook": W.notebook_pair, "small": W.small_pair, "small_rates": W.small_pair}[which]()
    if which == "small_rates":
        sysp.kS, sysp.kT = 20.0 / GAMMA_E, 5.0 / GAMMA_E
        sysp.J = 0.07
        sysp.D = W.axial_dipolar(-0.3)
    H = to_dense(*iso_csr(oracle, sysp, 0.31))
    assert np.max(np.abs(H - dense_of(sysp, 0.31))) < 1e-14


def test_reference_nonzero_count_and_row_order(oracle):
    sysp = W.small_pair()
    rp, col, val = iso_csr(oracle, sysp, 0.05)
    N = sysp.N
    g = sysp.e1.g_I + sysp.e2.g_I
    assert rp[-1] == N + N // 2 + sum((k - 1) * (N // k) for k in g)  # src/hamiltonian.f90:62-73
    # coo_to_csr puts each row's COO entries in reverse order
    e1, e2 = sysp.e1, sysp.e2
    r, c, v = oracle.build_h_iso_coo(e1.g_I, e1.a_iso, e2.g_I, e2.a_iso, 0.05, sysp.J, sysp.D,
                                     sysp.kS, sysp.kT)
    for row in (0, 5, 77, N - 1):
        coo_cols = [cc - 1 for rr, cc in zip(r, c) if rr - 1 == row]
        assert list(col[rp[row]:rp[row + 1]]) == coo_cols[::-1]


def test_general_hamiltonian_equals_dense_anisotropic(oracle):
    rng = np.random.default_rng(3)
    sysp = W.small_pair()
    for e in (sysp.e1, sysp.e2):
        e.A = [(lambda R: R @ np.diag(rng.uniform(-2, 2, 3)) @ R.T)(W._haar_rotation(rng)) for _ in e.A]
    sysp.D = np.array([[0.1, 0.02, -0.03], [0.02, 0.15, 0.01], [-0.03, 0.01, -0.25]])
    sysp.J = 0.03
    sysp.kS, sysp.kT = 3.0 / GAMMA_E, 1.0 / GAMMA_E
    B = np.array([0.02, -0.04, 0.03])
    H = to_dense(*general_csr(oracle, sysp, B))
    assert np.max(np.abs(H - dense_of(sysp, B))) < 1e-14


def test_general_reduces_to_reference_for_isotropic_z_field(oracle):
    sysp = W.small_pair()
    Hr = to_dense(*iso_csr(oracle, sysp, 0.2))
    Hg = to_dense(*general_csr(oracle, sysp, [0.0, 0.0, 0.2]))
    assert np.max(np.abs(Hr - Hg)) < 1e-15


def test_reference_builder_refuses_what_the_reference_refuses(oracle):
    sysp = W.small_pair()
    with pytest.raises(ValueError):
        oracle.build_h_iso([4], [0.1], [2], [0.2], 0.0, 0.0, np.zeros((3, 3)), 0, 0)  # mult 4
    with pytest.raises(ValueError):
        oracle.build_h_iso([2], [0.1], [2], [0.2], 0.0, 0.0, np.diag([0.1, 0.2, 0.3]), 0, 0)


# ------------------------------------------------------------------ expm
@pytest.mark.parametrize("scale", [0.0, 1e-3, 0.3, 1.0, 7.5, 60.0])
def test_expm_matches_scipy(oracle, scale):
    rng = np.random.default_rng(int(scale * 10) + 1)
    A = (rng.normal(size=(12, 12)) + 1j * rng.normal(size=(12, 12))) * scale / 12
    E = oracle.expm(A)
    ref = sl.expm(A)
    assert np.max(np.abs(E - ref)) <= 1e-13 * max(1.0, np.max(np.abs(ref)))


# ------------------------------------------------------------------ propagation
def test_exact_dynamics_matches_dense_at_full_krylov(oracle):
    """With m large enough to span each orbit the Krylov propagator is exact."""
    sysp = W.notebook_pair()
    rp, col, val = iso_csr(oracle, sysp, 0.2)
    zk = np.eye(sysp.Z, dtype=complex)
    t_end = 40 * DT
    r = oracle.trace_sampling(rp, col, val, zk, DT, t_end, 30, 1e-30)
    n = int(np.ceil(t_end / DT)) + 1
    times = np.arange(n) * DT
    PS, PT0, PTp, PTm = dense.trace_sampled_populations(dense_of(sysp, 0.2), zk, times)
    for got, ref in ((r["P_S"], PS), (r["P_T0"], PT0), (r["P_Tp"], PTp), (r["P_Tm"], PTm)):
        assert np.max(np.abs(got[:n] - ref)) < 1e-11


def test_krylov_truncation_error_bounded_by_tolerance(oracle):
    sysp = W.small_pair()
    sysp.kS = sysp.kT = 2.0 / GAMMA_E
    rp, col, val = iso_csr(oracle, sysp, 0.05)
    zk = W.random_phase_samples(sysp.Z, 6, seed=9)
    dt = 1.0 * GAMMA_E / 1000
    t_end = 200 * dt
    n = int(np.ceil(t_end / dt)) + 1
    PS = dense.trace_sampled_populations(dense_of(sysp, 0.05), zk, np.arange(n) * dt)[0]
    errs = []
    for tol in (1e-8, 1e-12, 1e-16):
        r = oracle.trace_sampling(rp, col, val, zk, dt, t_end, 20, tol)
        errs.append(np.max(np.abs(r["P_S"][:n] - PS)))
        # the rebuild test |c_m|^2 <= tol |c|^2 keeps the error near sqrt(tol)
        assert errs[-1] < 10 * np.sqrt(tol) + 1e-12
    assert errs[0] > errs[1] > errs[2]


def test_one_proton_closed_form(oracle):
    """One spin-1/2 nucleus (a) on radical 1, J = 0, B = 0, no recombination:
    P_S(t) = 5/8 + 3/8 cos(a t) averaged over the nuclear states."""
    a = 0.8
    sysp = SysParam(e1=Electron(g_I=[2], A=[np.eye(3) * a]), e2=Electron(g_I=[], A=[]))
    rp, col, val = iso_csr(oracle, sysp, 0.0)
    zk = np.eye(2, dtype=complex)
    t_end = 60 * DT
    # each nuclear basis state's orbit is 3-dimensional (Mz conservation);
    # m = 3 spans it (at m = 8 the reference's Arnoldi divides by a zero norm)
    r = oracle.trace_sampling(rp, col, val, zk, DT, t_end, 3, 1e-14)
    n = int(np.ceil(t_end / DT)) + 1
    t = np.arange(n) * DT
    assert np.max(np.abs(r["P_S"][:n] - (5 / 8 + 3 / 8 * np.cos(a * t)))) < 1e-12


def test_recombination_only_decay_and_trace(oracle):
    """No couplings: P_S = exp(-k t); with kS = kT the total population decays
    as exp(-k t) for any coupling set."""
    k = 3.0 / GAMMA_E
    bare = SysParam(e1=Electron(g_I=[2], A=[np.zeros((3, 3))]), e2=Electron(g_I=[3], A=[np.zeros((3, 3))]),
                    kS=k, kT=k)
    rp, col, val = iso_csr(oracle, bare, 0.0)
    zk = W.random_phase_samples(bare.Z, 3)
    t_end = 50 * DT
    # psi is an eigenvector: m = 1 is exact (a larger m breaks down at a zero norm)
    r = oracle.trace_sampling(rp, col, val, zk, DT, t_end, 1, 1e-12)
    n = int(np.ceil(t_end / DT)) + 1
    t = np.arange(n) * DT
    assert np.max(np.abs(r["P_S"][:n] - np.exp(-k * t))) < 1e-12
    sysp = W.small_pair()
    rp, col, val = iso_csr(oracle, sysp, 0.0)
    zk = np.eye(sysp.Z, dtype=complex)  # the exact trace: T+/T- symmetric at B = 0
    r = oracle.trace_sampling(rp, col, val, zk, DT, t_end, 20, 1e-12)
    tot = r["P_S"] + r["P_T0"] + r["P_Tp"] + r["P_Tm"]
    assert np.max(np.abs(tot[:n] - np.exp(-sysp.kS * t))) < 1e-9
    # T+ and T- populations coincide at zero field
    assert np.max(np.abs(r["P_Tp"][:n] - r["P_Tm"][:n])) < 1e-9


def test_time_grid_and_trailing_zeros(oracle):
    """t += dt accumulation and N_steps + 1 slots (src/qm_dynamics.f90:305,362)."""
    sysp = W.small_pair()
    rp, col, val = iso_csr(oracle, sysp, 0.05)
    dt = 0.17608596
    t_end = 880.4298
    assert oracle.num_time_points(dt, t_end) == int(np.ceil((t_end + dt) / dt)) + 1
    zk = W.random_phase_samples(sysp.Z, 2)
    r = oracle.trace_sampling(rp, col, val, zk, dt, 20 * dt, 10, 1e-5)
    t, n = 0.0, 0
    while t < 20 * dt:
        t += dt
        n += 1
    assert np.all(r["P_S"][1:n + 1] != 0.0) and np.all(r["P_S"][n + 1:] == 0.0)


# ------------------------------------------------------------------ RNG
MASK = (1 << 64) - 1


def py_next(s):
    s0, s1 = s
    res = (s0 + s1) & MASK
    s1 ^= s0
    rotl = lambda x, k: ((x << k) | (x >> (64 - k))) & MASK
    return res, [rotl(s0, 55) ^ s1 ^ ((s1 << 14) & MASK), rotl(s1, 36)]


def py_jump(s):
    J = [(-4707382666127344949) & MASK, (-2852180941702784734) & MASK]
    t = [0, 0]
    for j in J:
        for b in range(64):
            if j >> b & 1:
                t = [t[0] ^ s[0], t[1] ^ s[1]]
            _, s = py_next(s)
    return t


def test_xoroshiro_and_jump_match_independent_python(oracle):
    seed = [42, 99]
    s = py_jump(list(seed))
    want = []
    for _ in range(10):
        v, s = py_next(s)
        want.append(v)
    assert list(oracle.rng_stream(seed, 10)) == want
    s = list(seed)
    want = []
    for _ in range(5):
        v, s = py_next(s)
        want.append(v)
    assert list(oracle.rng_stream(seed, 5, do_seed=False)) == want


def test_normals_and_samples(oracle):
    x = oracle.rng_normals((7, 11), 200000)
    assert abs(x.mean()) < 0.01 and abs(x.var() - 1.0) < 0.01
    z = oracle.seeded_samples((42, 99), 50, 20)
    assert np.allclose(np.linalg.norm(z, axis=1), 1.0, atol=1e-14)
    assert not np.allclose(z[0], z[1])
    # mode 1 continues one stream: its first sample equals the first sample
    # drawn from the master generator directly
    assert not np.allclose(oracle.seeded_samples((42, 99), 50, 2, mode=1)[0], z[0])
