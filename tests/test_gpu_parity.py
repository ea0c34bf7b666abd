"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

Tolerance: the singlet yield must agree to |delta Phi_S| <= 1e-10 absolute. Every
population array and the Simpson yields are held to ABS_TOL = 1e-10; the
Hamiltonian assembly (integer structure and the values, which are rounded at
the same points on both sides) must be bit-exact.
"""
import numpy as np
import pytest

from conftest import general_csr, iso_csr
from spin_dynamics_gb300 import workloads as W
from spin_dynamics_gb300._native import SpcError
from spin_dynamics_gb300.spinsys import GAMMA_E

ABS_TOL = 1e-10
pytestmark = pytest.mark.gpu


def _compare(res_gpu, res_orc, dt, kS, kT, oracle, tol=ABS_TOL):
    for key, gk in (("P_S", "P_S"), ("P_T0", "P_T0"), ("P_Tp", "P_Tp"), ("P_Tm", "P_Tm")):
        g = getattr(res_gpu, gk)
        o = res_orc[key]
        assert g.shape == o.shape
        err = np.max(np.abs(g - o))
        assert err <= tol, f"{key}: max |gpu - oracle| = {err:.3e}"
    phi_g, _, _ = oracle.kinetics(res_gpu.P_S, res_gpu.P_T0, res_gpu.P_Tp, res_gpu.P_Tm, dt, kS, kT)
    phi_o, _, _ = oracle.kinetics(res_orc["P_S"], res_orc["P_T0"], res_orc["P_Tp"], res_orc["P_Tm"],
                                  dt, kS, kT)
    assert np.max(np.abs(phi_g - phi_o)) <= tol


# ---------------------------------------------------------------- Hamiltonian
@pytest.mark.parametrize("which", ["notebook", "small", "large_iso"])
def test_reference_hamiltonian_bit_exact(sampler, oracle, which):
    if which == "notebook":
        sysp, Bz = W.notebook_pair(), 0.2
    elif which == "small":
        sysp, Bz = W.small_pair(), 0.05
    else:
        sysp, B = W.large_pair(isotropic=True)
        Bz = B[2]
    rp_o, col_o, val_o = iso_csr(oracle, sysp, Bz)
    sampler.build_h(sysp, Bz, "reference")
    rp, col, val = sampler.get_h()
    assert np.array_equal(rp, rp_o)
    assert np.array_equal(col, col_o)
    assert np.array_equal(val, val_o)


@pytest.mark.parametrize("which", ["small_aniso", "large_aniso"])
def test_general_hamiltonian_bit_exact(sampler, oracle, which):
    if which == "small_aniso":
        rng = np.random.default_rng(5)
        sysp = W.small_pair()
        for e in (sysp.e1, sysp.e2):
            e.A = [a + (lambda r: r + r.T)(rng.normal(size=(3, 3)) * 0.3) for a in e.A]
        sysp.D = W.axial_dipolar(-0.4) + np.diag([0.05, -0.02, -0.03])
        sysp.J = 0.02
        B = np.array([0.03, -0.02, 0.04])
    else:
        sysp, B = W.large_pair()
    rp_o, col_o, val_o = general_csr(oracle, sysp, B)
    sampler.build_h(sysp, B, "general")
    rp, col, val = sampler.get_h()
    assert np.array_equal(rp, rp_o)
    assert np.array_equal(col, col_o)
    assert np.array_equal(val, val_o)


def test_reference_mode_refuses_what_the_reference_refuses(sampler):
    sysp, B = W.large_pair()  # anisotropic tensors
    with pytest.raises(SpcError) as ei:
        sampler.build_h(sysp, 0.05, "reference")
    assert "Anisotropic" in str(ei.value)
    s2 = W.small_pair()
    s2.D = np.diag([0.1, 0.2, -0.3])
    with pytest.raises(SpcError) as ei:
        sampler.build_h(s2, 0.05, "reference")
    assert "D(1,1) must equal sys%D(2,2)" in str(ei.value)
    with pytest.raises(SpcError):
        sampler.build_h(W.small_pair(), [0.01, 0.0, 0.05], "reference")


# ---------------------------------------------------------------- propagation
def test_notebook_exact_dynamics(sampler, oracle):
    """exact_dynamics on the 48-dim example system: all Z basis states."""
    sysp = W.notebook_pair()
    rp, col, val = iso_csr(oracle, sysp, 0.2)
    dt = 0.5 * GAMMA_E / 1000
    t_end = 99.5 * GAMMA_E / 1000
    zk = np.eye(sysp.Z, dtype=complex)
    ref = oracle.trace_sampling(rp, col, val, zk, dt, t_end, 10, 1e-8)
    sampler.build_h(sysp, 0.2, "reference")
    got = sampler.trace_sampling(zk, dt, t_end, 10, 1e-8)
    _compare(got, ref, dt, sysp.kS, sysp.kT, oracle)


def test_small_pair_full_length(sampler, oracle):
    """Plain small pair (dim 288): 64 random-phase samples, 5 us at 1 ns, m = 20."""
    sysp, sim = W.small_pair(), W.small_sim()
    rp, col, val = iso_csr(oracle, sysp, 0.05)
    zk = W.random_phase_samples(sysp.Z, 64)
    ref = oracle.trace_sampling(rp, col, val, zk, sim.dt, sim.t_end, sim.N_krylov, sim.tol)
    sampler.build_h(sysp, 0.05, "reference")
    got = sampler.trace_sampling(zk, sim.dt, sim.t_end, sim.N_krylov, sim.tol)
    _compare(got, ref, sim.dt, sysp.kS, sysp.kT, oracle)
    st = sampler.stats()
    assert st["krylov_builds"] == int(ref["n_builds"].sum())


def test_reference_sample_stream(sampler, oracle):
    """The reference's own sample_SUZ stream (seed 42 99) through the C ABI."""
    from spin_dynamics_gb300.dynamics import seeded_samples
    sysp, sim = W.small_pair(), W.small_sim(M=16, t_end_ns=400.0)
    zk = seeded_samples(sim.seed, sysp.Z, 16)
    assert np.array_equal(zk, oracle.seeded_samples(sim.seed, sysp.Z, 16))
    rp, col, val = iso_csr(oracle, sysp, 0.05)
    ref = oracle.trace_sampling(rp, col, val, zk, sim.dt, sim.t_end, sim.N_krylov, sim.tol)
    sampler.build_h(sysp, 0.05, "reference")
    got = sampler.trace_sampling(zk, sim.dt, sim.t_end, sim.N_krylov, sim.tol)
    _compare(got, ref, sim.dt, sysp.kS, sysp.kT, oracle)


def test_large_pair_isotropic_subset(sampler, oracle):
    """Dim 55296, the subset the reference accepts (isotropic, B along z)."""
    sysp, B = W.large_pair(isotropic=True)
    sim = W.large_sim(M=8, t_end_ns=60.0)
    rp, col, val = iso_csr(oracle, sysp, B[2])
    zk = W.random_phase_samples(sysp.Z, 8, seed=3)
    ref = oracle.trace_sampling(rp, col, val, zk, sim.dt, sim.t_end, sim.N_krylov, sim.tol)
    sampler.build_h(sysp, B[2], "reference")
    got = sampler.trace_sampling(zk, sim.dt, sim.t_end, sim.N_krylov, sim.tol)
    _compare(got, ref, sim.dt, sysp.kS, sysp.kT, oracle)


def test_large_pair_anisotropic(sampler, oracle):
    """Dim 55296, anisotropic tensors, tilted field, axial D (general builder)."""
    sysp, B = W.large_pair()
    sim = W.large_sim(M=4, t_end_ns=40.0)
    rp, col, val = general_csr(oracle, sysp, B)
    zk = W.random_phase_samples(sysp.Z, 4, seed=4)
    ref = oracle.trace_sampling(rp, col, val, zk, sim.dt, sim.t_end, sim.N_krylov, sim.tol)
    sampler.build_h(sysp, B, "general")
    got = sampler.trace_sampling(zk, sim.dt, sim.t_end, sim.N_krylov, sim.tol)
    _compare(got, ref, sim.dt, sysp.kS, sysp.kT, oracle)


@pytest.mark.parametrize("m", [47, 48])
@pytest.mark.parametrize("method", ["mgs", "lanczos"])
def test_largest_krylov_dimensions(sampler, oracle, m, method):
    """The largest accepted Krylov dimensions (the largest expm and projector
    shared-memory footprints, an odd size) at dim 55296 with anisotropic
    couplings and at dim 288, both orthogonalisations."""
    sampler.set_krylov(method)
    try:
        sysp, B = W.large_pair()
        rp, col, val = general_csr(oracle, sysp, B)
        zk = W.random_phase_samples(sysp.Z, 3, seed=m)
        dt, t_end = 0.17608596, 60 * 0.17608596
        ref = oracle.trace_sampling(rp, col, val, zk, dt, t_end, m, 1e-7)
        sampler.build_h(sysp, B, "general")
        got = sampler.trace_sampling(zk, dt, t_end, m, 1e-7)
        _compare(got, ref, dt, sysp.kS, sysp.kT, oracle)
        small = W.small_pair()
        rp, col, val = iso_csr(oracle, small, 0.05)
        zk = W.random_phase_samples(small.Z, 40, seed=m + 1)
        ref = oracle.trace_sampling(rp, col, val, zk, dt, 400 * dt, m, 1e-9)
        sampler.set_h(rp, col, val)
        got = sampler.trace_sampling(zk, dt, 400 * dt, m, 1e-9)
        _compare(got, ref, dt, small.kS, small.kT, oracle)
    finally:
        sampler.set_krylov("mgs")


@pytest.mark.parametrize("M", [1, 33, 70])
def test_ragged_sample_counts(sampler, oracle, M):
    sysp, sim = W.small_pair(), W.small_sim(M=M, t_end_ns=300.0)
    rp, col, val = iso_csr(oracle, sysp, 0.05)
    zk = W.random_phase_samples(sysp.Z, M, seed=M)
    ref = oracle.trace_sampling(rp, col, val, zk, sim.dt, sim.t_end, 12, sim.tol)
    sampler.set_h(rp, col, val)
    got = sampler.trace_sampling(zk, sim.dt, sim.t_end, 12, sim.tol)
    _compare(got, ref, sim.dt, sysp.kS, sysp.kT, oracle)


@pytest.mark.parametrize("state", ["T0", "Tp", "Tm"])
def test_other_initial_states(sampler, oracle, state):
    sysp = W.small_pair()
    rp, col, val = iso_csr(oracle, sysp, 0.3)
    dt, t_end = 0.17608596, 50 * 0.17608596
    zk = W.random_phase_samples(sysp.Z, 8, seed=11)
    ref = oracle.trace_sampling(rp, col, val, zk, dt, t_end, 16, 1e-6, init_state=state)
    sampler.set_h(rp, col, val, index_base=0)
    got = sampler.trace_sampling(zk, dt, t_end, 16, 1e-6, init_state=state)
    _compare(got, ref, dt, sysp.kS, sysp.kT, oracle)


def test_one_based_csr_input(sampler, oracle):
    """spc_set_h accepts the reference's 1-based CSR (stdlib CSR_cdp_type)."""
    sysp = W.small_pair()
    rp, col, val = iso_csr(oracle, sysp, 0.05)
    sampler.set_h(rp + 1, col + 1, val, index_base=1)
    rp2, col2, val2 = sampler.get_h()
    assert np.array_equal(rp2, rp) and np.array_equal(col2, col) and np.array_equal(val2, val)


def test_time_window_shorter_than_dt(sampler, oracle):
    sysp = W.small_pair()
    rp, col, val = iso_csr(oracle, sysp, 0.05)
    zk = W.random_phase_samples(sysp.Z, 3)
    for t_end in (0.0, 0.05, 0.17608596):
        ref = oracle.trace_sampling(rp, col, val, zk, 0.17608596, t_end, 8, 1e-5)
        sampler.set_h(rp, col, val)
        got = sampler.trace_sampling(zk, 0.17608596, t_end, 8, 1e-5)
        assert np.max(np.abs(got.P_S - ref["P_S"])) <= ABS_TOL


def test_argument_errors(sampler, oracle):
    sysp = W.small_pair()
    rp, col, val = iso_csr(oracle, sysp, 0.05)
    sampler.set_h(rp, col, val)
    zk = W.random_phase_samples(sysp.Z, 2)
    with pytest.raises(SpcError):
        sampler.trace_sampling(zk, 0.1, 1.0, 500, 1e-5)  # m > n
    with pytest.raises(SpcError):
        sampler.trace_sampling(zk, -0.1, 1.0, 8, 1e-5)   # dt <= 0


def test_exact_krylov_breakdown_gives_the_exact_answer(sampler, oracle):
    """One proton, m = 8 = n: the Krylov space is exhausted and the reference's
    get_krylov divides by a zero norm (NaN, reproduced by the oracle). The
    device path continues with a zero basis vector and returns the closed form
    P_S(t) = 5/8 + 3/8 cos(a t)."""
    from spin_dynamics_gb300.spinsys import Electron, SysParam
    a = 0.8
    sysp = SysParam(e1=Electron(g_I=[2], A=[np.eye(3) * a]), e2=Electron(g_I=[], A=[]))
    rp, col, val = iso_csr(oracle, sysp, 0.0)
    dt = 0.5 * GAMMA_E / 1000
    zk = np.eye(2, dtype=complex)
    ref = oracle.trace_sampling(rp, col, val, zk, dt, 30 * dt, 8, 1e-14)
    assert np.isnan(ref["P_S"][1])
    sampler.set_h(rp, col, val)
    got = sampler.trace_sampling(zk, dt, 30 * dt, 8, 1e-14)
    n = int(np.ceil(30 * dt / dt)) + 1
    t = np.arange(n) * dt
    assert np.max(np.abs(got.P_S[:n] - (5 / 8 + 3 / 8 * np.cos(a * t)))) < 1e-12


@pytest.mark.parametrize("method", ["mgs", "auto"])
def test_graph_replay_equals_direct_launches(sampler, method):
    """Rounds replayed as captured CUDA graphs give the same bits as the
    same launches issued one by one (single job and a batch; the tiled path,
    which small systems take only when the per-sample path is off)."""
    DT = 1.0 * GAMMA_E / 1000
    s = W.small_pair()
    zk = W.random_phase_samples(s.Z, 40, seed=12)
    nb = W.notebook_pair()
    nb.kS = nb.kT = s.kS
    zb = W.random_phase_samples(nb.Z, 7, seed=13)
    out = {}
    sampler.set_krylov(method)
    sampler.set_sample_path("off")
    try:
        for graphs in (False, True):
            sampler.set_graphs(graphs)
            sampler.build_h(s, 0.05, "reference")
            one = sampler.trace_sampling(zk, DT, 120 * DT, 12, 1e-6)
            sampler.build_h_batch([nb, s], [0.1, 0.05], "reference")
            many = sampler.trace_sampling_batch([zb, zk], DT, 120 * DT, 12, 1e-6)
            out[graphs] = (one, many, sampler.stats()["rounds"])
    finally:
        sampler.set_graphs(True)
        sampler.set_krylov("mgs")
        sampler.set_sample_path("auto")
    (a1, am, _), (b1, bm, rounds) = out[False], out[True]
    assert rounds > 2
    for k in ("P_S", "P_T0", "P_Tp", "P_Tm"):
        assert np.array_equal(getattr(a1, k), getattr(b1, k))
        for x, y in zip(am, bm):
            assert np.array_equal(getattr(x, k), getattr(y, k))
