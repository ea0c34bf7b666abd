"""Lanczos mode (three-term recurrence for H_eff = Hermitian - i*kappa) against
the oracle's literal MGS Arnoldi, at the same 1e-10 absolute tolerance."""
import numpy as np
import pytest

from conftest import general_csr, iso_csr
from spin_dynamics_gb300 import workloads as W
from spin_dynamics_gb300._native import SpcError
from spin_dynamics_gb300.spinsys import GAMMA_E

ABS_TOL = 1e-10
pytestmark = pytest.mark.gpu


@pytest.fixture
def lanczos(sampler):
    sampler.set_krylov("lanczos")
    yield sampler
    sampler.set_krylov("mgs")


def _max_err(got, ref):
    return max(np.max(np.abs(getattr(got, k) - ref[k])) for k in ("P_S", "P_T0", "P_Tp", "P_Tm"))


def test_small_pair_full_length(lanczos, oracle):
    sysp, sim = W.small_pair(), W.small_sim()
    rp, col, val = iso_csr(oracle, sysp, 0.05)
    zk = W.random_phase_samples(sysp.Z, 64)
    ref = oracle.trace_sampling(rp, col, val, zk, sim.dt, sim.t_end, sim.N_krylov, sim.tol)
    lanczos.build_h(sysp, 0.05, "reference")
    got = lanczos.trace_sampling(zk, sim.dt, sim.t_end, sim.N_krylov, sim.tol)
    assert _max_err(got, ref) <= ABS_TOL
    phi_g = oracle.kinetics(got.P_S, got.P_T0, got.P_Tp, got.P_Tm, sim.dt, sysp.kS, sysp.kT)[0]
    phi_o = oracle.kinetics(ref["P_S"], ref["P_T0"], ref["P_Tp"], ref["P_Tm"], sim.dt, sysp.kS, sysp.kT)[0]
    assert np.max(np.abs(phi_g - phi_o)) <= ABS_TOL
    assert lanczos.stats()["krylov_builds"] == int(ref["n_builds"].sum())


def test_large_pair_anisotropic(lanczos, oracle):
    sysp, B = W.large_pair()
    sim = W.large_sim(M=4, t_end_ns=40.0)
    rp, col, val = general_csr(oracle, sysp, B)
    zk = W.random_phase_samples(sysp.Z, 4, seed=4)
    ref = oracle.trace_sampling(rp, col, val, zk, sim.dt, sim.t_end, sim.N_krylov, sim.tol)
    lanczos.build_h(sysp, B, "general")
    got = lanczos.trace_sampling(zk, sim.dt, sim.t_end, sim.N_krylov, sim.tol)
    assert _max_err(got, ref) <= ABS_TOL


def test_large_pair_isotropic(lanczos, oracle):
    sysp, B = W.large_pair(isotropic=True)
    sim = W.large_sim(M=8, t_end_ns=60.0)
    rp, col, val = iso_csr(oracle, sysp, B[2])
    zk = W.random_phase_samples(sysp.Z, 8, seed=3)
    ref = oracle.trace_sampling(rp, col, val, zk, sim.dt, sim.t_end, sim.N_krylov, sim.tol)
    lanczos.build_h(sysp, B[2], "reference")
    got = lanczos.trace_sampling(zk, sim.dt, sim.t_end, sim.N_krylov, sim.tol)
    assert _max_err(got, ref) <= ABS_TOL


def test_small_space_falls_back_to_mgs(lanczos, oracle):
    """The 48-dim example with m = 10 over all basis states: Lanczos bases of
    the small invariant subspaces lose orthogonality; those samples are rebuilt
    with full MGS and the result still matches."""
    sysp = W.notebook_pair()
    rp, col, val = iso_csr(oracle, sysp, 0.2)
    dt = 0.5 * GAMMA_E / 1000
    t_end = 99.5 * GAMMA_E / 1000
    zk = np.eye(sysp.Z, dtype=complex)
    ref = oracle.trace_sampling(rp, col, val, zk, dt, t_end, 10, 1e-8)
    lanczos.build_h(sysp, 0.2, "reference")
    got = lanczos.trace_sampling(zk, dt, t_end, 10, 1e-8)
    assert _max_err(got, ref) <= ABS_TOL
    assert lanczos.stats()["krylov_builds"] == int(ref["n_builds"].sum())


def test_lanczos_refused_for_unequal_rates(lanczos, oracle):
    sysp = W.small_pair()
    sysp.kT = sysp.kS * 0.25  # kS != kT: H_eff is not Hermitian plus a scalar
    lanczos.build_h(sysp, 0.05, "reference")
    zk = W.random_phase_samples(sysp.Z, 2)
    with pytest.raises(SpcError):
        lanczos.trace_sampling(zk, 0.176, 5.0, 8, 1e-5)


def test_auto_uses_mgs_for_unequal_rates(sampler, oracle):
    sysp = W.small_pair()
    sysp.kT = sysp.kS * 0.25
    rp, col, val = iso_csr(oracle, sysp, 0.05)
    zk = W.random_phase_samples(sysp.Z, 6, seed=2)
    ref = oracle.trace_sampling(rp, col, val, zk, 0.17608596, 60 * 0.17608596, 14, 1e-6)
    sampler.set_krylov("auto")
    try:
        sampler.set_h(rp, col, val)  # Hermiticity detected from the CSR itself
        got = sampler.trace_sampling(zk, 0.17608596, 60 * 0.17608596, 14, 1e-6)
    finally:
        sampler.set_krylov("mgs")
    assert _max_err(got, ref) <= ABS_TOL


@pytest.mark.parametrize("method", ["lanczos", "mgs"])
def test_split_diagonal_shift_in_a_user_csr(sampler, oracle, method):
    """A caller's CSR whose rows carry the Haberkorn shift in two duplicate
    diagonal entries (a quarter and three quarters of -i*kbar/2): it is
    Hermitian plus a scalar shift once duplicates are summed, so Lanczos
    runs on the Hermitian part and MGS adds the shift back in the SpMM; both
    match the oracle on the same CSR."""
    sysp = W.small_pair()
    rp, col, val = iso_csr(oracle, sysp, 0.05)
    n = len(rp) - 1
    rp2, col2, val2 = [0], [], []
    for r in range(n):
        ks = range(rp[r], rp[r + 1])
        kap = -sum(val[k].imag for k in ks if col[k] == r)
        first = True
        for k in ks:
            v = val[k]
            col2.append(col[k])
            if col[k] == r:
                val2.append(complex(v.real, -0.25 * kap if first else 0.0))
                first = False
            else:
                val2.append(v)
        col2.append(r)
        val2.append(complex(0.0, -0.75 * kap))
        rp2.append(len(col2))
    rp2, col2, val2 = np.array(rp2, np.int32), np.array(col2, np.int32), np.array(val2)
    zk = W.random_phase_samples(sysp.Z, 40, seed=9)
    dt = 0.17608596
    ref = oracle.trace_sampling(rp2, col2, val2, zk, dt, 150 * dt, 16, 1e-7)
    sampler.set_krylov(method)
    try:
        sampler.set_h(rp2, col2, val2)
        got = sampler.trace_sampling(zk, dt, 150 * dt, 16, 1e-7)
        fallbacks = sampler.stats()["lanczos_fallbacks"]
    finally:
        sampler.set_krylov("mgs")
    assert _max_err(got, ref) <= ABS_TOL
    if method == "lanczos":
        assert fallbacks == 0
