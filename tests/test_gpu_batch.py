"""Batched propagation of independent systems of uneven dimension (pairs,
field orientations) in one call, against the oracle per job."""
import numpy as np
import pytest

from conftest import general_csr, iso_csr
from spin_dynamics_gb300 import workloads as W
from spin_dynamics_gb300.spinsys import GAMMA_E

ABS_TOL = 1e-10
pytestmark = pytest.mark.gpu
DT = 1.0 * GAMMA_E / 1000


def fib_sphere(n, r=0.05):
    i = np.arange(n) + 0.5
    phi = np.arccos(1 - 2 * i / n)
    th = np.pi * (1 + 5 ** 0.5) * i
    return r * np.stack([np.cos(th) * np.sin(phi), np.sin(th) * np.sin(phi), np.cos(phi)], 1)


def _check(got, ref):
    for k in ("P_S", "P_T0", "P_Tp", "P_Tm"):
        assert np.max(np.abs(getattr(got, k) - ref[k])) <= ABS_TOL, k


@pytest.mark.parametrize("method", ["mgs", "auto"])
def test_uneven_pairs_in_one_batch(sampler, oracle, method):
    iso_large, B = W.large_pair(isotropic=True)
    systems = [W.notebook_pair(), W.small_pair(), iso_large, W.small_pair()]
    fields = [0.2, 0.05, B[2], 0.3]
    for s in systems:
        s.kS = s.kT = 1.0 / GAMMA_E
    Ms = [5, 40, 3, 33]
    zks = [W.random_phase_samples(s.Z, M, seed=10 + i) for i, (s, M) in enumerate(zip(systems, Ms))]
    t_end = 30 * DT
    sampler.set_krylov(method)
    try:
        sampler.build_h_batch(systems, fields, "reference")
        got = sampler.trace_sampling_batch(zks, DT, t_end, 12, 1e-6)
    finally:
        sampler.set_krylov("mgs")
    for s, f, zk, g in zip(systems, fields, zks, got):
        rp, col, val = iso_csr(oracle, s, f)
        _check(g, oracle.trace_sampling(rp, col, val, zk, DT, t_end, 12, 1e-6))


def test_orientation_scan_batch_equals_single_calls(sampler, oracle):
    rng = np.random.default_rng(8)
    s = W.small_pair()
    for e in (s.e1, s.e2):
        e.A = [(lambda R: R @ np.diag(rng.uniform(-2, 2, 3)) @ R.T)(W._haar_rotation(rng)) for _ in e.A]
    s.J, s.D = 0.01, W.axial_dipolar(-0.4)
    dirs = fib_sphere(6)
    zk = W.random_phase_samples(s.Z, 32, seed=2)
    t_end = 25 * DT
    sampler.build_h_batch([s] * len(dirs), list(dirs), "general")
    got = sampler.trace_sampling_batch([zk] * len(dirs), DT, t_end, 16, 1e-5)
    for b, g in zip(dirs, got):
        rp, col, val = general_csr(oracle, s, b)
        _check(g, oracle.trace_sampling(rp, col, val, zk, DT, t_end, 16, 1e-5))
        sampler.build_h(s, b, "general")
        single = sampler.trace_sampling(zk, DT, t_end, 16, 1e-5)
        for k in ("P_S", "P_Tm"):
            assert np.max(np.abs(getattr(single, k) - getattr(g, k))) < 1e-13


def test_jobs_sharing_a_system(sampler, oracle):
    s = W.small_pair()
    sampler.build_h_batch([s], [0.05], "reference")
    za = W.random_phase_samples(s.Z, 7, seed=1)
    zb = W.random_phase_samples(s.Z, 9, seed=2)
    got = sampler.trace_sampling_batch([za, zb], DT, 20 * DT, 10, 1e-6, job_sys=[0, 0])
    rp, col, val = iso_csr(oracle, s, 0.05)
    _check(got[0], oracle.trace_sampling(rp, col, val, za, DT, 20 * DT, 10, 1e-6))
    _check(got[1], oracle.trace_sampling(rp, col, val, zb, DT, 20 * DT, 10, 1e-6))


def test_mixed_rates_batch_uses_mgs(sampler, oracle):
    a, b = W.small_pair(), W.small_pair()
    b.kT = b.kS * 0.2  # not Hermitian plus a scalar
    zk = W.random_phase_samples(a.Z, 6, seed=3)
    sampler.set_krylov("auto")
    try:
        sampler.build_h_batch([a, b], [0.05, 0.05], "reference")
        got = sampler.trace_sampling_batch([zk, zk], DT, 15 * DT, 10, 1e-6)
        assert sampler.stats()["lanczos_fallbacks"] == 0
    finally:
        sampler.set_krylov("mgs")
    for s, g in ((a, got[0]), (b, got[1])):
        rp, col, val = iso_csr(oracle, s, 0.05)
        _check(g, oracle.trace_sampling(rp, col, val, zk, DT, 15 * DT, 10, 1e-6))


def test_krylov_dimension_capped_at_job_dimension(sampler, oracle):
    """A 16-dim job at m = 20 runs with m = 16 (its whole space): exact."""
    import dense
    from spin_dynamics_gb300.spinsys import Electron, SysParam
    tiny = SysParam(e1=Electron(g_I=[2], A=[np.eye(3) * 0.6]), e2=Electron(g_I=[2], A=[np.eye(3) * 0.3]),
                    J=0.02, kS=1.0 / GAMMA_E, kT=1.0 / GAMMA_E)
    big = W.small_pair()
    zt = np.eye(tiny.Z, dtype=complex)
    zb = W.random_phase_samples(big.Z, 8, seed=4)
    t_end = 20 * DT
    sampler.build_h_batch([tiny, big], [0.1, 0.1], "reference")
    got = sampler.trace_sampling_batch([zt, zb], DT, t_end, 20, 1e-6)
    n = int(np.ceil(t_end / DT)) + 1
    H = dense.hamiltonian(tiny.e1.g_I, tiny.e1.A, tiny.e2.g_I, tiny.e2.A, [0, 0, 0.1], tiny.J, tiny.D,
                          tiny.kS, tiny.kT)
    PS = dense.trace_sampled_populations(H, zt, np.arange(n) * DT)[0]
    assert np.max(np.abs(got[0].P_S[:n] - PS)) < 1e-12
    rp, col, val = iso_csr(oracle, big, 0.1)
    _check(got[1], oracle.trace_sampling(rp, col, val, zb, DT, t_end, 20, 1e-6))


def test_autotuned_krylov_dimension(sampler, oracle):
    """The autotuner returns one of the candidates with a positive rate for
    each, and a batch run at the chosen dimension keeps parity."""
    systems = [W.notebook_pair(), W.small_pair()]
    for s in systems:
        s.kS = s.kT = 1.0 / GAMMA_E
    fields = [0.1, 0.05]
    zks = [W.random_phase_samples(s.Z, M, seed=30 + i) for i, (s, M) in enumerate(zip(systems, (40, 20)))]
    sampler.build_h_batch(systems, fields, "reference")
    best, rates = sampler.autotune_krylov(zks, DT, 8 * DT, 1e-6, candidates=(8, 12, 16))
    assert best in (8, 12, 16)
    assert all(r > 0 for r in rates.values()) and rates[best] == max(rates.values())
    got = sampler.trace_sampling_batch(zks, DT, 15 * DT, best, 1e-6)
    for s, f, zk, g in zip(systems, fields, zks, got):
        rp, col, val = iso_csr(oracle, s, f)
        _check(g, oracle.trace_sampling(rp, col, val, zk, DT, 15 * DT, best, 1e-6))


def test_torch_tensor_entry_points(sampler, oracle):
    """torch_ops.trace_sampling / trace_sampling_batch on CUDA tensors give
    the host path's populations."""
    import torch
    from spin_dynamics_gb300 import torch_ops
    s = W.small_pair()
    zk = W.random_phase_samples(s.Z, 9, seed=5)
    sampler.build_h(s, 0.05, "reference")
    host = sampler.trace_sampling(zk, DT, 20 * DT, 10, 1e-6)
    dev = torch_ops.trace_sampling(sampler, torch.from_numpy(zk).cuda(), DT, 20 * DT, 10, 1e-6)
    torch.cuda.synchronize()
    assert dev.is_cuda and dev.shape == (4, len(host.P_S))
    assert np.array_equal(dev.cpu().numpy()[0], host.P_S) and np.array_equal(dev.cpu().numpy()[3], host.P_Tm)
    nb = W.notebook_pair()
    zb = W.random_phase_samples(nb.Z, 4, seed=6)
    sampler.build_h_batch([nb, s], [0.1, 0.05], "reference")
    got = torch_ops.trace_sampling_batch(sampler, [torch.from_numpy(zb).cuda(), torch.from_numpy(zk).cuda()],
                                         DT, 20 * DT, 10, 1e-6)
    ref = sampler.trace_sampling_batch([zb, zk], DT, 20 * DT, 10, 1e-6)
    for j in range(2):
        assert np.array_equal(got[j].cpu().numpy()[0], ref[j].P_S)
    with pytest.raises(TypeError):
        torch_ops.trace_sampling(sampler, torch.from_numpy(zk), DT, 20 * DT, 10, 1e-6)


def test_job_runner_splits_by_device_memory(sampler, oracle, monkeypatch):
    """trace_sampling_many with a memory budget of a few jobs: several
    batches, every job against the oracle, in job order."""
    from spin_dynamics_gb300 import dynamics

    systems = [W.small_pair(), W.notebook_pair(), W.small_pair(), W.notebook_pair(), W.small_pair()]
    fields = [0.05, 0.2, 0.3, 0.1, 0.15]
    Ms = [40, 6, 33, 9, 64]
    zks = [W.random_phase_samples(s.Z, M, seed=30 + i) for i, (s, M) in enumerate(zip(systems, Ms))]
    m, t_end = 12, 20 * DT
    # free memory of two dim-288 jobs' bases and states at this m and fraction
    fake_free = 2 * 288 * 64 * 16.0 * (m + 4) / 0.5
    monkeypatch.setattr(dynamics, "device_memory", lambda device=0: (fake_free, fake_free))
    entries = [4 * s.Z * dynamics.padded_samples(M) for s, M in zip(systems, Ms)]
    assert len(dynamics.batch_groups(entries, fake_free * 0.5 / (16.0 * (m + 4)))) >= 3
    got = sampler.trace_sampling_many(systems, fields, zks, DT, t_end, m, 1e-6, mode="reference")
    assert len(got) == len(systems)
    for s, f, zk, g in zip(systems, fields, zks, got):
        rp, col, val = iso_csr(oracle, s, f)
        _check(g, oracle.trace_sampling(rp, col, val, zk, DT, t_end, m, 1e-6))


def test_samples_beyond_the_memory_limit_run_in_chunks(sampler, oracle):
    """A call whose Krylov bases exceed the handle's memory limit runs each
    build round over chunks of 32-sample tiles: same results as the
    unchunked call to rounding, the oracle within 1e-10; a limit below one
    tile is refused."""
    from spin_dynamics_gb300._native import SpcError

    s = W.small_pair()
    zk = W.random_phase_samples(s.Z, 200, seed=4)  # 7 tiles
    t_end, m = 40 * DT, 20
    sampler.set_sample_path("off")  # the tiled path's chunking
    sampler.build_h(s, 0.05, "reference")
    whole = sampler.trace_sampling(zk, DT, t_end, m, 1e-6)
    n_whole = sampler.stats()["kernel_launches"]
    # about 2.9 tiles of bases and per-sample matrices (5.2 MB per tile at
    # dim 288, m = 20) beside the states and populations
    sampler.set_memory_limit(16 << 20)
    try:
        part = sampler.trace_sampling(zk, DT, t_end, m, 1e-6)
        n_part = sampler.stats()["kernel_launches"]
        sampler.set_memory_limit(4 << 20)
        with pytest.raises(SpcError, match="32-sample tile"):
            sampler.trace_sampling(zk, DT, t_end, m, 1e-6)
    finally:
        sampler.set_memory_limit(0)
        sampler.set_sample_path("auto")
    assert n_part > n_whole
    for k in ("P_S", "P_T0", "P_Tp", "P_Tm"):
        assert np.max(np.abs(getattr(part, k) - getattr(whole, k))) < 1e-13, k
    rp, col, val = iso_csr(oracle, s, 0.05)
    _check(part, oracle.trace_sampling(rp, col, val, zk, DT, t_end, m, 1e-6))
    # the handle is usable after the refusal
    again = sampler.trace_sampling(zk[:40], DT, t_end, m, 1e-6)
    _check(again, oracle.trace_sampling(rp, col, val, zk[:40], DT, t_end, m, 1e-6))
