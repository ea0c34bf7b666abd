"""Adjoint gradient of the yields (spc_yield_gradient) against central finite
differences of the dense stepwise model, plus its schedule invariances."""
import numpy as np
import pytest

import dense
from spin_dynamics_gb300 import workloads as W
from spin_dynamics_gb300.dynamics import num_time_points
from spin_dynamics_gb300.spinsys import GAMMA_E, Electron, SysParam

pytestmark = pytest.mark.gpu
DT = 1.0 * GAMMA_E / 1000
# gradient entries: |g - g_fd| <= GRAD_RTOL * max|g_fd| (central differences of
# the dense model carry ~1e-9 relative error; the Gauss-Legendre rule with 8
# nodes and exact Krylov spaces are far below that)
GRAD_RTOL = 2e-7


def aniso_pair(g1, g2, seed, kS, kT):
    rng = np.random.default_rng(seed)
    t = lambda: (lambda R: R @ np.diag(rng.uniform(-1.5, 1.5, 3)) @ R.T)(W._haar_rotation(rng))
    return SysParam(e1=Electron(g_I=list(g1), A=[t() for _ in g1]),
                    e2=Electron(g_I=list(g2), A=[t() for _ in g2]),
                    J=0.03, D=W.axial_dipolar(-0.3) + 0.05 * np.eye(3)[[1, 0, 2]],
                    kS=kS, kT=kT)


def pack(s, B):
    A = [a.reshape(3, 3).T.reshape(9) for a in list(s.e1.A) + list(s.e2.A)]
    return np.concatenate([np.asarray(B, float), [s.J], np.asarray(s.D).T.reshape(9), [s.kS, s.kT]]
                          + A)


def dense_objective(s, v, zk, t_end, wS, wT):
    n1 = len(s.e1.g_I)
    A = [v[15 + 9 * j:24 + 9 * j].reshape(3, 3).T for j in range(len(s.e1.g_I) + len(s.e2.g_I))]
    H = dense.hamiltonian(s.e1.g_I, A[:n1], s.e2.g_I, A[n1:], v[0:3], v[3], v[4:13].reshape(3, 3).T,
                          v[13], v[14])
    T = num_time_points(DT, t_end)
    PhiS, PhiT = dense.stepwise_yields(H, zk, DT, T, v[13], v[14])
    return wS * PhiS + wT * PhiT, (PhiS, PhiT)


def fd_gradient(s, B, zk, t_end, wS, wT, h=1e-5):
    v0 = pack(s, B)
    g = np.zeros_like(v0)
    for i in range(v0.size):
        vp, vm = v0.copy(), v0.copy()
        vp[i] += h
        vm[i] -= h
        g[i] = (dense_objective(s, vp, zk, t_end, wS, wT)[0] -
                dense_objective(s, vm, zk, t_end, wS, wT)[0]) / (2 * h)
    return g


@pytest.mark.parametrize("rates", [(1.3, 0.4), (0.8, 0.8)], ids=["unequal", "equal"])
def test_gradient_matches_dense_finite_differences(sampler, rates):
    kS, kT = rates[0] / GAMMA_E * 50, rates[1] / GAMMA_E * 50
    s = aniso_pair([2], [2, 3], seed=5, kS=kS, kT=kT)  # dim 48
    B = np.array([0.11, -0.07, 0.2])
    zk = W.random_phase_samples(s.Z, 5, seed=9)
    t_end = 12 * DT
    got = sampler.yield_gradient(s, B, zk, DT, t_end, m=48, n_quad=8)
    _, (PhiS, PhiT) = dense_objective(s, pack(s, B), zk, t_end, 1.0, 0.0)
    assert abs(got.Phi_S - PhiS) <= 1e-12 * max(1.0, abs(PhiS))
    assert abs(got.Phi_T - PhiT) <= 1e-12 * max(1.0, abs(PhiT))
    ref = fd_gradient(s, B, zk, t_end, 1.0, 0.0)
    scale = np.max(np.abs(ref))
    err = np.abs(got.raw - ref)
    assert np.max(err) <= GRAD_RTOL * scale, (np.argmax(err), got.raw[np.argmax(err)], ref[np.argmax(err)])


def test_triplet_objective_and_truncated_krylov(sampler):
    """wT Phi_T at dim 288 with a Krylov dimension below the space (m = 28)."""
    s = W.small_pair()
    rng = np.random.default_rng(3)
    for e in (s.e1, s.e2):
        e.A = [(lambda R: R @ np.diag(rng.uniform(-1, 1, 3)) @ R.T)(W._haar_rotation(rng)) for _ in e.A]
    s.J, s.D = 0.02, W.axial_dipolar(-0.2)
    s.kS, s.kT = 20.0 / GAMMA_E, 5.0 / GAMMA_E
    B = np.array([0.0, 0.03, 0.05])
    zk = W.random_phase_samples(s.Z, 3, seed=4)
    t_end = 8 * DT
    got = sampler.yield_gradient(s, B, zk, DT, t_end, m=28, n_quad=8, wS=0.0, wT=1.0)
    ref = fd_gradient(s, B, zk, t_end, 0.0, 1.0)
    err = np.abs(got.raw - ref)
    assert np.max(err) <= 1e-6 * np.max(np.abs(ref)), (np.argmax(err), got.raw[np.argmax(err)], ref[np.argmax(err)])


def test_lanczos_matches_mgs_and_finite_differences(sampler):
    """kS == kT at dim 288 with m = 24: the three-term recurrence (explicit
    SPC_KRYLOV_LANCZOS) against full MGS and the dense model."""
    s = W.small_pair()
    rng = np.random.default_rng(11)
    for e in (s.e1, s.e2):
        e.A = [(lambda R: R @ np.diag(rng.uniform(-1, 1, 3)) @ R.T)(W._haar_rotation(rng)) for _ in e.A]
    s.J, s.D = 0.02, W.axial_dipolar(-0.2)
    s.kS = s.kT = 10.0 / GAMMA_E
    B = np.array([0.02, 0.0, 0.06])
    zk = W.random_phase_samples(s.Z, 4, seed=6)
    t_end = 9 * DT
    mgs = sampler.yield_gradient(s, B, zk, DT, t_end, m=24, n_quad=8)
    sampler.set_krylov("lanczos")
    try:
        lz = sampler.yield_gradient(s, B, zk, DT, t_end, m=24, n_quad=8)
    finally:
        sampler.set_krylov("mgs")
    scale = np.max(np.abs(mgs.raw))
    assert np.max(np.abs(lz.raw - mgs.raw)) <= 1e-10 * scale
    ref = fd_gradient(s, B, zk, t_end, 1.0, 0.0)
    assert np.max(np.abs(mgs.raw - ref)) <= 1e-6 * np.max(np.abs(ref))


def test_checkpoint_spacing_does_not_change_results(sampler):
    s = aniso_pair([2, 2], [3], seed=2, kS=0.02, kT=0.01)
    B = np.array([0.05, 0.0, 0.1])
    zk = W.random_phase_samples(s.Z, 40, seed=1)  # two tiles, one partial
    t_end = 13 * DT
    runs = [sampler.yield_gradient(s, B, zk, DT, t_end, m=20, n_quad=4, checkpoint_every=K)
            for K in (0, 1, 3, 100)]
    for r in runs[1:]:
        assert np.array_equal(r.raw, runs[0].raw)
        assert r.Phi_S == runs[0].Phi_S


def test_short_window_has_zero_yield(sampler):
    s = W.notebook_pair()
    zk = W.random_phase_samples(s.Z, 2, seed=1)
    got = sampler.yield_gradient(s, 0.05, zk, DT, 0.5 * DT, m=8)  # T = 3: no Simpson panel
    assert got.Phi_S == 0.0 and not np.any(got.raw)


def test_full_size_directional_derivatives(sampler):
    """dim 55296 (the large anisotropic pair): the adjoint gradient against
    central differences (h = 1e-6 relative) of the GPU's own stepwise yields
    along single parameters and a random direction."""
    from spin_dynamics_gb300.torch_ops import pack_params, unpack_params
    s, B = W.large_pair()
    s.kS, s.kT = 20.0 / GAMMA_E, 20.0 / GAMMA_E
    zk = W.random_phase_samples(s.Z, 2, seed=3)
    t_end = 6 * DT
    g = sampler.yield_gradient(s, B, zk, DT, t_end, m=30, n_quad=6, checkpoint_every=2)
    v0 = pack_params(s, B).numpy()
    rng = np.random.default_rng(1)
    dirs = {"Bx": 0, "J": 3, "kS": 13, "A0_xy": 15 + 3}
    cases = [(k, np.eye(v0.size)[i]) for k, i in dirs.items()]
    cases.append(("random", rng.normal(size=v0.size) * np.abs(v0).clip(1e-3)))
    for name, d in cases:
        h = 1e-6 * max(np.abs(v0 @ d) / np.linalg.norm(d), 1.0) / np.linalg.norm(d)
        sp, Bp = unpack_params(s, v0 + h * d)
        sm, Bm = unpack_params(s, v0 - h * d)
        fd = (sampler.stepwise_yields(sp, Bp, zk, DT, t_end, 30)[0] -
              sampler.stepwise_yields(sm, Bm, zk, DT, t_end, 30)[0]) / (2 * h)
        ad = g.raw @ d
        # 1e-6 of the gradient scale |g| |d|: a central difference of yields
        # evaluated to ~1e-15 carries ~1e-10 of rounding noise at h = 1e-6,
        # which is 1e-5 relative for the smallest entries (dPhi/dBx ~ 8e-6)
        assert abs(ad - fd) <= 1e-6 * np.linalg.norm(g.raw) * np.linalg.norm(d), (name, ad, fd)


def richardson(f, x0, d, h):
    """Central difference of f along d at x0, Richardson-extrapolated from
    steps h and 2h (truncation O(h^4))."""
    c = lambda k: (f(x0 + k * h * d) - f(x0 - k * h * d)) / (2 * k * h)
    return (4.0 * c(1) - c(2)) / 3.0


def test_gradient_components_within_1e6_relative_dense(sampler):
    """Every gradient component above 1e-4 of the largest agrees with the
    dense model's central difference to 1e-6 relative (dim 48, exact Krylov
    space, the node count of the library's rule)."""
    s = aniso_pair([2], [2, 3], seed=5, kS=1.3 / GAMMA_E * 50, kT=0.4 / GAMMA_E * 50)
    B = np.array([0.11, -0.07, 0.2])
    zk = W.random_phase_samples(s.Z, 3, seed=2)
    t_end = 12 * DT
    got = sampler.yield_gradient(s, B, zk, DT, t_end, m=48)
    v0 = pack(s, B)
    f = lambda v: dense_objective(s, v, zk, t_end, 1.0, 0.0)[0]
    fd = np.array([richardson(f, v0, np.eye(v0.size)[i], 1e-4 * max(1.0, abs(v0[i]))) for i in range(v0.size)])
    big = np.abs(fd) >= 1e-4 * np.max(np.abs(fd))
    assert big.sum() >= 20
    rel = np.abs(got.raw - fd)[big] / np.abs(fd)[big]
    assert np.max(rel) <= 1e-6, (np.argmax(rel), np.max(rel))


def test_full_size_gradient_components_within_1e6_relative(sampler):
    """dim 55296: single gradient components (field, exchange, dipolar, rates
    and hyperfine elements) above 1e-3 of the largest agree to 1e-6 relative
    with Richardson central differences of the GPU's own stepwise yields."""
    from spin_dynamics_gb300.torch_ops import pack_params, unpack_params
    s, B = W.large_pair()
    s.kS, s.kT = 20.0 / GAMMA_E, 20.0 / GAMMA_E
    zk = W.random_phase_samples(s.Z, 2, seed=3)
    t_end = 6 * DT
    g = sampler.yield_gradient(s, B, zk, DT, t_end, m=30, checkpoint_every=2)
    v0 = pack_params(s, B).numpy()

    def f(v):
        sv, Bv = unpack_params(s, v)
        return sampler.stepwise_yields(sv, Bv, zk, DT, t_end, 30)[0]

    # the largest components of each kind: field and couplings (0..14),
    # radical-1 and radical-2 hyperfine elements
    order = lambda lo, hi: [lo + i for i in np.argsort(-np.abs(g.raw[lo:hi]))]
    idx = order(0, 15)[:4] + order(15, 15 + 9 * 7)[:3] + order(15 + 9 * 7, g.raw.size)[:3]
    scale = np.max(np.abs(g.raw))
    for i in idx:
        assert abs(g.raw[i]) >= 1e-4 * scale, (i, g.raw[i])
        fd = richardson(f, v0, np.eye(v0.size)[i], 1e-4 * max(abs(v0[i]), 1e-2))
        assert abs(g.raw[i] - fd) <= 1e-6 * abs(fd), (i, g.raw[i], fd)


def test_torch_autograd_matches_adjoint(sampler):
    import torch
    from spin_dynamics_gb300.torch_ops import pack_params, yield_objective
    s = aniso_pair([2], [2, 2], seed=8, kS=0.02, kT=0.005)
    B = np.array([0.0, 0.04, 0.03])
    zk = W.random_phase_samples(s.Z, 6, seed=2)
    t_end = 10 * DT
    p = pack_params(s, B).clone().requires_grad_(True)
    val = yield_objective(p, sampler, s, zk, DT, t_end, 32, n_quad=8)
    val.backward()
    g = sampler.yield_gradient(s, B, zk, DT, t_end, 32, n_quad=8)
    assert val.item() == g.Phi_S
    assert torch.equal(p.grad, torch.from_numpy(g.raw))
    with torch.no_grad():
        v2 = yield_objective(p.detach(), sampler, s, zk, DT, t_end, 32)
    assert abs(v2.item() - g.Phi_S) <= 1e-14 * abs(g.Phi_S)
    ok = torch.autograd.gradcheck(
        lambda q: yield_objective(q, sampler, s, zk, DT, t_end, 32, n_quad=8),
        (p.detach().clone().requires_grad_(True),), eps=1e-6, atol=1e-8, rtol=1e-5)
    assert ok


def test_batch_equals_single_calls(sampler):
    """Jobs of dims 48, 288 and 72 with 5, 33 and 7 samples in one sweep
    against one call per job."""
    a = aniso_pair([2], [2, 3], seed=5, kS=0.03, kT=0.01)
    b = W.small_pair()
    rng = np.random.default_rng(4)
    for e in (b.e1, b.e2):
        e.A = [(lambda R: R @ np.diag(rng.uniform(-1, 1, 3)) @ R.T)(W._haar_rotation(rng)) for _ in e.A]
    b.kS, b.kT = 0.02, 0.05
    c = aniso_pair([3, 2], [3], seed=6, kS=0.01, kT=0.01)
    systems = [a, b, c]
    fields = [np.array([0.1, 0.0, 0.2]), np.array([0.0, 0.03, 0.05]), np.array([0.05, 0.05, 0.0])]
    zks = [W.random_phase_samples(s.Z, M, seed=20 + i) for i, (s, M) in enumerate(zip(systems, (5, 33, 7)))]
    t_end = 9 * DT
    got = sampler.yield_gradient_batch(systems, fields, zks, DT, t_end, 24, n_quad=6, checkpoint_every=3)
    for s, B, zk, g in zip(systems, fields, zks, got):
        one = sampler.yield_gradient(s, B, zk, DT, t_end, 24, n_quad=6, checkpoint_every=3)
        scale = np.max(np.abs(one.raw))
        assert np.max(np.abs(g.raw - one.raw)) <= 1e-12 * scale
        assert abs(g.Phi_S - one.Phi_S) <= 1e-14
        assert abs(g.Phi_T - one.Phi_T) <= 1e-14


def test_field_set_matches_full_set(sampler):
    s = aniso_pair([2, 2], [3], seed=3, kS=0.02, kT=0.01)
    B = np.array([0.02, -0.04, 0.1])
    zk = W.random_phase_samples(s.Z, 9, seed=5)
    t_end = 7 * DT
    full = sampler.yield_gradient(s, B, zk, DT, t_end, 24)
    fld = sampler.yield_gradient_batch([s], [B], [zk], DT, t_end, 24, hyperfine=False)[0]
    scale = np.max(np.abs(full.raw))
    assert np.max(np.abs(fld.raw[:15] - full.raw[:15])) <= 1e-12 * scale
    assert not np.any(fld.raw[15:])


def test_field_gradient_of_a_spin2_group(sampler):
    """A symmetry-block-like system: one effective nucleus of multiplicity 5
    (four equivalent 1H at total spin 2, gyromagnetic ratio of 1H) and one 1H;
    dPhi/d(B, J, D, kS, kT) against central differences of the dense model."""
    from spin_dynamics_gb300.spinsys import GAMMA_1H
    s = SysParam(e1=Electron(g_I=[5], A=[np.eye(3) * 0.4], gamma_I=[GAMMA_1H]),
                 e2=Electron(g_I=[2], A=[np.diag([0.3, 0.5, -0.2])], gamma_I=[GAMMA_1H]),
                 J=0.02, D=W.axial_dipolar(-0.3), kS=0.03, kT=0.01)
    B = np.array([0.3, 0.1, 0.4])
    zk = W.random_phase_samples(s.Z, 4, seed=8)
    t_end = 10 * DT
    got = sampler.yield_gradient_batch([s], [B], [zk], DT, t_end, 40, n_quad=8, hyperfine=False)[0]

    def phi(v):
        H = dense.hamiltonian(s.e1.g_I, s.e1.A, s.e2.g_I, s.e2.A, v[0:3], v[3], v[4:13].reshape(3, 3).T,
                              v[13], v[14], gam1=s.e1.gamma_I, gam2=s.e2.gamma_I)
        return dense.stepwise_yields(H, zk, DT, num_time_points(DT, t_end), v[13], v[14])[0]

    v0 = np.concatenate([B, [s.J], np.asarray(s.D).T.reshape(9), [s.kS, s.kT]])
    ref = np.zeros(15)
    for i in range(15):
        e = np.zeros(15)
        e[i] = 1e-5
        ref[i] = (phi(v0 + e) - phi(v0 - e)) / 2e-5
    assert abs(got.Phi_S - phi(v0)) <= 1e-12
    err = np.abs(got.raw[:15] - ref)
    assert np.max(err) <= 2e-7 * np.max(np.abs(ref)), (np.argmax(err), got.raw[:15], ref)


def test_gradient_argument_and_capacity_errors(sampler):
    """Errors come back as status codes with messages: bad arguments, a
    multiplicity the full gradient set does not take, Lanczos with unequal
    rates, and a request larger than device memory (refused by the memory
    plan before anything is allocated or launched)."""
    from spin_dynamics_gb300._native import SpcError
    from spin_dynamics_gb300.spinsys import GAMMA_1H
    s = aniso_pair([2], [2], seed=1, kS=0.02, kT=0.01)
    zk = W.random_phase_samples(s.Z, 3, seed=1)
    for kw in ({"m": 0}, {"m": 49}, {"n_quad": -1}, {"n_quad": 17}, {"checkpoint_every": -1}):
        args = dict(m=8, n_quad=4, checkpoint_every=0)
        args.update(kw)
        with pytest.raises(SpcError):
            sampler.yield_gradient(s, [0, 0, 0.1], zk, DT, 6 * DT, args["m"], n_quad=args["n_quad"],
                                   checkpoint_every=args["checkpoint_every"])
    with pytest.raises(SpcError, match="must be positive"):
        sampler.yield_gradient(s, [0, 0, 0.1], zk, -DT, 6 * DT, 8)
    s5 = SysParam(e1=Electron(g_I=[5], A=[np.eye(3) * 0.4], gamma_I=[GAMMA_1H]),
                  e2=Electron(g_I=[2], A=[np.eye(3) * 0.3]), kS=0.02, kT=0.02)
    z5 = W.random_phase_samples(s5.Z, 2, seed=2)
    with pytest.raises(SpcError, match="multiplicity"):
        sampler.yield_gradient(s5, [0, 0, 0.1], z5, DT, 6 * DT, 8)
    sampler.yield_gradient_batch([s5], [[0, 0, 0.1]], [z5], DT, 6 * DT, 8, hyperfine=False)  # field set: fine
    sampler.set_krylov("lanczos")
    try:
        with pytest.raises(SpcError, match="Lanczos"):
            sampler.yield_gradient(s, [0, 0, 0.1], zk, DT, 6 * DT, 8)
    finally:
        sampler.set_krylov("mgs")
    big, B = W.large_pair()
    zbig = W.random_phase_samples(big.Z, 1, seed=3)
    # a checkpoint every step over 20,000 steps: ~20,000 states of 28 MB (one
    # 32-sample tile of dim 55296), far above the device's memory
    with pytest.raises(SpcError, match="device memory"):
        sampler.yield_gradient(big, B, zbig, DT, 20000 * DT, 8, checkpoint_every=1)
