"""symmetry_dynamics on the GPU: the block-decomposed propagation equals the
full-space propagation (exact traces), and the sampled driver equals the
oracle on the same per-block seeds."""
import numpy as np
import pytest

from spin_dynamics_gb300 import symmetry as S
from spin_dynamics_gb300.dynamics import exact_dynamics, seeded_samples
from spin_dynamics_gb300.spinsys import GAMMA_E, SimParam
from test_symmetry import small_equivalent_system

pytestmark = pytest.mark.gpu


def sim(M=8):
    return SimParam.from_input_units(type="symmetry_dynamics", B=[0.1], init_state="singlet",
                                     seed=(42, 99), N_samples=M, t_end_ns=60.0, dt_ns=1.0,
                                     N_krylov=16, tol=1e-12, M1=1, M2=1, block_tol=0.0)


def test_blocks_reproduce_full_space(sampler):
    s = small_equivalent_system()
    sm = sim()
    # a rebuild every dt step makes both propagations exact to rounding (the
    # block and full Krylov spaces differ, so their truncation errors differ)
    sm.tol = 1e-30
    blk = S.symmetrised_dynamics(s, sm, sampler=sampler, exact_blocks=True)
    full = exact_dynamics(s, sm, sampler=sampler)
    n = int(np.ceil(sm.t_end / sm.dt)) + 1
    for k in ("P_S", "P_T0", "P_Tp", "P_Tm"):
        assert np.max(np.abs(getattr(blk, k)[:n] - getattr(full, k)[:n])) < 1e-10
    full.get_kinetics(sm.dt, s.kS, s.kT)
    assert np.max(np.abs(blk.Phi_S - full.Phi_S)) < 1e-10


def test_sampled_blocks_match_oracle(sampler, oracle):
    s = small_equivalent_system()
    sm = sim(M=6)
    got = S.symmetrised_dynamics(s, sm, sampler=sampler)
    bl = S.blocks(s, 1, 1)
    seeds = oracle.rng_stream(sm.seed, 2 * len(bl)).reshape(-1, 2)
    T = oracle.num_time_points(sm.dt, sm.t_end)
    tot = np.zeros((4, T))
    for i, (w, b, Zb) in enumerate(bl):
        e1, e2 = b.e1, b.e2
        rp, col, val = oracle.build_h_general(e1.g_I, e1.A, e1.gammas, e2.g_I, e2.A, e2.gammas,
                                              [0, 0, 0.1], b.J, b.D, b.kS, b.kT)
        zk = oracle.seeded_samples((int(seeds[i, 0]), int(seeds[i, 1])), Zb, sm.N_samples)
        assert np.array_equal(zk, seeded_samples((int(seeds[i, 0]), int(seeds[i, 1])), Zb, sm.N_samples))
        r = oracle.trace_sampling(rp, col, val, zk, sm.dt, sm.t_end, sm.N_krylov, sm.tol)
        tot += w * np.stack([r["P_S"], r["P_T0"], r["P_Tp"], r["P_Tm"]])
    for i, k in enumerate(("P_S", "P_T0", "P_Tp", "P_Tm")):
        assert np.max(np.abs(getattr(got, k) - tot[i])) < 1e-10


def test_block_tolerance_skips_light_blocks(sampler):
    s = small_equivalent_system()
    sm = sim()
    sm.block_tol = 0.3
    bl = S.blocks(s, 1, 1)
    kept = [w for w, _, _ in bl if w >= 0.3]
    assert 0 < len(kept) < len(bl)
    res = S.symmetrised_dynamics(s, sm, sampler=sampler, exact_blocks=True)
    assert abs(res.P_S[0] - sum(kept)) < 1e-14  # P_S(0) = 1 per block, weighted


def test_block_gradient_equals_full_space_gradient(sampler):
    """Exact traces: the weighted block yields and their field/coupling
    gradient equal the full-space ones (basis-state samples, Z of them)."""
    s = small_equivalent_system()
    sm = sim()
    sm.t_end = 12 * sm.dt
    B = np.array([0.03, 0.02, 0.1])
    blk = S.symmetrised_yield_gradient(s, sm, B, sampler=sampler, exact_blocks=True, n_quad=8)[0]
    full = sampler.yield_gradient_batch([s], [B], [np.eye(s.Z, dtype=complex)], sm.dt, sm.t_end,
                                        sm.N_krylov, n_quad=8, hyperfine=False)[0]
    assert abs(blk["Phi_S"] - full.Phi_S) <= 1e-9 * abs(full.Phi_S)
    scale = max(np.max(np.abs(full.B)), abs(full.J), abs(full.kS))
    for k in ("B", "J", "D", "kS", "kT"):
        assert np.max(np.abs(np.asarray(blk[k]) - np.asarray(getattr(full, k)))) <= 1e-8 * scale, k


def test_compass_map_angle_derivatives(sampler):
    """dPhi_S/dtheta, dPhi_S/dphi of the block decomposition against central
    differences of its own yields."""
    s = small_equivalent_system()
    sm = sim(M=4)
    sm.t_end = 10 * sm.dt
    dirs = np.array([[0.3, 0.4, 0.866], [-0.5, 0.2, 0.3]])
    Bmag = 0.2
    got = S.symmetrised_yield_gradient(s, sm, [0, 0, Bmag], sampler=sampler, directions=dirs, n_quad=8)
    for d, g in zip(dirs, got):
        th, ph = g["theta"], g["phi"]
        for key, (dth, dph) in (("dtheta", (1e-5, 0.0)), ("dphi", (0.0, 1e-5))):
            vals = []
            for sgn in (1, -1):
                t2, p2 = th + sgn * dth, ph + sgn * dph
                f = Bmag * np.array([np.sin(t2) * np.cos(p2), np.sin(t2) * np.sin(p2), np.cos(t2)])
                vals.append(S.symmetrised_yield_gradient(s, sm, f, sampler=sampler, n_quad=8)[0]["Phi_S"])
            fd = (vals[0] - vals[1]) / 2e-5
            assert abs(g[key] - fd) <= 1e-6 * max(abs(fd), 1e-3 * abs(g["Phi_S"])), (key, g[key], fd)
