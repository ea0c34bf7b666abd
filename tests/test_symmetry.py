"""Total-spin block decomposition (src/symmetry.f90, src/moments.f90) on the
CPU: multiplicity combinations and weights, moment matching, and the
exactness of the decomposition: the weighted sum of the blocks' exact traces
equals the full-space exact trace (both propagated by the oracle)."""
import numpy as np
import pytest

from spin_dynamics_gb300 import symmetry as S
from spin_dynamics_gb300.spinsys import GAMMA_14N, GAMMA_1H, GAMMA_E, Electron, SimParam, SysParam


def test_cartesian_product_order_and_weights():
    K = S.cartesian_product([3, 2])
    # group 1 (n = 3): k in {2, 4}; group 2 (n = 2): k in {1, 3}; group 1 fastest
    assert K.tolist() == [[2, 4, 2, 4], [1, 1, 3, 3]]
    assert S.weight([3], [2]) == 2 and S.weight([3], [4]) == 1
    assert S.weight([2], [1]) == 1 and S.weight([2], [3]) == 1
    # degeneracies times block size sum to the full dimension 2^n
    for n in range(1, 9):
        ks = S.cartesian_product([n])[0]
        assert sum(S.weight([n], [k]) * k for k in ks) == 2 ** n
    Z, Ks = S.sort_col_prod(S.cartesian_product([4, 4]))
    assert list(Z) == sorted(Z)


def test_quad_rule_and_shrink():
    a = np.array([0.1, 0.1, 0.4, 0.4, 0.4, 0.9])
    w, x = S.quad_rule(np.ones(6), a, 3)
    assert np.allclose(np.sort(x), [0.1, 0.4, 0.9], atol=1e-12)
    assert np.allclose(w[np.argsort(x)], [2, 3, 1], atol=1e-10)
    rng = np.random.default_rng(0)
    a = rng.uniform(0.2, 0.8, 7)
    a_bar, n_bar, M = S.shrink(a, 2)
    assert n_bar.sum() == 7 and M == 2
    for k in (1, 2):
        assert abs(np.dot(n_bar, a_bar ** k) - np.sum(a ** k)) < 1e-8 * np.sum(a ** k)
    with pytest.raises(Exception):
        S.shrink(a, 7)


def small_equivalent_system():
    """Radical 1: three equivalent 1H (0.5 mT) + one 14N (0.3 mT);
    radical 2: two equivalent 1H (0.4 mT)."""
    e1 = Electron(g_I=[2, 2, 2, 3], A=[np.eye(3) * 0.5] * 3 + [np.eye(3) * 0.3])
    e2 = Electron(g_I=[2, 2], A=[np.eye(3) * 0.4] * 2)
    s = SysParam(e1=e1, e2=e2, J=0.05, kS=1.0 / GAMMA_E, kT=1.0 / GAMMA_E)
    s.e1.w = s.e2.w = -0.1
    return s


def test_block_weights_sum_to_one_and_keep_14N_explicit():
    s = small_equivalent_system()
    bl = S.blocks(s, 1, 1)
    assert len(bl) == 4
    assert abs(sum(w for w, _, _ in bl) - 1.0) < 1e-15
    for w, b, Zb in bl:
        assert 3 in b.e1.g_I and b.e1.gammas[-1] == GAMMA_14N
        assert all(g == GAMMA_1H for g in b.e1.gammas[:-1])
        assert Zb == b.Z
    assert [Zb for _, _, Zb in bl] == sorted(Zb for _, _, Zb in bl)


def test_block_sum_equals_full_trace(oracle):
    s = small_equivalent_system()
    dt = 1.0 * GAMMA_E / 1000
    t_end = 40 * dt

    def run(sysb):
        e1, e2 = sysb.e1, sysb.e2
        rp, col, val = oracle.build_h_general(e1.g_I, e1.A, e1.gammas, e2.g_I, e2.A, e2.gammas,
                                              [0, 0, -sysb.e1.w], sysb.J, sysb.D, sysb.kS, sysb.kT)
        return oracle.trace_sampling(rp, col, val, np.eye(sysb.Z, dtype=complex), dt, t_end,
                                     min(24, sysb.N), 1e-14)

    full = run(s)
    tot = {k: 0.0 for k in ("P_S", "P_T0", "P_Tp", "P_Tm")}
    for w, b, _ in S.blocks(s, 1, 1):
        r = run(b)
        for k in tot:
            tot[k] = tot[k] + w * r[k]
    n = int(np.ceil(t_end / dt)) + 1
    for k in tot:
        assert np.max(np.abs(tot[k][:n] - full[k][:n])) < 1e-11, k


def test_selected_blocks_and_their_seeded_vectors():
    from spin_dynamics_gb300.dynamics import seeded_samples
    s = small_equivalent_system()
    sm = SimParam.from_input_units(type="symmetry_dynamics", B=[0.1], init_state="singlet",
                                   seed=(42, 99), N_samples=3, t_end_ns=10.0, dt_ns=1.0,
                                   N_krylov=8, tol=1e-5, M1=1, M2=1, block_tol=0.2)
    sel = S._selected(s, sm)
    bl = S.blocks(s, 1, 1)
    assert [i for i, *_ in sel] == [i + 1 for i, (w, _, _) in enumerate(bl) if w >= 0.2]
    seeds = S.rng_stream(sm.seed, 2 * len(bl)).reshape(-1, 2)
    zks = S._block_vectors(sel, sm, exact_blocks=False)
    for (i, w, b, Zb, seed), z in zip(sel, zks):
        assert seed == (int(seeds[i - 1, 0]), int(seeds[i - 1, 1]))
        assert np.array_equal(z, seeded_samples(seed, Zb, 3))
    from spin_dynamics_gb300.dynamics import batch_groups
    assert batch_groups([5, 5, 5, 20, 1], 10) == [[0, 1], [2], [3], [4]]
