"""Seeded synthetic radical-pair systems with the sizes and value
distributions of the benchmark configurations.

The reference publishes no dataset; every system here is generated from a
fixed seed. Energies are in mT, times in ns, rates in 1/us, i.e. input.ini
units (src/spinsys.f90:60-135 converts them at read time; so does
`spinsys.SimParam`).
"""
from __future__ import annotations

import numpy as np

from .spinsys import Electron, SimParam, SysParam, GAMMA_1H, GAMMA_14N


def _haar_rotation(rng: np.random.Generator) -> np.ndarray:
    q, r = np.linalg.qr(rng.normal(size=(3, 3)))
    q = q * np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def axial_dipolar(D: float) -> np.ndarray:
    """Axial dipolar tensor 2/3 D diag(-1,-1,2) (example/utils.py:58-59)."""
    return 2.0 / 3.0 * np.diag((-1.0, -1.0, 2.0)) * D


def _tensors(rng, n, lo, hi, aniso):
    out = []
    for _ in range(n):
        if aniso:
            R = _haar_rotation(rng)
            out.append(R @ np.diag(rng.uniform(lo, hi, 3)) @ R.T)
        else:
            out.append(np.eye(3) * rng.uniform(lo, hi))
    return out


def small_pair(seed: int = 1234) -> SysParam:
    """Plain small pair, Hilbert dim 288: radical A = 1H, 1H, 14N; radical B =
    14N, 1H; isotropic couplings uniform in [0.1, 1.5] mT; J = D = 0;
    kS = kT = 1/us."""
    rng = np.random.default_rng(seed)
    g1, g2 = [2, 2, 3], [3, 2]
    A1 = _tensors(rng, 3, 0.1, 1.5, False)
    A2 = _tensors(rng, 2, 0.1, 1.5, False)
    return SysParam.from_input_units(Electron(g_I=g1, A=A1), Electron(g_I=g2, A=A2), J=0.0,
                                     D=np.zeros((3, 3)), kS_per_us=1.0, kT_per_us=1.0)


def large_pair(seed: int = 2024, isotropic: bool = False) -> tuple[SysParam, np.ndarray]:
    """Single large pair, Hilbert dim 4*3^3*2^9 = 55296: radical A = two 14N
    + five 1H, radical B = one 14N + four 1H; anisotropic couplings
    R diag(U[-2,2]^3) R^T with Haar-random R; J = 0.01 mT; D = -0.4 mT axial;
    kS = kT = 1/us; B = 0.05 mT along a seeded random direction.

    isotropic=True gives the subset the reference itself accepts: each tensor
    replaced by trace(A)/3 times the identity and the field along z.
    Returns (system, field vector in mT)."""
    rng = np.random.default_rng(seed)
    g1, g2 = [3, 3, 2, 2, 2, 2, 2], [3, 2, 2, 2, 2]
    A1 = _tensors(rng, len(g1), -2.0, 2.0, True)
    A2 = _tensors(rng, len(g2), -2.0, 2.0, True)
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    B = 0.05 * d
    if isotropic:
        A1 = [np.eye(3) * (np.trace(a) / 3.0) for a in A1]
        A2 = [np.eye(3) * (np.trace(a) / 3.0) for a in A2]
        B = np.array([0.0, 0.0, 0.05])
    sys_ = SysParam.from_input_units(Electron(g_I=g1, A=A1), Electron(g_I=g2, A=A2), J=0.01,
                                     D=axial_dipolar(-0.4), kS_per_us=1.0, kT_per_us=1.0)
    return sys_, B


def notebook_pair() -> SysParam:
    """The 48-dim system of example/input.ini (1H | 1H + 14N, J = 0.1 mT)."""
    return SysParam.from_input_units(Electron(g_I=[2], A=[np.eye(3) * 0.5]),
                                     Electron(g_I=[2, 3], A=[np.eye(3) * 0.4, np.eye(3) * 0.5]),
                                     J=0.1, D=np.zeros((3, 3)), kS_per_us=0.0, kT_per_us=0.0)


def fibonacci_sphere(n: int, radius: float = 0.05) -> np.ndarray:
    """n field vectors of length `radius` (mT) on a Fibonacci sphere."""
    i = np.arange(n) + 0.5
    phi = np.arccos(1.0 - 2.0 * i / n)
    th = np.pi * (1.0 + 5.0 ** 0.5) * i
    return radius * np.stack([np.cos(th) * np.sin(phi), np.sin(th) * np.sin(phi), np.cos(phi)], 1)


def uneven_pairs(n_pairs: int = 256, seed: int = 3) -> list:
    """The batched uneven set: independent pairs with 2-10 nuclei drawn from
    {1H, 14N} (14N with probability 0.3), split at random between the two
    radicals, Hilbert dimensions 16 ... 4*3^2*2^8 = 9216; couplings as in the
    large pair (anisotropic, principal values in [-2, 2] mT); J = 0.01 mT,
    D = -0.4 mT axial, kS = kT = 1/us; 32-256 samples each.
    Returns [(SysParam, n_samples)]."""
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < n_pairs:
        nn = int(rng.integers(2, 11))
        g = [3 if rng.random() < 0.3 else 2 for _ in range(nn)]
        if 4 * int(np.prod(g)) > 9216:
            continue
        side = rng.random(nn) < 0.5
        g1 = [x for x, s in zip(g, side) if s]
        g2 = [x for x, s in zip(g, side) if not s]
        A1 = _tensors(rng, len(g1), -2.0, 2.0, True)
        A2 = _tensors(rng, len(g2), -2.0, 2.0, True)
        sys_ = SysParam.from_input_units(Electron(g_I=g1, A=A1), Electron(g_I=g2, A=A2), J=0.01,
                                         D=axial_dipolar(-0.4), kS_per_us=1.0, kT_per_us=1.0)
        out.append((sys_, int(rng.integers(32, 257))))
    return out


def symmetric_large_pair(seed: int = 5) -> SysParam:
    """The symmetry-reduced large system: radical A = one 14N + 12 equivalent
    1H in 3 groups of 4 (one isotropic coupling per group, uniform in
    [0.2, 0.8] mT), radical B = one 14N + 8 1H in 2 groups of 4; full Hilbert
    dimension 4*3^2*2^20 = 37,748,736. The 14N tensors are anisotropic
    (principal values uniform in [-2, 2] mT, Haar rotation) so the yield
    depends on the field direction; J = 0.01 mT, D = -0.4 mT axial,
    kS = kT = 1/us. The decomposition into total-spin blocks of the groups is
    exact (symmetry.blocks with M1 = 3, M2 = 2): 243 blocks."""
    rng = np.random.default_rng(seed)
    a1 = rng.uniform(0.2, 0.8, 3)
    a2 = rng.uniform(0.2, 0.8, 2)
    N1 = _tensors(rng, 1, -2.0, 2.0, True)
    N2 = _tensors(rng, 1, -2.0, 2.0, True)
    e1 = Electron(g_I=[2] * 12 + [3], A=[np.eye(3) * a for a in np.repeat(a1, 4)] + N1)
    e2 = Electron(g_I=[2] * 8 + [3], A=[np.eye(3) * a for a in np.repeat(a2, 4)] + N2)
    return SysParam.from_input_units(e1, e2, J=0.01, D=axial_dipolar(-0.4), kS_per_us=1.0, kT_per_us=1.0)


def random_phase_samples(Z: int, M: int, seed: int = 7) -> np.ndarray:
    """M normalised random-phase vectors e^{i phi}/sqrt(Z), phi ~ U[0, 2 pi)."""
    rng = np.random.default_rng(seed)
    phi = rng.uniform(0.0, 2.0 * np.pi, size=(M, Z))
    return np.exp(1j * phi) / np.sqrt(Z)


def small_sim(M: int = 64, t_end_ns: float = 5000.0) -> SimParam:
    return SimParam.from_input_units(type="trace_sampling", B=[0.05], init_state="singlet",
                                     seed=(42, 99), N_samples=M, t_end_ns=t_end_ns, dt_ns=1.0,
                                     N_krylov=20, tol=1e-5)


def large_sim(M: int = 512, t_end_ns: float = 2000.0) -> SimParam:
    return SimParam.from_input_units(type="trace_sampling", B=[0.05], init_state="singlet",
                                     seed=(42, 99), N_samples=M, t_end_ns=t_end_ns, dt_ns=1.0,
                                     N_krylov=30, tol=1e-5)


__all__ = ["small_pair", "large_pair", "notebook_pair", "symmetric_large_pair", "uneven_pairs", "random_phase_samples", "small_sim",
           "large_sim", "axial_dipolar", "GAMMA_1H", "GAMMA_14N"]
