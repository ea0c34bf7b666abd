"""ORACLE — test infrastructure only.

Dense FP64 restatement of the radical-pair Hamiltonian and its exact
propagation by eigendecomposition, used to pin the C++ restatement
(spinchem_oracle.cpp) and the CUDA product at small Hilbert dimension.

The Hamiltonian is assembled independently of the sparse COO code, with
numpy Kronecker products, in getHiso_sp's conventions
(src/hamiltonian.f90:17-205, electron Larmor w = -B from app/main.f90:53-54)
and extended to anisotropic tensors and arbitrary field directions as the
general builder defines them:

    H = -B.(S1+S2) + sum_j (gamma_j/gamma_e) B.I_j + S1.(D + 2J 1).S2
        + sum_j S_e(j).A_j.I_j - i/2 (kS P_S + kT P_T)

Populations follow convert_to_krylov's block definitions
(src/qm_dynamics.f90:469-498) applied to the exact state.
"""
from __future__ import annotations

import numpy as np

GAMMA_E = 176.08596
GAMMA_1H = 0.26752218708
GAMMA_14N = 0.0193297792


def spin_ops(g):
    """Sx, Sy, Sz for multiplicity g, basis m = +S ... -S."""
    S = (g - 1) / 2
    m = S - np.arange(g)
    Sp = np.zeros((g, g), complex)
    for i in range(1, g):
        Sp[i - 1, i] = np.sqrt(S * (S + 1) - m[i] * m[i - 1])
    Sm = Sp.T.copy()
    return (Sp + Sm) / 2, (Sp - Sm) / 2j, np.diag(m).astype(complex)


def hamiltonian(g1, A1, g2, A2, Bvec, J, D, kS, kT, gam1=None, gam2=None):
    """Dense H_eff. A1/A2: sequences of 3x3 (row, col) tensors. Bvec: field (mT)."""
    gs = list(g1) + list(g2)
    As = [np.asarray(a, float).reshape(3, 3) for a in list(A1) + list(A2)]
    if gam1 is None:
        gam1 = [GAMMA_1H if g == 2 else GAMMA_14N for g in g1]
    if gam2 is None:
        gam2 = [GAMMA_1H if g == 2 else GAMMA_14N for g in g2]
    gams = list(gam1) + list(gam2)
    owner = [0] * len(g1) + [1] * len(g2)
    Z = int(np.prod(gs)) if gs else 1
    s = spin_ops(2)
    I2 = np.eye(2)
    S1 = [np.kron(o, I2) for o in s]
    S2 = [np.kron(I2, o) for o in s]
    B = np.asarray(Bvec, float)
    D = np.asarray(D, float).reshape(3, 3)
    Hel = -sum(B[r] * (S1[r] + S2[r]) for r in range(3)).astype(complex)
    Dt = D + 2 * J * np.eye(3)
    for r in range(3):
        for c in range(3):
            Hel = Hel + Dt[r, c] * S1[r] @ S2[c]
    S1S2 = sum(S1[r] @ S2[r] for r in range(3))
    kbar = (kS + 3 * kT) / 4
    dk = (kS - kT) / 4
    Hel = Hel - 0.5j * kbar * np.eye(4) + 2j * dk * S1S2
    H = np.kron(Hel, np.eye(Z))
    for j, g in enumerate(gs):
        I = spin_ops(g)
        Zl = int(np.prod(gs[:j])) if j else 1
        Zr = int(np.prod(gs[j + 1:])) if j + 1 < len(gs) else 1
        emb = lambda E, X: np.kron(E, np.kron(np.eye(Zl), np.kron(X, np.eye(Zr))))
        Se = S1 if owner[j] == 0 else S2
        for r in range(3):
            for c in range(3):
                if As[j][r, c] != 0.0:
                    H = H + As[j][r, c] * emb(Se[r], I[c])
        for c in range(3):
            if B[c] != 0.0:
                H = H + (gams[j] / GAMMA_E) * B[c] * emb(np.eye(4), I[c])
    return H


def theta(which="singlet"):
    h = 1 / np.sqrt(2)
    return {"singlet": np.array([0, h, -h, 0], complex), "T0": np.array([0, h, h, 0], complex),
            "Tp": np.array([1, 0, 0, 0], complex), "Tm": np.array([0, 0, 0, 1], complex)}[which]


def populations(psi_t, Z):
    """psi_t: (..., N) states. Returns (P_S, P_T0, P_Tp, P_Tm) arrays over leading dims."""
    b = [psi_t[..., q * Z:(q + 1) * Z] for q in range(4)]
    dot = lambda x, y: np.sum(np.conj(x) * y, axis=-1)
    Pab, Pba, zqc = dot(b[1], b[1]), dot(b[2], b[2]), dot(b[2], b[1])
    PS = np.real(0.5 * (Pab + Pba) - zqc)
    PT0 = np.real(0.5 * (Pab + Pba) + zqc)
    return PS, PT0, np.real(dot(b[0], b[0])), np.real(dot(b[3], b[3]))


def propagate(H, psi0, times):
    """Exact psi(t) = exp(-i H t) psi0 for every t; psi0: (M, N). Returns (T, M, N)."""
    w, V = np.linalg.eig(H)
    Vi = np.linalg.inv(V)
    c0 = psi0 @ Vi.T  # (M, N)
    ph = np.exp(-1j * np.outer(times, w))  # (T, N)
    return np.einsum("tn,mn,kn->tmk", ph, c0, V)


def trace_sampled_populations(H, zkets, times, which="singlet"):
    """Sample-averaged populations for psi = theta (x) z over the given samples."""
    Z = zkets.shape[1]
    th = theta(which)
    psi0 = np.stack([np.kron(th, z) for z in zkets])
    ps = propagate(H, psi0, times)
    PS, PT0, PTp, PTm = populations(ps, Z)
    return PS.mean(1), PT0.mean(1), PTp.mean(1), PTm.mean(1)


def simpson_weights(T, dt):
    """Weights c_k with Phi_X = k_X sum_k c_k P_X(k) equal to the last value
    get_kinetics returns over T points (src/observables.f90:74-101): panels
    (2i-2, 2i-1, 2i) for i = 1 .. T//2 - 1, each dt/3 (1, 4, 1)."""
    w = np.zeros(T)
    for i in range(1, T // 2):
        w[2 * i - 2] += dt / 3.0
        w[2 * i - 1] += 4.0 * dt / 3.0
        w[2 * i] += dt / 3.0
    return w


def stepwise_yields(H, zkets, dt, T, kS, kT, which="singlet"):
    """(Phi_S, Phi_T) of psi_{k+1} = expm(-i H dt) psi_k, sample-averaged
    populations and get_kinetics' Simpson rule over T points."""
    from scipy.linalg import expm
    Z = zkets.shape[1]
    U = expm(-1j * dt * H)
    psi = np.stack([np.kron(theta(which), z) for z in zkets])
    w = simpson_weights(T, dt)
    aS = aT = 0.0
    for k in range(T):
        if w[k] != 0.0:
            PS, PT0, PTp, PTm = populations(psi, Z)
            aS += w[k] * PS.mean()
            aT += w[k] * (PT0 + PTp + PTm).mean()
        psi = psi @ U.T
    return kS * aS, kT * aT
