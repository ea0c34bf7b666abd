"""Total-spin block decomposition of equivalent spin-1/2 nuclei
(symmetry_dynamics; src/symmetry.f90, src/moments.f90; PRL 120, 220604).

A group of n equivalent spin-1/2 nuclei (equal isotropic coupling, same
gyromagnetic ratio) couples to total spins I = n/2, n/2-1, ..., each
occurring d(n, I) times; the Hamiltonian is block diagonal in them, and the
trace over the full nuclear space is the sum over blocks of d(block) x the
trace over the block. Each block is an ordinary radical pair whose "nuclei"
are the groups with multiplicity 2I+1, so it runs through the same GPU
propagator. A block's result enters with weight
w = (prod_groups d) * Z_block / Z_full (src/symmetry.f90:95-96, weight
:210-225).

Generalisations over the reference (its defects are listed in the module
docstrings' source lines):
* radical 2's group sizes are used (the reference copies them into an empty
  slice, src/symmetry.f90:62, so its radical-2 groups are undefined);
* blocks of any multiplicity: the group's nuclear Zeeman uses the group's
  gyromagnetic ratio instead of stopping on multiplicity outside {2, 3}
  (src/hamiltonian.f90:132-138);
* nuclei that are not spin-1/2 (14N) are kept as explicit nuclei of every
  block instead of refusing the system (src/symmetry.f90:54);
* couplings that fall into exactly M distinct values form their groups
  directly; otherwise `shrink` (moment matching, src/moments.f90:15-95)
  approximates N inequivalent couplings by M groups as the reference does.
"""
from __future__ import annotations

import math
import os
from itertools import product as _product
from typing import Optional

import numpy as np
import scipy.linalg as sl

from .observables import Observables
from .spinsys import GAMMA_1H, Electron, SimParam, SpinchemError, SysParam


# ---------------------------------------------------------------- moments
def count_set_bits(i: int) -> int:
    """count_set_bits (src/moments.f90:160-180)."""
    return bin(i & ((1 << 64) - 1)).count("1")


def quad_rule(W_init: np.ndarray, X_init: np.ndarray, N: int):
    """quad_rule (src/moments.f90:97-158): discrete Stieltjes (Lanczos)
    contraction of the len(X_init)-point rule (W_init, X_init) to an N-point
    Gauss rule; returns (weights W, nodes X), nodes ascending."""
    W_init = np.asarray(W_init, float)
    X_init = np.asarray(X_init, float)
    q = np.sqrt(W_init)
    P = np.zeros((len(X_init), N))
    w = np.zeros(N)
    x = np.zeros(N)
    for k in range(N):
        q2 = np.linalg.norm(q)
        if q2 == 0.0:
            raise SpinchemError("quad_rule 1")
        P[:, k] = q / q2
        q = X_init * P[:, k]
        for j in range(k, -1, -1):
            pq = float(np.dot(P[:, j], q))
            if j == k:
                w[k] = q2
                x[k] = pq
            q = q - pq * P[:, j]
    weight = w[0]
    E = np.roll(w, -1)[: N - 1]  # cshift(W, 1)
    if N > 1:
        vals, Z = sl.eigh_tridiagonal(x, E)
    else:
        vals, Z = x.copy(), np.ones((1, 1))
    return (weight * Z[0, :]) ** 2, vals


def newton(aw_bar, w_bar, a_bar, n_bar, M, maxit=30):
    """newton (src/moments.f90:182-240): solve sum_j n_j a_j^k =
    sum_j w_j aw_j^k, k = 1..M, for a; returns (a, icode)."""
    a_bar = np.array(a_bar, float)
    n_bar = np.asarray(n_bar, float)
    dap = None
    for it in range(1, maxit + 1):
        f = np.array([np.dot(n_bar, a_bar ** k) - np.dot(w_bar, aw_bar ** k) for k in range(1, M + 1)])
        g = np.array([k * n_bar * a_bar ** (k - 1) for k in range(1, M + 1)])
        try:
            q = np.linalg.solve(g, f)
        except np.linalg.LinAlgError:
            return a_bar, 1
        a_abs = np.sum(np.abs(a_bar))
        d_abs = np.sum(np.abs(q))
        a_old = a_bar.copy()
        a_bar = a_bar - q
        da = d_abs / a_abs
        if da > 1.0:
            return a_bar, 1
        if 1.0 + da == 1.0:
            return a_bar, 0
        if it > 1 and da >= dap:
            return a_old, 0
        dap = da
    return a_bar, 2


def shrink(a_iso, M: int):
    """shrink (src/moments.f90:15-95): M groups (a_bar, n_bar) of equivalent
    nuclei approximating the couplings a_iso by moment matching."""
    a_iso = np.asarray(a_iso, float)
    if a_iso.size == 0:
        return np.zeros(0), np.zeros(0, int), 0
    if M >= a_iso.size:
        raise SpinchemError("Error: Symetry reduction requires M<N")
    w_bar, aw_bar = quad_rule(np.ones(a_iso.size), a_iso, M)
    nfloor = w_bar.astype(int)  # int() truncates
    ndiff = a_iso.size - int(nfloor.sum())
    best = None
    dmom = np.finfo(float).max
    for ib in range(1 << M):
        if count_set_bits(ib) != ndiff:
            continue
        ntemp = nfloor + np.array([(ib >> i) & 1 for i in range(M)])
        atemp, icode = newton(aw_bar, w_bar, aw_bar.copy(), ntemp, M)
        if icode != 0:
            continue
        # moment error as the reference evaluates it (src/moments.f90:81-86)
        emom = sum(abs(np.sum(atemp ** k) - np.sum(a_iso ** k)) for k in range(1, M + 2))
        if emom < dmom:
            dmom = emom
            best = (atemp.copy(), ntemp.copy())
    if best is None:
        raise SpinchemError("Error: moment matching found no integer group sizes")
    return best[0], best[1], M


# ---------------------------------------------------------------- blocks
def cartesian_product(n):
    """cartesian_product (src/symmetry.f90:171-208): every combination of
    block multiplicities, group i taking k = 2(j-1)+1+mod(n_i,2),
    j = 1..n_i/2+1; the first group varies fastest. Returns (len(n), combos)."""
    n = [int(v) for v in n]
    opts = [[2 * j + 1 + (ni % 2) for j in range(ni // 2 + 1)] for ni in n]
    if not n:
        return np.zeros((0, 1), int)
    combos = [c[::-1] for c in _product(*opts[::-1])]
    return np.array(combos, int).T


def nCr(n: int, r: int) -> int:
    return math.comb(n, r)


def weight(n, k) -> int:
    """weight (src/symmetry.f90:210-225): number of times the block with
    group multiplicities k occurs, prod_i C(n_i, (n_i+k_i-1)/2) 2k_i/(n_i+k_i+1)."""
    w = 1
    for ni, ki in zip(n, k):
        w = w * (nCr(int(ni), (int(ni) + int(ki) - 1) // 2) * (2 * int(ki)) // (int(ni) + int(ki) + 1))
    return w


def sort_col_prod(K):
    """sort_col_prod (src/utils.f90:25-50): columns ordered by the product of
    their entries (stable)."""
    Z = np.prod(K, axis=0).astype(np.int64) if K.size else np.ones(K.shape[1], np.int64)
    idx = np.argsort(Z, kind="stable")
    return Z[idx], K[:, idx]


def exact_groups(a_iso, M: int):
    """Groups of exactly equal couplings when there are exactly M distinct
    values (the decomposition is then exact), else None."""
    vals, counts = np.unique(np.asarray(a_iso, float), return_counts=True)
    if len(vals) == M:
        return vals, counts
    return None


def _radical_groups(e: Electron, M: int):
    """Split a radical's nuclei into spin-1/2 groups and explicit nuclei."""
    half = [i for i, g in enumerate(e.g_I) if g == 2 and (e.gamma_I is None or e.gamma_I[i] == GAMMA_1H)]
    other = [i for i in range(len(e.g_I)) if i not in half]
    a = e.a_iso[half] if half else np.zeros(0)
    if len(half) == 0 or M == 0:
        return np.zeros(0), np.zeros(0, int), other
    ex = exact_groups(a, M)
    if ex is not None:
        return ex[0], ex[1], other
    a_bar, n_bar, _ = shrink(a, M)
    return a_bar, n_bar, other


def reduce_system(sys_: SysParam, gI1, a1_bar, other1, gI2, a2_bar, other2) -> SysParam:
    """reduce_system (src/symmetry.f90:141-169): the block's radical pair; a
    group of multiplicity k is one nucleus with isotropic coupling a_bar and
    the 1H gyromagnetic ratio; explicit nuclei are copied."""
    def radical(e, gI, a_bar, other):
        g = [int(k) for k in gI] + [e.g_I[i] for i in other]
        A = [np.eye(3) * float(a) for a in a_bar] + [e.A[i] for i in other]
        gam = [GAMMA_1H] * len(gI) + [e.gammas[i] for i in other]
        return Electron(g_I=g, A=A, g=e.g, w=e.w, gamma_I=gam)
    return SysParam(e1=radical(sys_.e1, gI1, a1_bar, other1), e2=radical(sys_.e2, gI2, a2_bar, other2),
                    J=sys_.J, D=sys_.D.copy(), kS=sys_.kS, kT=sys_.kT)


def blocks(sys_: SysParam, M1: int, M2: int):
    """All blocks of the decomposition: list of (weight, SysParam, Z_block),
    in the reference's order (by block dimension)."""
    a1, n1, o1 = _radical_groups(sys_.e1, M1)
    a2, n2, o2 = _radical_groups(sys_.e2, M2)
    n_bar = list(n1) + list(n2)
    K = cartesian_product(n_bar)
    Zc, K = sort_col_prod(K)
    Z_full = sys_.Z
    Z_explicit = int(np.prod([sys_.e1.g_I[i] for i in o1] or [1])) * int(np.prod([sys_.e2.g_I[i] for i in o2] or [1]))
    out = []
    for c in range(K.shape[1]):
        gI1 = K[: len(n1), c]
        gI2 = K[len(n1):, c]
        w_ij = weight(n1, gI1) * weight(n2, gI2)
        Zb = int(Zc[c]) * Z_explicit
        w_k = float(w_ij * Zb) / float(Z_full)
        out.append((w_k, reduce_system(sys_, gI1, a1, o1, gI2, a2, o2), Zb))
    return out


def rng_stream(seed, n: int) -> np.ndarray:
    from . import _native as nat
    import ctypes as C
    out = np.zeros(max(n, 1), np.uint64)
    s0, s1 = (int(seed[0]), int(seed[1]))
    s0 = s0 - 2**64 if s0 >= 2**63 else s0
    s1 = s1 - 2**64 if s1 >= 2**63 else s1
    nat.check(nat.lib().spc_rng_stream(s0, s1, n, out.ctypes.data_as(C.c_void_p)))
    return out[:n]


def _selected(sys_: SysParam, sim: SimParam, from_restart: bool = True):
    """Blocks that count (weight >= sim.block_tol; from sim.restart on unless
    from_restart is False), with their 1-based indices and per-block seeds
    drawn from sim.seed."""
    bl = blocks(sys_, sim.M1, sim.M2)
    seeds = rng_stream(sim.seed, 2 * len(bl)).reshape(-1, 2) if bl else np.zeros((0, 2), np.uint64)
    start = sim.restart if sim.isRestart and from_restart else 1
    out = []
    for i, (w_k, sysb, Zb) in enumerate(bl, start=1):
        if i < start or w_k < sim.block_tol:
            continue
        out.append((i, w_k, sysb, Zb, (int(seeds[i - 1, 0]), int(seeds[i - 1, 1]))))
    return out


BLOCK_FILES = (("S_prob.data", "P_S"), ("T0_prob.data", "P_T0"), ("Tp_prob.data", "P_Tp"),
               ("Tm_prob.data", "P_Tm"))


def block_folder(field_folder: str, i: int) -> str:
    """Where block i (1-based) of a field keeps its populations."""
    return os.path.join(field_folder, f"hamiltonian_{i}")


def read_block(field_folder: str, i: int, T: int) -> Observables:
    """A block's populations as its run wrote them (17 significant digits:
    the same doubles)."""
    arrs = {}
    for name, key in BLOCK_FILES:
        path = os.path.join(block_folder(field_folder, i), name)
        if not os.path.exists(path):
            raise SpinchemError(f"Error: restart: no saved block results in {path}")
        with open(path) as f:
            v = np.array([float(x) for x in f.read().split()], dtype=np.float64)
        if v.size != T:
            raise SpinchemError(f"Error: restart: {path} holds {v.size} values, expected {T}")
        arrs[key] = v
    return Observables(arrs["P_S"], arrs["P_T0"], arrs["P_Tp"], arrs["P_Tm"])


def _block_vectors(sel, sim: SimParam, exact_blocks: bool):
    from . import dynamics
    if exact_blocks:
        return [np.eye(Zb, dtype=np.complex128) for _, _, _, Zb, _ in sel]
    return [dynamics.seeded_samples(seed, Zb, sim.N_samples) for _, _, _, Zb, seed in sel]


def _budget_entries(states_per_entry: float) -> float:
    """Vector entries (rows x samples) a batch may hold: a third of the free
    device memory over `states_per_entry` complex states per entry."""
    from .dynamics import device_memory
    free, _ = device_memory()
    return max(1.0, free / 3.0 / (16.0 * states_per_entry))


def symmetrised_dynamics(sys_: SysParam, sim: SimParam, out: Optional[str] = None, sampler=None,
                         exact_blocks: bool = False, field=None) -> Observables:
    """symmetrised_dynamics (src/symmetry.f90:16-139) for one field: trace
    sampling over every block whose weight reaches sim.block_tol
    (sim.N_samples vectors per block, seeds drawn per block from sim.seed),
    each scaled by its weight, summed in block order, then yields
    (get_kinetics) and the output files. The blocks propagate together
    through the batch API (groups bounded by device memory). With
    exact_blocks=True every block is traced exactly over its basis states.
    field (a 3-vector, mT) switches to the general Hamiltonian (anisotropic
    explicit nuclei, tilted field); by default the reference's builder with
    the field -w along z. With `out`, each propagated block's populations go
    to out/hamiltonian_<i>/ and a restart reads the blocks before it from
    there (symmetrised_fields)."""
    if field is None:
        return symmetrised_fields(sys_, sim, [-sys_.e1.w], [out] if out is not None else None, sampler,
                                  exact_blocks)[0]
    return symmetrised_fields(sys_, sim, [np.asarray(field, float)], [out] if out is not None else None,
                              sampler, exact_blocks, mode="general")[0]


def symmetrised_fields(sys_: SysParam, sim: SimParam, fields, folders=None, sampler=None,
                       exact_blocks: bool = False, mode: str = "reference") -> list:
    """symmetrised_dynamics for every field of `fields` (scalars along z for
    the reference builder, 3-vectors for mode="general"): all (block, field)
    jobs from the restart block on, block-major, in batches bounded by device
    memory. With folders, block i's populations of field k go to
    folders[k]/hamiltonian_<i>/ (the reference writes them to
    <output_folder>/hamiltonian_<i>/, which every field overwrites), and the
    blocks before sim.restart are read back from there instead of being left
    unset: a stopped run resumes where it left off and writes the same files
    as an uninterrupted one. Returns one Observables per field (with yields);
    writes each field's seven files into folders[k]."""
    from . import dynamics
    from .dynamics import batch_groups, padded_samples
    sp = sampler or dynamics.default_sampler()
    sel = _selected(sys_, sim, from_restart=False)
    start = sim.restart if sim.isRestart else 1
    if start > 1 and folders is None:
        raise SpinchemError("Error: restart needs the output folders that hold the earlier blocks")
    run = [b for b in sel if b[0] >= start]
    zks = _block_vectors(run, sim, exact_blocks)
    T = dynamics.num_time_points(sim.dt, sim.t_end)
    # block-major: a run stopped after some batches has finished every field
    # of its first blocks, so restart = the first unfinished block resumes it
    jobs = [(k, r) for r in range(len(run)) for k in range(len(fields))]
    sizes = [4 * run[r][3] * padded_samples(zks[r].shape[0]) for _, r in jobs]
    got = {}
    for grp in batch_groups(sizes, _budget_entries(sim.N_krylov + 4)):
        sp.build_h_batch([run[jobs[q][1]][2] for q in grp], [fields[jobs[q][0]] for q in grp], mode)
        rs = sp.trace_sampling_batch([zks[jobs[q][1]] for q in grp], sim.dt, sim.t_end, sim.N_krylov, sim.tol,
                                     sim.init_state)
        for q, r in zip(grp, rs):
            k, i = jobs[q][0], run[jobs[q][1]][0]
            got[(k, i)] = r
            if folders is not None:  # as soon as the batch is done
                bf = block_folder(folders[k], i)
                os.makedirs(bf, exist_ok=True)
                r.output(bf)
    out = []
    for k in range(len(fields)):
        res = Observables.zeros(T)
        for i, w_k, _, _, _ in sel:
            r = got[(k, i)] if i >= start else read_block(folders[k], i, T)
            r.scale(w_k)
            res.update(r)
        res.get_kinetics(sim.dt, sys_.kS, sys_.kT)
        if folders is not None:
            res.output(folders[k])
        out.append(res)
    return out


def symmetrised_yield_gradient(sys_: SysParam, sim: SimParam, B, sampler=None, directions=None,
                               n_quad: int = 0, checkpoint_every: int = 0, wS: float = 1.0,
                               wT: float = 0.0, exact_blocks: bool = False, gradient: bool = True) -> list:
    """Yields of the block decomposition and their gradient with respect to
    the field vector, J, D, kS and kT (the field set of
    spc_yield_gradient_batch), for the field B (mT, 3-vector) or for each of
    `directions` (n x 3 unit vectors, field |B| along each). Every (block,
    direction) job shares one adjoint sweep (groups bounded by device
    memory). Block results enter with their weights. Returns one dict per
    direction: Phi_S, Phi_T, B (3), J, D (3 x 3), kS, kT, and for directions
    the derivatives with respect to the polar and azimuthal angles theta, phi
    of the field. gradient=False runs the forward sweep alone (the stepwise
    yields; derivatives zero)."""
    from . import dynamics
    from .dynamics import batch_groups, padded_samples
    sp = sampler or dynamics.default_sampler()
    B = np.asarray(B, float).reshape(3)
    if directions is None:
        fields = [B]
    else:
        fields = [np.linalg.norm(B) * np.asarray(d, float) / np.linalg.norm(d) for d in directions]
    sel = _selected(sys_, sim, from_restart=False)
    zks = _block_vectors(sel, sim, exact_blocks)
    jobs = [(f, j) for f in range(len(fields)) for j in range(len(sel))]
    acc = [dict(Phi_S=0.0, Phi_T=0.0, B=np.zeros(3), J=0.0, D=np.zeros((3, 3)), kS=0.0, kT=0.0)
           for _ in fields]
    sizes = [4 * sel[j][3] * padded_samples(zks[j].shape[0]) for _, j in jobs]
    # nodes per step: as given, or the largest count the norm bound asks of
    # any (block, field) job (what the batched call takes with n_quad = 0)
    nq = n_quad or max(dynamics.gradient_nodes(sel[j][2], fields[f], sim.dt) for f, j in jobs)
    # states per vector entry held by the sweep: basis, checkpoints, segment, node states
    for grp in batch_groups(sizes, _budget_entries(sim.N_krylov + 6 + 8 * (nq + 1))):
        systems = [sel[jobs[q][1]][2] for q in grp]
        got = sp.yield_gradient_batch(systems, [fields[jobs[q][0]] for q in grp], [zks[jobs[q][1]] for q in grp],
                                      sim.dt, sim.t_end, sim.N_krylov, n_quad=nq,
                                      checkpoint_every=checkpoint_every, wS=wS, wT=wT, hyperfine=False,
                                      init_state=sim.init_state, gradient=gradient)
        for q, g in zip(grp, got):
            f, j = jobs[q]
            w = sel[j][1]
            a = acc[f]
            a["Phi_S"] += w * g.Phi_S
            a["Phi_T"] += w * g.Phi_T
            a["B"] += w * g.B
            a["J"] += w * g.J
            a["D"] += w * g.D
            a["kS"] += w * g.kS
            a["kT"] += w * g.kT
    if directions is not None:
        for f, a in zip(fields, acc):
            r = np.linalg.norm(f)
            th = np.arccos(np.clip(f[2] / r, -1.0, 1.0))
            ph = np.arctan2(f[1], f[0])
            dth = r * np.array([np.cos(th) * np.cos(ph), np.cos(th) * np.sin(ph), -np.sin(th)])
            dph = r * np.array([-np.sin(th) * np.sin(ph), np.sin(th) * np.cos(ph), 0.0])
            a["theta"], a["phi"] = float(th), float(ph)
            a["dtheta"] = float(a["B"] @ dth)
            a["dphi"] = float(a["B"] @ dph)
    return acc
