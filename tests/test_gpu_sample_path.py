"""The per-sample propagation of small systems (spc_set_sample_path) against
the CPU oracle (1e-10 absolute, as every parity test) and against the tiled
path (rounding-level agreement, the same Krylov rebuild schedule), in both
of its forms: 'on' runs these calls (at most half as many samples as SMs) on
a cluster of two CTAs per sample, 'single' on one CTA per sample."""
import numpy as np
import pytest

from conftest import general_csr, iso_csr
from spin_dynamics_gb300 import workloads as W
from spin_dynamics_gb300.spinsys import GAMMA_E

ABS_TOL = 1e-10
pytestmark = pytest.mark.gpu
DT = 1.0 * GAMMA_E / 1000
KEYS = ("P_S", "P_T0", "P_Tp", "P_Tm")


def _err(got, ref):
    return max(np.max(np.abs(getattr(got, k) - ref[k])) for k in KEYS)


def _diff(a, b):
    return max(np.max(np.abs(getattr(a, k) - getattr(b, k))) for k in KEYS)


MODES = ("on", "single", "off")


def _both(sampler, run, method):
    """run() on the per-sample path (two CTAs per sample, then one) and on
    the tiled path; returns the results and their stats by mode."""
    out = {}
    sampler.set_krylov(method)
    try:
        for mode in MODES:
            sampler.set_sample_path(mode)
            res = run()
            out[mode] = (res, sampler.stats())
    finally:
        sampler.set_sample_path("auto")
        sampler.set_krylov("mgs")
    return out


def _anisotropic_small_pair(rates=(1.0, 1.0)):
    rng = np.random.default_rng(8)
    s = W.small_pair()
    for e in (s.e1, s.e2):
        e.A = [(lambda R: R @ np.diag(rng.uniform(-2, 2, 3)) @ R.T)(W._haar_rotation(rng)) for _ in e.A]
    s.J, s.D = 0.01, W.axial_dipolar(-0.4)
    s.kS, s.kT = rates[0] / GAMMA_E, rates[1] / GAMMA_E
    return s


@pytest.mark.parametrize("method", ["mgs", "lanczos", "auto"])
@pytest.mark.parametrize("m", [12, 20, 32])
def test_small_pair_reference_builder(sampler, oracle, method, m):
    s = W.small_pair()
    rp, col, val = iso_csr(oracle, s, 0.05)
    zk = W.random_phase_samples(s.Z, 37, seed=m)
    t_end = 300 * DT
    ref = oracle.trace_sampling(rp, col, val, zk, DT, t_end, m, 1e-6)

    def run():
        sampler.build_h(s, 0.05, "reference")
        return sampler.trace_sampling(zk, DT, t_end, m, 1e-6)

    r = _both(sampler, run, method)
    for mode in MODES:
        assert _err(r[mode][0], ref) <= ABS_TOL
        assert _diff(r[mode][0], r["off"][0]) <= 1e-12
        assert r[mode][1]["krylov_builds"] == int(ref["n_builds"].sum())
        assert r[mode][1]["sample_steps"] == r["off"][1]["sample_steps"]


@pytest.mark.parametrize("rates", [(1.0, 1.0), (3.0, 0.5)])
def test_anisotropic_tilted_field(sampler, oracle, rates):
    """General builder (complex off-diagonal entries), tilted field; equal
    rates run Lanczos on the Hermitian part, unequal ones MGS on H_eff."""
    s = _anisotropic_small_pair(rates)
    B = np.array([0.02, -0.03, 0.04])
    rp, col, val = general_csr(oracle, s, B)
    zk = W.random_phase_samples(s.Z, 20, seed=3)
    t_end = 200 * DT
    ref = oracle.trace_sampling(rp, col, val, zk, DT, t_end, 16, 1e-5)

    def run():
        sampler.build_h(s, B, "general")
        return sampler.trace_sampling(zk, DT, t_end, 16, 1e-5)

    r = _both(sampler, run, "auto")
    for mode in MODES:
        assert _err(r[mode][0], ref) <= ABS_TOL
        assert _diff(r[mode][0], r["off"][0]) <= 1e-12


def test_uneven_batch(sampler, oracle):
    """Jobs of dims 48, 288 and 288 (another field) with their own samples
    in one launch."""
    systems = [W.notebook_pair(), W.small_pair(), W.small_pair()]
    fields = [0.2, 0.05, 0.3]
    for sy in systems:
        sy.kS = sy.kT = 1.0 / GAMMA_E
    Ms = [5, 30, 33]  # 68 samples: the two-CTA form on a 152-SM part
    zks = [W.random_phase_samples(sy.Z, M, seed=20 + i) for i, (sy, M) in enumerate(zip(systems, Ms))]
    t_end = 60 * DT

    def run():
        sampler.build_h_batch(systems, fields, "reference")
        return sampler.trace_sampling_batch(zks, DT, t_end, 14, 1e-6)

    r = _both(sampler, run, "auto")
    for i, (sy, f, zk) in enumerate(zip(systems, fields, zks)):
        rp, col, val = iso_csr(oracle, sy, f)
        ref = oracle.trace_sampling(rp, col, val, zk, DT, t_end, 14, 1e-6)
        for mode in MODES:
            assert _err(r[mode][0][i], ref) <= ABS_TOL
            assert _diff(r[mode][0][i], r["off"][0][i]) <= 1e-12


def test_exact_basis_and_lanczos_fallback(sampler, oracle):
    """The 48-dim pair over all basis states with m = 10: small invariant
    subspaces (exact breakdown) and Lanczos bases that lose orthogonality and
    are rebuilt with MGS inside the sample's CTA."""
    s = W.notebook_pair()
    rp, col, val = iso_csr(oracle, s, 0.2)
    dt = 0.5 * GAMMA_E / 1000
    t_end = 99.5 * GAMMA_E / 1000
    zk = np.eye(s.Z, dtype=complex)
    ref = oracle.trace_sampling(rp, col, val, zk, dt, t_end, 10, 1e-8)

    def run():
        sampler.build_h(s, 0.2, "reference")
        return sampler.trace_sampling(zk, dt, t_end, 10, 1e-8)

    r = _both(sampler, run, "lanczos")
    for mode in MODES:
        assert _err(r[mode][0], ref) <= ABS_TOL
        assert r[mode][1]["krylov_builds"] == int(ref["n_builds"].sum())
        assert r[mode][1]["lanczos_fallbacks"] > 0


@pytest.mark.parametrize("method", ["mgs", "lanczos"])
def test_one_build_over_many_steps(sampler, oracle, method):
    """tol = 1 never triggers a rebuild (|c_{m-1}|^2 <= |c|^2), so one Krylov
    basis serves all 150 dt steps: the two-CTA form's dt loop then runs in
    several history segments of at most 64 steps."""
    s = W.small_pair()
    rp, col, val = iso_csr(oracle, s, 0.05)
    zk = W.random_phase_samples(s.Z, 20, seed=9)
    t_end = 150 * DT
    ref = oracle.trace_sampling(rp, col, val, zk, DT, t_end, 20, 1.0)
    assert int(ref["n_builds"].sum()) == 20

    def run():
        sampler.set_h(rp, col, val)
        return sampler.trace_sampling(zk, DT, t_end, 20, 1.0)

    r = _both(sampler, run, method)
    for mode in MODES:
        assert _err(r[mode][0], ref) <= ABS_TOL
        assert _diff(r[mode][0], r["off"][0]) <= 1e-12
        assert r[mode][1]["krylov_builds"] == 20
        assert r[mode][1]["sample_steps"] == r["off"][1]["sample_steps"]


@pytest.mark.parametrize("mode", ["on", "single"])
def test_windows_shorter_than_dt_and_initial_states(sampler, oracle, mode):
    s = W.small_pair()
    rp, col, val = iso_csr(oracle, s, 0.05)
    zk = W.random_phase_samples(s.Z, 3, seed=5)
    sampler.set_sample_path(mode)
    try:
        sampler.set_h(rp, col, val)
        for t_end in (0.0, 0.05, DT):
            ref = oracle.trace_sampling(rp, col, val, zk, DT, t_end, 8, 1e-5)
            got = sampler.trace_sampling(zk, DT, t_end, 8, 1e-5)
            assert _err(got, ref) <= ABS_TOL
        for state in ("T0", "Tp", "Tm"):
            ref = oracle.trace_sampling(rp, col, val, zk, DT, 40 * DT, 12, 1e-6, init_state=state)
            got = sampler.trace_sampling(zk, DT, 40 * DT, 12, 1e-6, init_state=state)
            assert _err(got, ref) <= ABS_TOL
    finally:
        sampler.set_sample_path("auto")


def test_auto_mode_picks_by_size(sampler, oracle):
    """Auto mode: the dim-288 pair with 64 samples runs in one sample launch;
    the dim-55296 pair stays on the tiled path."""
    s = W.small_pair()
    rp, col, val = iso_csr(oracle, s, 0.05)
    sampler.set_h(rp, col, val)
    zk = W.random_phase_samples(s.Z, 64, seed=1)
    sampler.trace_sampling(zk, DT, 50 * DT, 20, 1e-5)
    st = sampler.stats()
    assert st["rounds"] == 1 and st["kernel_launches"] <= 4
    big, B = W.large_pair(isotropic=True)
    sampler.build_h(big, B[2], "reference")
    zk = W.random_phase_samples(big.Z, 2, seed=1)
    sampler.trace_sampling(zk, DT, 3 * DT, 8, 1e-5)
    assert sampler.stats()["kernel_launches"] > 10


@pytest.mark.parametrize("m", [1, 2])
@pytest.mark.parametrize("rates", [(1.0, 1.0), (2.0, 1.0)])
def test_pair_without_nuclei(sampler, oracle, m, rates):
    """Dimension 4 (no nuclei, one nuclear row), Krylov dimensions 1 and 2,
    Lanczos (equal rates) and MGS (unequal): both paths against the oracle."""
    from spin_dynamics_gb300.spinsys import Electron, SysParam

    s = SysParam.from_input_units(Electron(g_I=[], A=[]), Electron(g_I=[], A=[]), J=0.1,
                                  kS_per_us=rates[0], kT_per_us=rates[1])
    rp, col, val = iso_csr(oracle, s, 0.3)
    zk = np.ones((3, s.Z), complex)
    ref = oracle.trace_sampling(rp, col, val, zk, DT, 20 * DT, m, 1e-6)

    def run():
        sampler.set_h(rp, col, val)
        return sampler.trace_sampling(zk, DT, 20 * DT, m, 1e-6)

    r = _both(sampler, run, "auto")
    for mode in MODES:
        assert _err(r[mode][0], ref) <= ABS_TOL
        assert r[mode][1]["krylov_builds"] == int(ref["n_builds"].sum())


def test_mode_switch_errors(sampler):
    """The C ABI refuses unknown modes; the Python binding refuses unknown names."""
    from spin_dynamics_gb300 import _native as nat
    from spin_dynamics_gb300._native import SpcError

    with pytest.raises(SpcError, match="sample-path mode"):
        nat.check(nat.lib().spc_set_sample_path(sampler.handle, 7))
    with pytest.raises(KeyError):
        sampler.set_sample_path("sometimes")
    sampler.set_sample_path("auto")
