"""The field loop and the symmetry-block resume of the drivers, on the CPU with
a deterministic stand-in for the GPU propagation (no GPU needed):

* every field of sim.B goes through one batched build + propagation
  (app/main.f90:48-79 loops them one by one);
* symmetry_dynamics writes each block's populations to
  <field folder>/hamiltonian_<i>/ as its batch finishes, and a restart reads
  the blocks before sim.restart back from there. A run stopped after some
  batches, resumed from its first unfinished block, writes files
  byte-identical to those of an uninterrupted run (src/symmetry.f90:81-87,
  129-131 leave those blocks unallocated instead)."""
import filecmp
import hashlib
import os

import numpy as np
import pytest

from spin_dynamics_gb300 import dynamics
from spin_dynamics_gb300 import symmetry as S
from spin_dynamics_gb300.observables import Observables, field_folder_name
from spin_dynamics_gb300.spinsys import GAMMA_E, Electron, SimParam, SpinchemError, SysParam


class Stopped(Exception):
    pass


class FakeSampler:
    """build_h_batch / trace_sampling_batch with populations that depend only
    on each job (its system, field and first sample), like the real ones;
    `stop_after` batches, then raises (a run killed mid-way)."""

    def __init__(self, stop_after=None):
        self.stop_after = stop_after
        self.batches = []

    def build_h_batch(self, systems, fields, mode="reference"):
        self.cur = list(zip(systems, fields))
        return [4 * s.Z for s in systems]

    def trace_sampling_batch(self, zks, dt, t_end, m, tol, init_state="singlet"):
        if self.stop_after is not None and len(self.batches) >= self.stop_after:
            raise Stopped()
        self.batches.append(len(zks))
        self.zks = list(zks)
        T = dynamics.num_time_points(dt, t_end)
        out = []
        for (s, f), z in zip(self.cur, zks):
            key = repr((s.Z, s.e1.g_I, s.e2.g_I, np.round(np.asarray(f, float), 12).tolist(),
                        complex(z[0, 0]), z.shape)).encode()
            rng = np.random.default_rng(int.from_bytes(hashlib.sha256(key).digest()[:8], "little"))
            out.append(Observables(*(rng.random(T) * 1e-3 ** rng.integers(0, 3) for _ in range(4))))
        return out


def equivalent_system():
    e1 = Electron(g_I=[2, 2, 2, 3], A=[np.eye(3) * 0.5] * 3 + [np.eye(3) * 0.3])
    e2 = Electron(g_I=[2, 2], A=[np.eye(3) * 0.4] * 2)
    return SysParam(e1=e1, e2=e2, J=0.05, kS=1.0 / GAMMA_E, kT=1.0 / GAMMA_E)


def sim_params(restart=None, fields=(0.1, 0.25)):
    sim = SimParam.from_input_units(type="symmetry_dynamics", B=list(fields), init_state="singlet",
                                    seed=(42, 99), N_samples=5, t_end_ns=20.0, dt_ns=1.0, N_krylov=6,
                                    tol=1e-5, M1=1, M2=1, block_tol=0.0)
    sim.restart = restart
    return sim


def run(tmp, sampler, sim):
    folders = []
    for B in sim.B:
        folders.append(os.path.join(tmp, field_folder_name(B)))
        os.makedirs(folders[-1], exist_ok=True)
    return S.symmetrised_fields(equivalent_system(), sim, list(sim.B), folders, sampler), folders


@pytest.fixture
def one_job_per_batch(monkeypatch):
    # a budget of one block per batch: every (block, field) job its own batch
    monkeypatch.setattr(S, "_budget_entries", lambda states: 1.0)


def test_resumed_run_writes_the_uninterrupted_files(tmp_path, one_job_per_batch):
    full, fa = run(str(tmp_path / "a"), FakeSampler(), sim_params())
    n_blocks = len(S.blocks(equivalent_system(), 1, 1))
    assert n_blocks == 4
    # stopped after the first 5 batches: blocks 1, 2 done for both fields,
    # block 3 for the first field only
    with pytest.raises(Stopped):
        run(str(tmp_path / "b"), FakeSampler(stop_after=5), sim_params())
    fb = [os.path.join(str(tmp_path / "b"), field_folder_name(B)) for B in (0.1, 0.25)]
    assert os.path.isdir(os.path.join(fb[0], "hamiltonian_3"))
    assert not os.path.isdir(os.path.join(fb[1], "hamiltonian_3"))
    resumed_sampler = FakeSampler()
    resumed, _ = run(str(tmp_path / "b"), resumed_sampler, sim_params(restart=3))
    assert sum(resumed_sampler.batches) == 2 * 2  # blocks 3 and 4, both fields
    for a, b in zip(fa, fb):
        names = sorted(os.listdir(a))
        assert names == sorted(os.listdir(b))
        for n in names:
            if os.path.isfile(os.path.join(a, n)):
                assert filecmp.cmp(os.path.join(a, n), os.path.join(b, n), shallow=False), n
        for i in range(1, n_blocks + 1):
            for n in ("S_prob.data", "T0_prob.data", "Tp_prob.data", "Tm_prob.data"):
                assert filecmp.cmp(os.path.join(a, f"hamiltonian_{i}", n), os.path.join(b, f"hamiltonian_{i}", n),
                                   shallow=False)
    for x, y in zip(full, resumed):
        assert np.array_equal(x.P_S, y.P_S) and np.array_equal(x.Phi_S, y.Phi_S)


def test_reloaded_blocks_are_the_same_doubles(tmp_path):
    T = 9
    rng = np.random.default_rng(5)
    vals = [rng.random(T) * 10.0 ** rng.integers(-12, 3, T) for _ in range(4)]
    vals[0][0] = 0.0
    o = Observables(*[v.copy() for v in vals])
    os.makedirs(S.block_folder(str(tmp_path), 2))
    o.output(S.block_folder(str(tmp_path), 2))
    r = S.read_block(str(tmp_path), 2, T)
    for a, b in zip(vals, (r.P_S, r.P_T0, r.P_Tp, r.P_Tm)):
        assert np.array_equal(a, b)


def test_restart_without_saved_blocks_is_an_error(tmp_path, one_job_per_batch):
    with pytest.raises(SpinchemError, match="restart"):
        run(str(tmp_path), FakeSampler(), sim_params(restart=2))
    with pytest.raises(SpinchemError, match="restart"):
        S.symmetrised_fields(equivalent_system(), sim_params(restart=2), [0.1], None, FakeSampler())


def test_fields_share_one_batch(tmp_path, monkeypatch):
    monkeypatch.setattr(dynamics, "device_memory", lambda device=0: (80 << 30, 100 << 30))
    s = SysParam(e1=Electron(g_I=[2, 3], A=[np.eye(3) * 0.5, np.eye(3) * 0.3]),
                 e2=Electron(g_I=[2], A=[np.eye(3) * 0.4]), kS=1.0 / GAMMA_E, kT=1.0 / GAMMA_E)
    sim = SimParam.from_input_units(type="trace_sampling", B=[0.0, 0.05, 0.2], init_state="singlet",
                                    seed=(42, 99), N_samples=7, t_end_ns=10.0, dt_ns=1.0, N_krylov=6, tol=1e-5)
    sp = FakeSampler()
    folders = [str(tmp_path / field_folder_name(B)) for B in sim.B]
    for f in folders:
        os.makedirs(f)
    res = dynamics.field_dynamics(s, sim, folders, sp)
    assert sp.batches == [3]  # one propagation for the three fields
    assert len(res) == 3 and all(os.path.exists(os.path.join(f, "S_prob.data")) for f in folders)
    # every field propagates the same vectors (the generator is re-seeded per
    # field): the trace_sampling_para stream of sim.seed
    ref = dynamics.seeded_samples(sim.seed, s.Z, sim.N_samples)
    assert all(np.array_equal(z, ref) for z in sp.zks)
    assert [f for _, f in sp.cur] == [0.0, 0.05, 0.2]
