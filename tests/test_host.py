"""Host layer without a GPU: input.ini reading (keys, units, errors of
src/spinsys.f90), output files (src/observables.f90, app/main.f90 folder
names), yields, and the two-rank sample sharding over gloo."""
import os
import socket

import numpy as np
import pytest

from spin_dynamics_gb300 import Observables, SpinchemError, field_folder_name, fortran_list_directed
from spin_dynamics_gb300.observables import write_data
from spin_dynamics_gb300.parallel import shard
from spin_dynamics_gb300.spinsys import GAMMA_E, read_inp

INI = """[system variables]
J = 0.1
D = -0.2 0.0 0.0 0.0 -0.2 0.0 0.0 0.0 0.4
kS = 20.0
kT = 5.0
[electron 1]
g = 2.0023193
I = 2 3
N_I = 2 1
A1 = 0.5 0.0 0.0 0.0 0.5 0.0 0.0 0.0 0.5
A2 = 0.3 0.0 0.0 0.0 0.3 0.0 0.0 0.0 0.3
A3 = 1.0 0.1 0.2 0.0 1.0 0.0 0.0 0.0 1.0
[electron 2]
g = 2.0023193
[simulation parameters]
simulation_type = trace_sampling
output_folder = {out}
seed = 1436699015287340820  6992165104747523623
B = 0.0 0.2 25.0
initial_state = singlet
N_samples = 64
simulation_time = 50
dt = 0.5
N_krylov = 12
integrator_tolerance = 1e-06
"""


def write_ini(tmp_path, text):
    p = tmp_path / "input.ini"
    p.write_text(text)
    return str(p)


def test_read_inp_units_and_layout(tmp_path):
    sys_, sim = read_inp(write_ini(tmp_path, INI.format(out=tmp_path)))
    assert sys_.J == 0.1
    assert sys_.kS == pytest.approx(20.0 / GAMMA_E, rel=0, abs=0)
    assert sim.dt == (0.5 * GAMMA_E) / 1000.0 and sim.t_end == (50 * GAMMA_E) / 1000.0
    assert sys_.e1.g_I == [2, 2, 3] and sys_.e2.g_I == []
    assert sys_.Z1 == 12 and sys_.Z2 == 1 and sys_.N == 48
    # column-major reshape: A3 = (1.0 0.1 0.2 | 0 1 0 | 0 0 1) -> A(2,1) = 0.1
    assert sys_.e1.A[2][1, 0] == 0.1 and sys_.e1.A[2][0, 1] == 0.0
    assert sys_.e1.a_iso[2] == pytest.approx(1.0)
    assert sys_.D[2, 2] == 0.4 and sys_.D[0, 0] == -0.2
    assert sim.seed == (1436699015287340820, 6992165104747523623)
    assert sim.B == [0.0, 0.2, 25.0] and sim.N_samples == 64 and sim.N_krylov == 12
    assert sim.tol == 1e-6 and sim.init_state == "singlet" and not sim.isRestart
    assert sys_.e1.isotropic and sys_.e2.isotropic


@pytest.mark.parametrize("mutate,msg", [
    (lambda s: s.replace("[electron 2]\ng = 2.0023193\n", ""), "less than expected"),
    (lambda s: s + "[extra]\nx = 1\n", "more than expected"),
    (lambda s: s.replace("J = 0.1\n", ""), "Exchange coupling is missing"),
    (lambda s: s.replace("A2 = 0.3 0.0 0.0 0.0 0.3 0.0 0.0 0.0 0.3\n", ""), "Hyperfine copuling A2"),
    (lambda s: s.replace("N_I = 2 1", "N_I = 2"), "must have the sam length"),
    (lambda s: s.replace("dt = 0.5\n", ""), "Propagation timestep is missing"),
])
def test_read_inp_errors(tmp_path, mutate, msg):
    with pytest.raises(SpinchemError) as ei:
        read_inp(write_ini(tmp_path, mutate(INI.format(out=tmp_path))))
    assert msg in str(ei.value)


def test_missing_output_folder_and_input(tmp_path):
    with pytest.raises(SpinchemError, match="Output folder does not exist"):
        read_inp(write_ini(tmp_path, INI.format(out=tmp_path / "nope")))
    with pytest.raises(SpinchemError, match="Input file does not exist"):
        read_inp(str(tmp_path / "absent.ini"))


def test_anisotropy_flag_follows_the_reference_check(tmp_path):
    text = INI.format(out=tmp_path).replace("A1 = 0.5 0.0 0.0 0.0 0.5", "A1 = 0.5 0.0 0.0 0.0 0.6")
    sys_, _ = read_inp(write_ini(tmp_path, text))
    assert not sys_.e1.isotropic  # A(1,1) /= A(2,2)


def test_list_directed_format():
    assert fortran_list_directed(1.0) == "   1.0000000000000000     "
    assert fortran_list_directed(0.5) == "  0.50000000000000000     "
    assert fortran_list_directed(-1.0) == "  -1.0000000000000000     "
    assert fortran_list_directed(0.0) == "   0.0000000000000000     "
    assert fortran_list_directed(1e-2) == "   1.0000000000000000E-002"
    assert fortran_list_directed(123.456) == "   123.45600000000000     "
    for v in (0.998726, 3.2e-7, 0.1, 12345.678):
        assert float(fortran_list_directed(v).replace("E", "e")) == pytest.approx(v, rel=1e-16)


def test_field_folder_names():
    assert field_folder_name(0.0) == ".000"
    assert field_folder_name(0.2) == ".200"
    assert field_folder_name(25.0) == "25.000"
    assert field_folder_name(1.5) == "1.500"
    assert field_folder_name(-0.05) == "-.050"


def test_output_files_and_parse_back(tmp_path, oracle):
    rng = np.random.default_rng(1)
    obs = Observables(*(rng.random(11) for _ in range(4)))
    obs.output(str(tmp_path))
    for name in ("S_prob.data", "Tp_prob.data", "T0_prob.data", "Tm_prob.data"):
        assert np.allclose(np.loadtxt(tmp_path / name), getattr(obs, {"S": "P_S", "Tp": "P_Tp", "T0": "P_T0", "Tm": "P_Tm"}[name.split("_")[0]]), rtol=1e-16)
    assert not (tmp_path / "S_yield.data").exists()
    obs.get_kinetics(0.17, 0.005, 0.002)
    ph, pt, iden = oracle.kinetics(obs.P_S, obs.P_T0, obs.P_Tp, obs.P_Tm, 0.17, 0.005, 0.002)
    assert np.array_equal(obs.Phi_S, ph) and np.array_equal(obs.Phi_T, pt) and np.array_equal(obs.iden, iden)
    obs.output(str(tmp_path))
    assert np.allclose(np.loadtxt(tmp_path / "S_yield.data"), ph, rtol=1e-16)
    write_data([1.0, 2.0], str(tmp_path), "x.data")
    assert (tmp_path / "x.data").read_text().splitlines()[1] == "   2.0000000000000000     "


def test_shards_cover_every_sample_once():
    for M in (1, 7, 64, 513):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                s = shard(M, r, world)
                seen += list(range(M))[s]
            assert seen == list(range(M))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, result_path):
    import sys
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    sys.path.insert(0, os.path.join(root, "oracle"))
    import pyoracle
    from spin_dynamics_gb300 import workloads as W
    from spin_dynamics_gb300.parallel import trace_sampling_sharded
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sysp, sim = W.small_pair(), W.small_sim(M=10, t_end_ns=120.0)
    e1, e2 = sysp.e1, sysp.e2
    rp, col, val = pyoracle.build_h_iso(e1.g_I, e1.a_iso, e2.g_I, e2.a_iso, 0.05, sysp.J, sysp.D, sysp.kS, sysp.kT)

    def propagate(zk):
        r = pyoracle.trace_sampling(rp, col, val, zk, sim.dt, sim.t_end, 12, sim.tol)
        return Observables(r["P_S"], r["P_T0"], r["P_Tp"], r["P_Tm"])

    zk = W.random_phase_samples(sysp.Z, 10)
    res = trace_sampling_sharded(propagate, zk)
    if rank == 0:
        np.save(result_path, np.stack([res.P_S, res.P_T0, res.P_Tp, res.P_Tm]))
    dist.destroy_process_group()


def test_two_rank_sharding_matches_single_process(tmp_path, oracle):
    import torch.multiprocessing as mp
    from spin_dynamics_gb300 import workloads as W
    out = str(tmp_path / "res.npy")
    mp.spawn(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True)
    sysp, sim = W.small_pair(), W.small_sim(M=10, t_end_ns=120.0)
    e1, e2 = sysp.e1, sysp.e2
    rp, col, val = oracle.build_h_iso(e1.g_I, e1.a_iso, e2.g_I, e2.a_iso, 0.05, sysp.J, sysp.D, sysp.kS, sysp.kT)
    ref = oracle.trace_sampling(rp, col, val, W.random_phase_samples(sysp.Z, 10), sim.dt, sim.t_end, 12, sim.tol)
    got = np.load(out)
    for i, k in enumerate(("P_S", "P_T0", "P_Tp", "P_Tm")):
        assert np.max(np.abs(got[i] - ref[k])) < 1e-14


def test_batch_marshalling_converts_each_system_once_and_keeps_fields():
    import ctypes as C
    from spin_dynamics_gb300 import workloads as W
    from spin_dynamics_gb300.dynamics import make_system, make_systems
    a, b = W.small_pair(), W.notebook_pair()
    systems = [a, a, b, a]
    fields = [0.05, np.array([0.01, 0.02, 0.03]), 0.1, np.array([0.0, 0.0, -0.2])]
    arr, keep = make_systems(systems, fields)
    assert len(keep[0]) == 2  # one template per distinct system object
    for st, sy, f in zip(arr, systems, fields):
        ref, _ = make_system(sy, f)
        for name, _t in ref._fields_:
            x, y = getattr(st, name), getattr(ref, name)
            if name in ("mult1", "mult2", "A1", "A2", "gamma1", "gamma2"):
                n = 9 * (ref.n_nuc1 if name == "A1" else ref.n_nuc2) if name in ("A1", "A2") else \
                    (ref.n_nuc1 if name.endswith("1") else ref.n_nuc2)
                if bool(x) != bool(y):
                    raise AssertionError(name)
                if x:
                    assert [x[i] for i in range(n)] == [y[i] for i in range(n)], name
            elif name in ("B", "D"):
                assert list(x) == list(y), name
            else:
                assert x == y, name


def test_torch_parameter_vector_round_trip():
    torch = pytest.importorskip("torch")
    from spin_dynamics_gb300 import workloads as W
    from spin_dynamics_gb300.torch_ops import pack_params, unpack_params
    s, B = W.large_pair()
    v = pack_params(s, B)
    assert v.dtype == torch.float64 and v.numel() == 15 + 9 * 12
    s2, B2 = unpack_params(s, v.numpy())
    assert np.array_equal(B2, B)
    for a1, a2 in zip(s.e1.A + s.e2.A, s2.e1.A + s2.e2.A):
        assert np.array_equal(np.asarray(a1), a2)
    assert np.array_equal(np.asarray(s.D), s2.D) and s2.J == s.J and s2.kS == s.kS
    with pytest.raises(ValueError):
        unpack_params(s, v.numpy()[:-1])
