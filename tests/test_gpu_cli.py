"""The two drop-in drivers (C++ `spinchem` and `python -m spin_dynamics_gb300`)
on an input.ini: same folders and files as the reference, populations equal
to the oracle's on the reference's own sample stream within 1e-10."""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT
from spin_dynamics_gb300.spinsys import read_inp

pytestmark = pytest.mark.gpu

INI = """[system variables]
J = 0.1
D = 0.0 0.0 0.0 0.0 0.0 0.0 0.0 0.0 0.0
kS = 2.0
kT = 2.0
[electron 1]
g = 2.0023193
I = 2 3
N_I = 1 1
A1 = 0.5 0.0 0.0 0.0 0.5 0.0 0.0 0.0 0.5
A2 = 0.3 0.0 0.0 0.0 0.3 0.0 0.0 0.0 0.3
[electron 2]
g = 2.0023193
I = 2
N_I = 1
A1 = 0.4 0.0 0.0 0.0 0.4 0.0 0.0 0.0 0.4
[simulation parameters]
simulation_type = {kind}
output_folder = {out}
seed = 42 99
B = 0.0 0.2
initial_state = singlet
N_samples = 12
simulation_time = 60
dt = 0.5
N_krylov = 10
integrator_tolerance = 1e-08
"""


def run_cli(cmd, tmp_path, kind):
    out = tmp_path / "out"
    out.mkdir()
    ini = tmp_path / "input.ini"
    ini.write_text(INI.format(kind=kind, out=out))
    r = subprocess.run(cmd + [str(ini)], capture_output=True, text=True, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    return str(ini), out


def expected(oracle, ini, B):
    sys_, sim = read_inp(ini)
    e1, e2 = sys_.e1, sys_.e2
    rp, col, val = oracle.build_h_iso(e1.g_I, e1.a_iso, e2.g_I, e2.a_iso, B, sys_.J, sys_.D,
                                      sys_.kS, sys_.kT)
    if sim.type == "exact_dynamics":
        zk = np.eye(sys_.Z, dtype=complex)
    else:
        zk = oracle.seeded_samples(sim.seed, sys_.Z, sim.N_samples,
                                   mode=1 if sim.type == "trace_sampling_serial" else 0)
    return oracle.trace_sampling(rp, col, val, zk, sim.dt, sim.t_end, sim.N_krylov, sim.tol)


@pytest.mark.parametrize("driver", ["cpp", "python"])
@pytest.mark.parametrize("kind", ["trace_sampling", "trace_sampling_serial", "exact_dynamics"])
def test_driver_output_files(tmp_path, oracle, driver, kind):
    cmd = ([os.path.join(ROOT, "spin_dynamics_gb300", "_build", "spinchem")] if driver == "cpp"
           else [sys.executable, "-m", "spin_dynamics_gb300"])
    ini, out = run_cli(cmd, tmp_path, kind)
    assert sorted(os.listdir(out)) == [".000", ".200"]
    for B, sub in ((0.0, ".000"), (0.2, ".200")):
        ref = expected(oracle, ini, B)
        assert sorted(os.listdir(out / sub)) == ["S_prob.data", "T0_prob.data", "Tm_prob.data", "Tp_prob.data"]
        for fname, key in (("S_prob.data", "P_S"), ("T0_prob.data", "P_T0"), ("Tp_prob.data", "P_Tp"),
                           ("Tm_prob.data", "P_Tm")):
            got = np.loadtxt(out / sub / fname)
            assert got.shape == ref[key].shape
            assert np.max(np.abs(got - ref[key])) <= 1e-10


def test_cpp_and_python_writers_agree_byte_for_byte(tmp_path):
    a = tmp_path / "a"
    b = tmp_path / "b"
    a.mkdir()
    b.mkdir()
    _, out_a = run_cli([os.path.join(ROOT, "spin_dynamics_gb300", "_build", "spinchem")], a, "exact_dynamics")
    _, out_b = run_cli([sys.executable, "-m", "spin_dynamics_gb300"], b, "exact_dynamics")
    for f in ("S_prob.data", "Tm_prob.data"):
        assert (out_a / ".200" / f).read_text() == (out_b / ".200" / f).read_text()


def test_driver_errors(tmp_path):
    out = tmp_path / "out"
    out.mkdir()
    ini = tmp_path / "input.ini"
    ini.write_text(INI.format(kind="trace_sampling", out=out).replace("A1 = 0.5 0.0 0.0 0.0 0.5",
                                                                      "A1 = 0.5 0.0 0.0 0.0 0.6"))
    for cmd in ([os.path.join(ROOT, "spin_dynamics_gb300", "_build", "spinchem")],
                [sys.executable, "-m", "spin_dynamics_gb300"]):
        r = subprocess.run(cmd + [str(ini)], capture_output=True, text=True, cwd=ROOT)
        assert r.returncode == 1 and "Anisotropic Hamiltoninans" in r.stderr


SYM_INI = """[system variables]
J = 0.05
D = 0.0 0.0 0.0 0.0 0.0 0.0 0.0 0.0 0.0
kS = 1.0
kT = 1.0
[electron 1]
g = 2.0023193
I = 2 3
N_I = 3 1
A1 = 0.5 0.0 0.0 0.0 0.5 0.0 0.0 0.0 0.5
A2 = 0.5 0.0 0.0 0.0 0.5 0.0 0.0 0.0 0.5
A3 = {a3} 0.0 0.0 0.0 {a3} 0.0 0.0 0.0 {a3}
A4 = 0.3 0.0 0.0 0.0 0.3 0.0 0.0 0.0 0.3
[electron 2]
g = 2.0023193
I = 2
N_I = 2
A1 = 0.4 0.0 0.0 0.0 0.4 0.0 0.0 0.0 0.4
A2 = 0.4 0.0 0.0 0.0 0.4 0.0 0.0 0.0 0.4
[simulation parameters]
simulation_type = symmetry_dynamics
output_folder = {out}
seed = 42 99
B = 0.1
initial_state = singlet
N_samples = 6
simulation_time = 40
dt = 1.0
N_krylov = 12
integrator_tolerance = 1e-10
M1 = 1
M2 = 1
block_tolerance = 0.0
"""


@pytest.mark.parametrize("case", ["exact_groups", "moment_matched"])
def test_symmetry_dynamics_in_both_drivers(tmp_path, case):
    """symmetry_dynamics through the C++ executable and the Python twin: the
    same seven files; byte-identical when the groups are exact (three equal
    1H couplings), within 1e-12 when the couplings (0.5, 0.5, 0.3) are
    moment-matched to one group."""
    a3 = "0.5" if case == "exact_groups" else "0.3"
    outs = []
    for name, cmd in (("cpp", [os.path.join(ROOT, "spin_dynamics_gb300", "_build", "spinchem")]),
                      ("py", [sys.executable, "-m", "spin_dynamics_gb300"])):
        d = tmp_path / name
        d.mkdir()
        out = d / "out"
        out.mkdir()
        ini = d / "input.ini"
        ini.write_text(SYM_INI.format(a3=a3, out=out))
        r = subprocess.run(cmd + [str(ini)], capture_output=True, text=True, cwd=ROOT)
        assert r.returncode == 0, r.stderr
        outs.append(out / ".100")
    files = sorted(f for f in os.listdir(outs[0]) if os.path.isfile(outs[0] / f))
    assert files == sorted(f for f in os.listdir(outs[1]) if os.path.isfile(outs[1] / f)) == sorted(
        ["S_prob.data", "T0_prob.data", "Tm_prob.data", "Tp_prob.data", "total_prob.data", "S_yield.data",
         "T_yield.data"])
    # every block's populations beside them, for a restart
    assert sorted(d for d in os.listdir(outs[0]) if d.startswith("hamiltonian_")) == [
        f"hamiltonian_{i}" for i in range(1, 5)]
    for f in files:
        if case == "exact_groups":
            assert (outs[0] / f).read_text() == (outs[1] / f).read_text(), f
        else:
            assert np.max(np.abs(np.loadtxt(outs[0] / f) - np.loadtxt(outs[1] / f))) <= 1e-12, f
    ps = np.loadtxt(outs[0] / "S_prob.data")
    assert abs(ps[0] - 1.0) < 1e-12  # the block weights sum to one


def test_symmetry_restart_reloads_the_saved_blocks(tmp_path):
    """Two fields; the first run keeps every block's populations under
    <field>/hamiltonian_<i>/. A second run given only blocks 1-2 of it and
    restart = 3 propagates blocks 3-4 and reads 1-2 back: its files equal the
    full run's (to the rounding of a batch of another composition), and the
    two drivers' resumed files are byte-identical."""
    import shutil
    ini_txt = SYM_INI.replace("B = 0.1", "B = 0.1 0.3")
    full = tmp_path / "full"
    full.mkdir()
    (tmp_path / "full.ini").write_text(ini_txt.format(a3="0.5", out=full))
    exe = os.path.join(ROOT, "spin_dynamics_gb300", "_build", "spinchem")
    r = subprocess.run([exe, str(tmp_path / "full.ini")], capture_output=True, text=True, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    resumed = []
    for name, cmd in (("cpp", [exe]), ("py", [sys.executable, "-m", "spin_dynamics_gb300"])):
        out = tmp_path / name
        for fld in (".100", ".300"):
            for i in (1, 2):
                shutil.copytree(full / fld / f"hamiltonian_{i}", out / fld / f"hamiltonian_{i}")
        (tmp_path / f"{name}.ini").write_text(ini_txt.format(a3="0.5", out=out) + "restart = 3\n")
        r = subprocess.run(cmd + [str(tmp_path / f"{name}.ini")], capture_output=True, text=True, cwd=ROOT)
        assert r.returncode == 0, r.stderr
        resumed.append(out)
    for fld in (".100", ".300"):
        for f in ("S_prob.data", "T0_prob.data", "Tp_prob.data", "Tm_prob.data", "S_yield.data"):
            a = np.loadtxt(full / fld / f)
            assert np.max(np.abs(np.loadtxt(resumed[0] / fld / f) - a)) <= 1e-13, (fld, f)
            assert (resumed[0] / fld / f).read_text() == (resumed[1] / fld / f).read_text(), (fld, f)
    # without the saved blocks the restart is refused
    bare = tmp_path / "bare"
    bare.mkdir()
    (tmp_path / "bare.ini").write_text(ini_txt.format(a3="0.5", out=bare) + "restart = 3\n")
    r = subprocess.run([exe, str(tmp_path / "bare.ini")], capture_output=True, text=True, cwd=ROOT)
    assert r.returncode == 1 and "restart" in r.stderr
