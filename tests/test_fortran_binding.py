"""The Fortran drop-in of INTEGRATION.md, checked without a Fortran compiler.

* Every `bind(C)` interface shown there names a function the header declares,
  with as many dummy arguments as the C prototype has parameters and no two
  dummies that Fortran (case-insensitive) would take for the same name.
* The replacement body of trace_sampling_para (src/qm_dynamics.f90:257-384)
  is replayed through ctypes with the argument types the interfaces give:
  the master seed sim%seed (integer(i8), src/spinsys.f90:44) as read from an
  input.ini -> spc_seeded_samples -> spc_build_h -> spc_trace_sampling. The
  vectors must be the reference's per-sample stream (two next() per sample of
  the generator main seeds with set_seed, src/qm_dynamics.f90:315-327) bit
  for bit, and the populations the oracle's on them."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT, gpu_available
from spin_dynamics_gb300 import _native as nat
from spin_dynamics_gb300.spinsys import read_inp

DOC = os.path.join(ROOT, "INTEGRATION.md")
HEADER = os.path.join(ROOT, "include", "spinchem_gpu.h")

INI = """[system variables]
J = 0.0
D = 0.0 0.0 0.0 0.0 0.0 0.0 0.0 0.0 0.0
kS = 1.0
kT = 1.0
[electron 1]
g = 2.0023193
I = 2 3
N_I = 2 1
A1 = 0.5 0.0 0.0 0.0 0.5 0.0 0.0 0.0 0.5
A2 = 0.3 0.0 0.0 0.0 0.3 0.0 0.0 0.0 0.3
A3 = 1.0 0.0 0.0 0.0 1.0 0.0 0.0 0.0 1.0
[electron 2]
g = 2.0023193
I = 2 3
N_I = 1 1
A1 = 0.8 0.0 0.0 0.0 0.8 0.0 0.0 0.0 0.8
A2 = 0.2 0.0 0.0 0.0 0.2 0.0 0.0 0.0 0.2
[simulation parameters]
simulation_type = trace_sampling
output_folder = {out}
seed = 1436699015287340820  6992165104747523623
B = 0.05
initial_state = singlet
N_samples = 12
simulation_time = 100
dt = 1.0
N_krylov = 16
integrator_tolerance = 1e-05
"""


def fortran_interfaces():
    """(Fortran name, dummy arguments, bound C name) of every interface
    function in the document's fortran code blocks."""
    text = open(DOC).read()
    out = []
    for block in re.findall(r"```fortran\n(.*?)```", text, flags=re.S):
        # free-form continuation: a line ending in '&' continues on the next
        joined = re.sub(r"&\s*\n\s*&?", " ", block)
        for name, args, cname in re.findall(
                r"function\s+(\w+)\s*\(([^)]*)\)\s*bind\(C,\s*name=\"(\w+)\"\)", joined):
            out.append((name, [a.strip() for a in args.split(",") if a.strip()], cname))
    return out


def c_prototypes():
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    src = re.sub(r"\s+", " ", src)
    return {n: [p for p in params.split(",") if p.strip() and p.strip() != "void"]
            for n, params in re.findall(r"\bint (spc_\w+)\s*\(([^)]*)\)\s*;", src)}


def test_fortran_interfaces_match_the_header():
    ifs = fortran_interfaces()
    protos = c_prototypes()
    assert len(ifs) >= 8
    for name, args, cname in ifs:
        assert cname in protos, f"{cname} is bound in INTEGRATION.md but not declared in the header"
        assert len(args) == len(protos[cname]), f"{name}: {len(args)} dummies, C has {len(protos[cname])}"
        lower = [a.lower() for a in args]
        assert len(set(lower)) == len(lower), f"{name}: dummy names collide case-insensitively: {args}"


def test_replacement_body_passes_the_master_seed():
    text = open(DOC).read()
    # first two actual arguments of the call in the replacement body
    calls = re.findall(r"ierr = spc_seeded_samples\(\s*([^,]+),\s*([^,]+),", text.split("## 2.")[0])
    assert calls == [("sim%seed(1)", "sim%seed(2)")], calls


def _binding_samples(oracle, tmp_path):
    ini = tmp_path / "input.ini"
    ini.write_text(INI.format(out=tmp_path))
    sys_, sim = read_inp(str(ini))
    Z = sys_.Z
    zk = np.empty((sim.N_samples, Z), dtype=np.complex128)
    # integer(c_int64_t), value :: s0, s1 -- the two i8 words of sim%seed
    s0 = C.c_int64(int(np.int64(np.uint64(sim.seed[0] & (2**64 - 1)))))
    s1 = C.c_int64(int(np.int64(np.uint64(sim.seed[1] & (2**64 - 1)))))
    nat.check(nat.lib().spc_seeded_samples(s0, s1, Z, sim.N_samples, 0, zk.ctypes.data_as(C.c_void_p)))
    return sys_, sim, zk


def test_binding_sequence_draws_the_reference_stream(oracle, tmp_path):
    sys_, sim, zk = _binding_samples(oracle, tmp_path)
    ref = oracle.seeded_samples(sim.seed, sys_.Z, sim.N_samples, mode=0)
    assert np.array_equal(zk, ref)
    assert np.allclose(np.linalg.norm(zk, axis=1), 1.0, atol=1e-14)


@pytest.mark.gpu
def test_binding_sequence_propagates_like_the_oracle(oracle, tmp_path):
    if not gpu_available():
        pytest.skip("no GPU")
    from spin_dynamics_gb300.dynamics import make_system

    sys_, sim, zk = _binding_samples(oracle, tmp_path)
    B = sim.B[0]
    sys_.e1.w = sys_.e2.w = -B
    L = nat.lib()
    h = C.c_void_p()
    nat.check(L.spc_create(0, C.byref(h)))
    try:
        st, keep = make_system(sys_, B)
        nat.check(L.spc_build_h(h, C.byref(st), nat.SPC_H_REFERENCE))
        theta = np.zeros(8)
        pop = np.zeros(4)
        nat.check(L.spc_init_el_state(0, theta.ctypes.data_as(C.c_void_p), pop.ctypes.data_as(C.c_void_p)))
        T = L.spc_num_time_points(sim.dt, sim.t_end)
        P = [np.zeros(T) for _ in range(4)]
        ptr = lambda a: a.ctypes.data_as(C.c_void_p)
        nat.check(L.spc_trace_sampling(h, ptr(theta), ptr(pop), ptr(zk), sim.N_samples, sim.dt, sim.t_end,
                                       sim.N_krylov, sim.tol, *(ptr(p) for p in P), T))
    finally:
        L.spc_destroy(h)
    e1, e2 = sys_.e1, sys_.e2
    rp, col, val = oracle.build_h_iso(e1.g_I, e1.a_iso, e2.g_I, e2.a_iso, B, sys_.J, sys_.D, sys_.kS, sys_.kT)
    ref = oracle.trace_sampling(rp, col, val, zk, sim.dt, sim.t_end, sim.N_krylov, sim.tol)
    for got, key in zip(P, ("P_S", "P_T0", "P_Tp", "P_Tm")):
        assert np.max(np.abs(got - ref[key])) <= 1e-10, key
