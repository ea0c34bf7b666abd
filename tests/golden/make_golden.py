"""Generates tests/golden/oracle_golden.npz from the CPU oracle (parity build).

The reference itself cannot be built here (Fortran toolchain and its stdlib
dependency are absent), so these vectors are the oracle's outputs on fixed
inputs. They pin the oracle across machines (x86-64 here, aarch64 on the GPU
hosts) and across edits: tests/test_golden.py recomputes them.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import pyoracle  # noqa: E402

from spin_dynamics_gb300 import workloads as W  # noqa: E402
from spin_dynamics_gb300.spinsys import GAMMA_E  # noqa: E402


def cases(po):
    out = {}
    out["rng_next_42_99"] = po.rng_stream((42, 99), 16)
    out["rng_normals_42_99"] = po.rng_normals((42, 99), 16)
    out["samples_para_Z12_M3"] = po.seeded_samples((42, 99), 12, 3, mode=0)
    out["samples_serial_Z12_M3"] = po.seeded_samples((42, 99), 12, 3, mode=1)
    nb = W.notebook_pair()
    rp, col, val = po.build_h_iso(nb.e1.g_I, nb.e1.a_iso, nb.e2.g_I, nb.e2.a_iso, 0.2, nb.J, nb.D,
                                  nb.kS, nb.kT)
    out["h_notebook_rowptr"], out["h_notebook_col"], out["h_notebook_val"] = rp, col, val
    dt = 0.5 * GAMMA_E / 1000
    r = po.trace_sampling(rp, col, val, np.eye(nb.Z, dtype=complex), dt, 99.5 * GAMMA_E / 1000, 10,
                          1e-8)
    for k in ("P_S", "P_T0", "P_Tp", "P_Tm"):
        out["ts_notebook_" + k] = r[k]
    sp_ = W.small_pair()
    rng = np.random.default_rng(17)
    A1 = [a + (lambda x: x + x.T)(rng.normal(size=(3, 3)) * 0.2) for a in sp_.e1.A]
    A2 = [a + (lambda x: x + x.T)(rng.normal(size=(3, 3)) * 0.2) for a in sp_.e2.A]
    rp, col, val = po.build_h_general(sp_.e1.g_I, A1, sp_.e1.gammas, sp_.e2.g_I, A2, sp_.e2.gammas,
                                      [0.02, -0.01, 0.04], 0.01, W.axial_dipolar(-0.4), sp_.kS, sp_.kT)
    out["h_small_general_rowptr"], out["h_small_general_col"], out["h_small_general_val"] = rp, col, val
    rp, col, val = po.build_h_iso(sp_.e1.g_I, sp_.e1.a_iso, sp_.e2.g_I, sp_.e2.a_iso, 0.05, sp_.J,
                                  sp_.D, sp_.kS, sp_.kT)
    zk = po.seeded_samples((42, 99), sp_.Z, 8)
    dt = 1.0 * GAMMA_E / 1000
    r = po.trace_sampling(rp, col, val, zk, dt, 300 * dt, 20, 1e-5)
    for k in ("P_S", "P_T0", "P_Tp", "P_Tm"):
        out["ts_small_" + k] = r[k]
    out["ts_small_n_builds"] = r["n_builds"]
    phis, phit, iden = po.kinetics(r["P_S"], r["P_T0"], r["P_Tp"], r["P_Tm"], dt, sp_.kS, sp_.kT)
    out["ts_small_Phi_S"], out["ts_small_Phi_T"] = phis, phit
    A = (np.arange(36).reshape(6, 6) % 7 - 3.0) * 0.11 + 1j * (np.arange(36).reshape(6, 6) % 5 - 2.0) * 0.07
    out["expm_in"] = A
    out["expm_out"] = po.expm(A)
    return out


if __name__ == "__main__":
    pyoracle.build()
    np.savez_compressed(os.path.join(HERE, "oracle_golden.npz"), **cases(pyoracle))
    print("wrote", os.path.join(HERE, "oracle_golden.npz"))
