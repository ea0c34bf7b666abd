"""Spin-system and simulation parameters, and the input.ini reader.

Mirrors module `variables` (src/spinsys.f90): the constants (:16-19), the
types `electron`, `sys_param`, `sim_param` (:21-56), `read_inp` (:60-135) with
its unit conversions, `check_inp` (:137-163), `electron_init` (:165-235) and
`is_isotropic` (:237-254). Errors that the reference reports with
`stop 'Error: ...'` raise `SpinchemError` with the same message.

Units after reading (as in the reference): energies in mT; kS, kT divided by
gamma_e; t_end and dt multiplied by gamma_e/1000 (ns -> mT^-1 scaled time).
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

g_e = 2.002319              # src/spinsys.f90:16
GAMMA_E = 176.08596         # src/spinsys.f90:17
GAMMA_1H = 0.26752218708    # src/spinsys.f90:18
GAMMA_14N = 0.0193297792    # src/spinsys.f90:19


class SpinchemError(RuntimeError):
    """Raised where the reference stops with an error message."""


def default_gamma(mult: int) -> float:
    """Nuclear gyromagnetic ratio the reference assigns by multiplicity
    (src/hamiltonian.f90:132-138): 3 -> 14N, 2 -> 1H."""
    if mult == 3:
        return GAMMA_14N
    if mult == 2:
        return GAMMA_1H
    raise SpinchemError("Error: sys%e1%g_I(i) must be 3 or 2")


@dataclass
class Electron:
    """type electron (src/spinsys.f90:21-29)."""
    g_I: list = field(default_factory=list)   # nuclear multiplicities
    A: list = field(default_factory=list)     # 3x3 hyperfine tensors (mT), [row, col]
    g: float = g_e
    w: float = 0.0                            # Larmor frequency, set per field (w = -B)
    gamma_I: Optional[list] = None            # per-nucleus gyromagnetic ratios

    def __post_init__(self):
        self.g_I = [int(x) for x in self.g_I]
        self.A = [np.asarray(a, dtype=np.float64).reshape(3, 3) for a in self.A]
        if len(self.A) != len(self.g_I):
            raise SpinchemError("Error: number of hyperfine tensors does not match the nuclei")

    @property
    def a_iso(self) -> np.ndarray:
        # e%a_iso(i) = trace(e%A(i,:,:))/3 (src/spinsys.f90:232)
        return np.array([np.trace(a) / 3.0 for a in self.A], dtype=np.float64)

    @property
    def isotropic(self) -> bool:
        # only A(1,1) == A(2,2) is checked (src/spinsys.f90:251)
        return all(a[0, 0] == a[1, 1] for a in self.A)

    @property
    def gammas(self) -> list:
        if self.gamma_I is not None:
            return [float(x) for x in self.gamma_I]
        return [default_gamma(g) for g in self.g_I]

    @property
    def Z(self) -> int:
        return int(np.prod(self.g_I)) if self.g_I else 1


@dataclass
class SysParam:
    """type sys_param (src/spinsys.f90:31-38). kS, kT are stored divided by
    gamma_e, as read_inp leaves them."""
    e1: Electron
    e2: Electron
    J: float = 0.0
    D: np.ndarray = field(default_factory=lambda: np.zeros((3, 3)))
    kS: float = 0.0
    kT: float = 0.0

    def __post_init__(self):
        self.D = np.asarray(self.D, dtype=np.float64).reshape(3, 3)

    @classmethod
    def from_input_units(cls, e1, e2, J=0.0, D=None, kS_per_us=0.0, kT_per_us=0.0):
        """Build from input.ini units (rates in 1/us)."""
        return cls(e1=e1, e2=e2, J=float(J), D=np.zeros((3, 3)) if D is None else D,
                   kS=kS_per_us / GAMMA_E, kT=kT_per_us / GAMMA_E)

    @property
    def Z1(self) -> int:
        return self.e1.Z

    @property
    def Z2(self) -> int:
        return self.e2.Z

    @property
    def Z(self) -> int:
        return self.Z1 * self.Z2

    @property
    def N(self) -> int:
        return 4 * self.Z


@dataclass
class SimParam:
    """type sim_param (src/spinsys.f90:40-56). t_end and dt are stored in the
    scaled time unit (ns * gamma_e / 1000), as read_inp leaves them."""
    type: str = "trace_sampling"
    B: list = field(default_factory=lambda: [0.0])
    init_state: str = "singlet"
    seed: tuple = (123456789, 987654321)
    N_samples: int = 1
    t_end: float = 0.0
    dt: float = 0.0
    N_krylov: int = 7
    tol: float = 1e-5
    M1: int = 1
    M2: int = 1
    block_tol: float = 1e-5
    output_folder: str = "."
    restart: Optional[int] = None

    @classmethod
    def from_input_units(cls, *, t_end_ns, dt_ns, **kw):
        return cls(t_end=t_end_ns * GAMMA_E / 1000.0, dt=dt_ns * GAMMA_E / 1000.0, **kw)

    @property
    def isRestart(self) -> bool:
        return self.restart is not None


def _to_int64(tok: str) -> int:
    v = int(tok)
    if not -(2**63) <= v < 2**63:
        raise SpinchemError("Error: seed does not fit a 64-bit integer")
    return v


class IniFile:
    """A small INI reader with the semantics the reference relies on from
    FiNeR's `file_ini` (src/spinsys.f90:60-235): sections, `key = value`
    options, whitespace-separated lists."""

    def __init__(self, path: str):
        self.sections: dict[str, dict[str, str]] = {}
        cur = None
        with open(path) as f:
            for raw in f:
                line = raw.strip()
                if not line or line[0] in ";#!":
                    continue
                if line.startswith("[") and "]" in line:
                    cur = line[1:line.index("]")].strip()
                    self.sections.setdefault(cur, {})
                    continue
                if "=" in line and cur is not None:
                    k, v = line.split("=", 1)
                    self.sections[cur][k.strip()] = v.strip()

    @property
    def Ns(self) -> int:
        return len(self.sections)

    def has_section(self, name: str) -> bool:
        return name in self.sections

    def get(self, section: str, option: str) -> Optional[str]:
        return self.sections.get(section, {}).get(option)

    def values(self, section: str, option: str) -> Optional[list]:
        v = self.get(section, option)
        return None if v is None else v.split()


def check_inp(ini: IniFile) -> None:
    """check_inp (src/spinsys.f90:137-163)."""
    sections = ["system variables", "simulation parameters", "electron 1", "electron 2"]
    if ini.Ns < len(sections):
        raise SpinchemError("Error: Number of sections in input file is less than expected.")
    if ini.Ns > len(sections):
        raise SpinchemError("Error: Number of sections in input file is more than expected.")
    for s in sections:
        if not ini.has_section(s):
            raise SpinchemError(f'Error: Section "{s}" is missing from input file.')


def electron_init(ini: IniFile, el_number: int) -> Electron:
    """electron_init (src/spinsys.f90:165-235)."""
    sec = f"electron {el_number}"
    g = ini.get(sec, "g")
    mult = ini.values(sec, "I")
    nI = ini.values(sec, "N_I")
    if mult is None or nI is None:
        mult, nI = [], []
    mult = [int(x) for x in mult]
    nI = [int(x) for x in nI]
    if len(mult) != len(nI):
        raise SpinchemError("Sections N_I and I must have the sam length.")
    g_I = []
    for m_, n_ in zip(mult, nI):
        g_I += [m_] * n_
    A = []
    for i in range(1, len(g_I) + 1):
        vals = ini.values(sec, f"A{i}")
        if vals is None or len(vals) < 9:
            raise SpinchemError(f"Error: Hyperfine copuling A{i} for electron {el_number} is missing.")
        # reshape(A_tmp, [3,3]) is column-major
        A.append(np.array([float(x) for x in vals[:9]]).reshape(3, 3, order="F"))
    return Electron(g_I=g_I, A=A, g=float(g) if g is not None else g_e)


def read_inp(filename: str) -> tuple[SysParam, SimParam]:
    """read_inp (src/spinsys.f90:60-135): parse input.ini, apply the unit
    conversions, and check the output folder exists."""
    if not os.path.exists(filename):
        raise SpinchemError("Error: Input file does not exist.")
    ini = IniFile(filename)
    check_inp(ini)
    sv, sp = "system variables", "simulation parameters"

    def need(sec, key, msg):
        v = ini.get(sec, key)
        if v is None:
            raise SpinchemError(msg)
        return v

    J = float(need(sv, "J", "Error: Exchange coupling is missing"))
    Dv = ini.values(sv, "D")
    if Dv is None or len(Dv) < 9:
        raise SpinchemError("Error: Dipolar coupling is missing")
    D = np.array([float(x) for x in Dv[:9]]).reshape(3, 3, order="F")
    kS = float(need(sv, "kS", "Error: Singlet recombination rate is missing")) / GAMMA_E
    kT = float(need(sv, "kT", "Error: Triplet recombination rate is missing")) / GAMMA_E

    sim = SimParam()
    sim.type = need(sp, "simulation_type", "Error: Simulation type is missing").strip()
    Bv = ini.values(sp, "B")
    if Bv is None:
        raise SpinchemError("Error: List of experiment magnetic fields is missing")
    sim.B = [float(x) for x in Bv]
    sim.init_state = need(sp, "initial_state", "Error: Initial state is missing").strip()
    dt = float(need(sp, "dt", "Error: Propagation timestep is missing"))
    seed = ini.values(sp, "seed")
    if seed is not None and len(seed) >= 2:
        sim.seed = (_to_int64(seed[0]), _to_int64(seed[1]))
    if ini.get(sp, "N_samples") is not None:
        sim.N_samples = int(ini.get(sp, "N_samples"))
    t_end = float(ini.get(sp, "simulation_time") or 0.0)
    sim.t_end = (t_end * GAMMA_E) / 1000.0
    sim.dt = (dt * GAMMA_E) / 1000.0
    if ini.get(sp, "block_tolerance") is not None:
        sim.block_tol = float(ini.get(sp, "block_tolerance"))
    if ini.get(sp, "N_krylov") is not None:
        sim.N_krylov = int(ini.get(sp, "N_krylov"))
    if ini.get(sp, "integrator_tolerance") is not None:
        sim.tol = float(ini.get(sp, "integrator_tolerance"))
    if ini.get(sp, "M1") is not None:
        sim.M1 = int(ini.get(sp, "M1"))
    if ini.get(sp, "M2") is not None:
        sim.M2 = int(ini.get(sp, "M2"))
    if ini.get(sp, "restart") is not None:
        sim.restart = int(ini.get(sp, "restart"))
    sim.output_folder = (ini.get(sp, "output_folder") or "").strip()
    if not os.path.isdir(sim.output_folder):
        raise SpinchemError("Error: Output folder does not exist.")
    e1 = electron_init(ini, 1)
    e2 = electron_init(ini, 2)
    return SysParam(e1=e1, e2=e2, J=J, D=D, kS=kS, kT=kT), sim
