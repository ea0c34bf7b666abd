"""Time-resolved radical-pair populations and yields, and their output files.

Mirrors type `observables` (src/observables.f90): malloc/set/scale/update
(:21-72), get_kinetics (:74-101, Simpson's rule), output (:103-131) and
write_data (:133-148), whose files hold one value per line in gfortran's
list-directed REAL(8) format.
"""
from __future__ import annotations

import os
from dataclasses import dataclass
from typing import Optional

import numpy as np


def fortran_list_directed(x: float) -> str:
    """One REAL(8) as gfortran's list-directed WRITE prints it: a leading
    blank, then 1PG25.17E3-style editing (17 significant digits; fixed
    notation for 0.1 <= |x| < 1e17 followed by 5 blanks, otherwise
    d.dddE+xxx)."""
    x = float(x)
    if x == 0.0:
        body = "0.0000000000000000" + " " * 5
    elif not np.isfinite(x):
        body = ("NaN" if np.isnan(x) else ("Infinity" if x > 0 else "-Infinity")).rjust(23)
    else:
        mant, exp = f"{x:.16e}".split("e")
        e = int(exp)
        if -1 <= e < 17:
            # F editing with 17 significant digits
            decimals = 16 - e
            body = f"{x:.{decimals}f}" + " " * 5
            if e == -1:
                body = f"{x:.17f}" + " " * 5
        else:
            sign = "-" if e < 0 else "+"
            body = f"{mant}E{sign}{abs(e):03d}"
    return " " + body.rjust(25)


@dataclass
class Observables:
    P_S: np.ndarray
    P_T0: np.ndarray
    P_Tp: np.ndarray
    P_Tm: np.ndarray
    iden: Optional[np.ndarray] = None
    Phi_S: Optional[np.ndarray] = None
    Phi_T: Optional[np.ndarray] = None

    @classmethod
    def zeros(cls, n: int) -> "Observables":
        return cls(*(np.zeros(n) for _ in range(4)))

    def scale(self, f: float) -> None:
        for a in (self.P_S, self.P_T0, self.P_Tp, self.P_Tm):
            a *= f

    def update(self, other: "Observables") -> None:
        self.P_S += other.P_S
        self.P_T0 += other.P_T0
        self.P_Tp += other.P_Tp
        self.P_Tm += other.P_Tm

    def get_kinetics(self, dt: float, kS: float, kT: float) -> None:
        """Simpson yields (src/observables.f90:74-101); dt, kS, kT in the
        reference's internal units."""
        P_T = (self.P_Tp + self.P_T0) + self.P_Tm
        self.iden = self.P_S + P_T
        nh = len(self.P_S) // 2
        self.Phi_S = np.zeros(nh)
        self.Phi_T = np.zeros(nh)
        fS = (1.0 / 3.0) * dt * kS
        fT = (1.0 / 3.0) * dt * kT
        ps = pt = 0.0
        for i in range(1, nh):
            ps = ps + fS * ((self.P_S[2 * i - 2] + 4.0 * self.P_S[2 * i - 1]) + self.P_S[2 * i])
            pt = pt + fT * ((P_T[2 * i - 2] + 4.0 * P_T[2 * i - 1]) + P_T[2 * i])
            self.Phi_S[i] = ps
            self.Phi_T[i] = pt

    def output(self, path: str) -> None:
        """Write S/Tp/T0/Tm_prob.data (+ total_prob, S_yield, T_yield when
        kinetics were computed) into `path` (src/observables.f90:103-131)."""
        files = [("S_prob.data", self.P_S), ("Tp_prob.data", self.P_Tp),
                 ("T0_prob.data", self.P_T0), ("Tm_prob.data", self.P_Tm)]
        if self.iden is not None:
            files.append(("total_prob.data", self.iden))
        if self.Phi_S is not None:
            files.append(("S_yield.data", self.Phi_S))
        if self.Phi_T is not None:
            files.append(("T_yield.data", self.Phi_T))
        for name, data in files:
            write_data(data, path, name)


def write_data(data, path: str, filename: str) -> None:
    with open(os.path.join(path, filename), "w") as f:
        for v in data:
            f.write(fortran_list_directed(v) + "\n")


def field_folder_name(B: float) -> str:
    """write(guz,'(F0.3)') B (app/main.f90:58): minimal width, 3 decimals, no
    leading zero for |B| < 1 (e.g. '.200', '-.050', '25.000')."""
    s = f"{abs(B):.3f}"
    if s.startswith("0."):
        s = s[1:]
    return ("-" if B < 0 and float(s) != 0.0 else "") + s
