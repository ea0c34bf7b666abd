"""spin_dynamics_gb300 — GB300-native trace-sampling hot path of spinchem
(KenHino/Spin_dynamics): device Hamiltonian assembly and batched complex128
Krylov propagation behind a C ABI (include/spinchem_gpu.h), with this
package as the Python host layer.
"""
from .spinsys import (GAMMA_14N, GAMMA_1H, GAMMA_E, Electron, SimParam, SpinchemError, SysParam,
                      read_inp)
from .observables import Observables, field_folder_name, fortran_list_directed

__all__ = ["GAMMA_E", "GAMMA_1H", "GAMMA_14N", "Electron", "SysParam", "SimParam",
           "SpinchemError", "read_inp", "Observables", "field_folder_name",
           "fortran_list_directed", "TraceSampler", "trace_sampling_para", "trace_sampling",
           "exact_dynamics"]


def __getattr__(name):
    # the GPU-facing names load libspinchem_gpu on first use
    if name in ("TraceSampler", "trace_sampling_para", "trace_sampling", "exact_dynamics",
                "seeded_samples", "init_el_state", "num_time_points"):
        from . import dynamics
        return getattr(dynamics, name)
    raise AttributeError(name)
