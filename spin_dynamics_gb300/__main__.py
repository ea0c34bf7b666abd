"""python -m spin_dynamics_gb300 input.ini — the Python twin of the `spinchem`
executable (app/main.f90): read input.ini, loop over the fields, run the
simulation type on the GPU library, write the output files."""
from __future__ import annotations

import os
import sys
import time

from .observables import field_folder_name
from .spinsys import SpinchemError, read_inp


def main(argv=None) -> int:
    argv = sys.argv[1:] if argv is None else argv
    t0 = time.time()
    print(" Program initialised")
    try:
        if not argv or not os.path.exists(argv[0]):
            raise SpinchemError("Error: Input file does not exist.")
        sys_, sim = read_inp(argv[0])
        from . import dynamics
        sampler = dynamics.TraceSampler(int(os.environ.get("SPINCHEM_DEVICE", "0")))
        if os.environ.get("SPINCHEM_KRYLOV"):
            sampler.set_krylov(os.environ["SPINCHEM_KRYLOV"])
        for B in sim.B:
            sys_.e1.w = -B  # app/main.f90:53-54
            sys_.e2.w = -B
            folder = os.path.join(sim.output_folder, field_folder_name(B))
            os.makedirs(folder, exist_ok=True)
            if sim.type == "trace_sampling":
                dynamics.trace_sampling_para(sys_, sim, folder, sampler)
            elif sim.type == "trace_sampling_serial":
                dynamics.trace_sampling(sys_, sim, folder, sampler)
            elif sim.type == "exact_dynamics":
                dynamics.exact_dynamics(sys_, sim, folder, sampler)
            elif sim.type == "symmetry_dynamics":
                from . import symmetry
                print(f" {B}")
                symmetry.symmetrised_dynamics(sys_, sim, folder, sampler)
            elif sim.type == "semi_classical":
                print(" method not yet implemented")
            else:
                raise SpinchemError("Error: Invalid simulation type entered.")
        sampler.close()
    except SpinchemError as e:
        print(str(e), file=sys.stderr)
        return 1
    el = int(time.time() - t0)
    if sim.type != "symmetry_dynamics":
        print(f"Time elapsed:  {el // 3600:2d}:{(el // 60) % 60:2d}:{el % 60:2d}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
