"""python -m spin_dynamics_gb300 input.ini — the Python twin of the `spinchem`
executable (app/main.f90): read input.ini, run the simulation type for all
the listed fields together on the GPU library, write the output files."""
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
        folders = []
        for B in sim.B:
            folders.append(os.path.join(sim.output_folder, field_folder_name(B)))
            os.makedirs(folders[-1], exist_ok=True)
        # every field of the list together (app/main.f90:48-79 loops them)
        if sim.type in ("trace_sampling", "trace_sampling_serial", "exact_dynamics"):
            dynamics.field_dynamics(sys_, sim, folders, sampler)
        elif sim.type == "symmetry_dynamics":
            from . import symmetry
            for B in sim.B:
                print(f" {B}")
            symmetry.symmetrised_fields(sys_, sim, list(sim.B), folders, sampler)
        elif sim.type == "semi_classical":
            for _ in sim.B:
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
