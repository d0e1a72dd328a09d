"""Command line mirroring the reference's L-HySEA.exe (src/GPU/main.cxx):

    python -m landslidehysea_gb300 <data.dat> [--pouliquen]

loads the problem, prints its summary and runs shallowWater() on the GPU.
"""
import sys

from . import io


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    if not argv:
        sys.stderr.write(__doc__)
        return 1
    law = 1 if "--pouliquen" in argv else 0
    prob = io.LoadedProblem(argv[0], friction_law=law)
    p = prob.params
    print(f"Volumes: {p.nx} x {p.ny}, total {p.nx * p.ny}")
    print(f"X: [{prob.xmin * p.L}, {prob.xmax * p.L}]  Y: [{prob.ymin * p.L}, {prob.ymax * p.L}]")
    print(f"CFL: {p.cfl}  r: {p.r}  angle: {io.reference_units_to_deg(p.angle1):.4f}")
    print(f"Simulation time: {prob.tiempo_tot * prob.T} s")
    if io.lib().comprobarSoporteCUDA() != 0:
        sys.stderr.write("Error: no CUDA device\n")
        return 1
    st, wall, _, _ = io.shallow_water(prob)
    if st == 1:
        sys.stderr.write("Error: not enough GPU memory\n")
        return 1
    if st == 2:
        sys.stderr.write("Error: not enough CPU memory\n")
        return 1
    if st != 0:
        sys.stderr.write(f"Error: status {st}\n")
        return 1
    print(f"Time: {wall:e} s")
    return 0


if __name__ == "__main__":
    sys.exit(main())
