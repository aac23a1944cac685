"""Small cases for the drop-in program (lbm_solver) against the reference program.

Each case is a generated mesh plus the 16 SetUpData.ini values in the
reference's order (serial/FileIO.c:263-289): Uavg, Vavg, rho_ini, viscosity,
InletProfile, CollisionModel, CurvedBoundaries, OutletProfile, Iterations,
AutosaveEvery, AutosaveAfter, PostprocProg, CalculateDragLift,
ConvergenceCritVeloc, ConvergenceCritRho, ReadFormerData.
"""
import os

import parallellbmcranfield_gb300 as G

CASES = {
    "cavity30_bgk_csv": (("cavity", 30), [0.08, 0.0, 5, 0.02, 2, 1, 2, 2, 300, 100, 150, 1, 0, -1.0, -1.0, 0]),
    "cavity30_mrt_tecplot": (("cavity", 30), [0.05, 0.0, 1, 0.02, 2, 3, 1, 2, 250, 100, 0, 2, 0, -1.0, -1.0, 0]),
    "chan_trt_velout_drag": (("channel", 40, 14, [(12.0, 7.4, 3.1)]),
                             [0.04, 0.0, 1, 0.05, 2, 2, 1, 1, 200, 100, 50, 1, 5, -1.0, -1.0, 0]),
}


def build_mesh(spec):
    if spec[0] == "cavity":
        return G.Mesh.cavity(spec[1])
    return G.Mesh.channel(spec[1], spec[2], spec[3])


def write_case(case, directory):
    spec, ini = case
    os.makedirs(os.path.join(directory, "Mesh"), exist_ok=True)
    build_mesh(spec).write(os.path.join(directory, "Mesh", "D2node.dat"),
                           os.path.join(directory, "Mesh", "BCconnectors.dat"))
    with open(os.path.join(directory, "SetUpData.ini"), "w") as f:
        for v in ini:
            f.write(f"{v}\n")
