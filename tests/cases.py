"""Parity cases shared by the golden-fixture script and the tests.

Each case names a mesh (built by the library's generator, so the GPU machine can
rebuild it without the reference tree), the SetUpData.ini switches, the
start state and the number of iterations.  The cavity of side 125 is the
shipped ``cases/coarse`` mesh (127 x 128 array); the channels exercise the
inlet, the three serial outlets, the constant-pressure outlet and curved
walls around a cylinder.
"""
import numpy as np

import parallellbmcranfield_gb300 as G

W = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4)

# shipped coarse ini: Uavg 0.08, rho 5, nu 0.01 (cases/coarse/SetUpData.ini)
COARSE = dict(uavg=0.08, vavg=0.0, rho_ini=5.0, viscosity=0.01, inlet_profile=2)
CHANNEL = dict(uavg=0.04, vavg=0.0, rho_ini=1.0, viscosity=0.05)
CYL = [(14.0, 10.3, 4.2)]

CASES = {
    # name: (mesh spec, params, start, steps)
    "cavity_bgk_bb": (("cavity", 125), dict(COARSE, collision_model=1, curved_boundaries=2), "feq", 200),
    "cavity_bgk_refstart": (("cavity", 125), dict(COARSE, collision_model=1, curved_boundaries=2), "ref", 200),
    "cavity_trt_curved": (("cavity", 125), dict(COARSE, viscosity=0.05, collision_model=2, curved_boundaries=1), "feq", 200),
    "cavity_mrt_bb": (("cavity", 125), dict(COARSE, collision_model=3, curved_boundaries=2), "feq", 200),
    "cavity_mrt_curved": (("cavity", 125), dict(COARSE, collision_model=3, curved_boundaries=1), "feq", 200),
    "chan_bgk_velout": (("channel", 48, 20, CYL), dict(CHANNEL, inlet_profile=1, collision_model=1, curved_boundaries=1, outlet_profile=1, drag_lift_id=5), "feq", 300),
    "chan_mrt_extrap": (("channel", 48, 20, CYL), dict(CHANNEL, inlet_profile=2, collision_model=3, curved_boundaries=1, outlet_profile=2, drag_lift_id=5), "feq", 300),
    "chan_trt_bb_none": (("channel", 48, 20, CYL), dict(CHANNEL, inlet_profile=2, collision_model=2, curved_boundaries=2, outlet_profile=3), "feq", 300),
    "chan_mrt_bb_extrap": (("channel", 48, 20, CYL), dict(CHANNEL, inlet_profile=1, collision_model=3, curved_boundaries=2, outlet_profile=2), "feq", 300),
}
# constant-pressure outlet: not in the reference, oracle restatement only
ORACLE_ONLY = {
    "chan_mrt_pressure": (("channel", 48, 20, CYL), dict(CHANNEL, inlet_profile=1, collision_model=3, curved_boundaries=1, outlet_profile=4, rho_out=1.0, drag_lift_id=5), "feq", 300),
}
ALL = dict(CASES, **ORACLE_ONLY)


def build_mesh(spec):
    if spec[0] == "cavity":
        return G.Mesh.cavity(spec[1])
    return G.Mesh.channel(spec[1], spec[2], spec[3])


def start_state(mesh, params, start):
    """(F, rho, u, v) for 'feq' (f = f_eq at rest) or None for the reference's own start."""
    if start == "ref":
        return None
    n, m = mesh.shape
    N = n * m
    rho0 = float(np.float32(params["rho_ini"]))
    return (np.tile(rho0 * W, (N, 1)), np.full(N, rho0), np.zeros(N), np.zeros(N))


def sample_cells(mesh, count=24, seed=7):
    """Fixed sample: every class-3 (boundary) cell type plus random fluid cells."""
    n, m = mesh.shape
    fluid = np.flatnonzero(mesh.nodes[:, 4] == 1)
    # node records are row-major i fastest for generated meshes
    idx = (mesh.nodes[fluid, 1].astype(np.int64) * n + mesh.nodes[fluid, 0].astype(np.int64))
    rng = np.random.default_rng(seed)
    pick = rng.choice(idx, size=min(count, len(idx)), replace=False)
    conn_cells = np.unique(mesh.conns[:, 1].astype(np.int64) * n + mesh.conns[:, 0].astype(np.int64))
    pick2 = rng.choice(conn_cells, size=min(count, len(conn_cells)), replace=False)
    return np.unique(np.concatenate([pick, pick2]))


def oracle_params(params):
    """Port keyword arguments from library-style params."""
    p = dict(params)
    return dict(uavg=p["uavg"], vavg=p["vavg"], rho_ini=p["rho_ini"], viscosity=p["viscosity"],
                inlet_profile=p.get("inlet_profile", 2), model=p["collision_model"],
                curved=p["curved_boundaries"], outlet=p.get("outlet_profile", 2),
                drag_id=p.get("drag_lift_id", 0), rho_out=p.get("rho_out", 1.0))
