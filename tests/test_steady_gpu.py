"""GPU: steady-state accuracy of every storage against the FP64 parity mode.

A lid-driven cavity (MRT, Re 100, lid 0.05, the reference's boundary
treatment) runs from rest for a fixed number of steps in FP64 and in every
other storage, and the states are compared at the same step.  The reference's
lid treatment (serial/BoundaryConditions.c:25-37) adds mass every step in
every precision, so the mean density rises linearly and a small cavity never
becomes exactly steady (64^2: du_rel stays near 4e-9 in FP64; 256^2 reaches
1.6e-10 at 128k steps); comparing at the same step keeps that drift out of
the errors.  Velocity is compared as max |(u, v) - (u, v)_FP64| over
max |(u, v)_FP64|; density after removing the mean offset (the shape of the
field), with the mean offset checked separately.

Stated tolerances (|u| max rel, de-meaned rho max / rho0, mean offset / rho0):
  FP32       1e-5   1e-5   1e-4
  FP16NEQ    1e-4   1e-5   1e-4   (moment storage: the 1e-4 velocity target)
  FP16-dev   2e-2   2e-3   5e-2   (16-bit populations: rounding in the conserved moments)
  BF16-dev   3e-1   2e-2   3e-1
"""
import numpy as np
import pytest

import parallellbmcranfield_gb300 as G

pytestmark = pytest.mark.gpu

TOL = {
    G.FP32: (1e-5, 1e-5, 1e-4),
    G.FP16NEQ: (1e-4, 1e-5, 1e-4),
    G.FP16DEV: (2e-2, 2e-3, 5e-2),
    G.BF16DEV: (3e-1, 2e-2, 3e-1),
}
STEPS = {64: 150000, 254: 130000}  # FP64 du_rel near its floor (64) or below 1e-9 (254)
_ref_cache = {}


def run(side, precision, steps):
    mesh = G.Mesh.cavity(side)
    s = G.Solver(mesh, uavg=0.05, viscosity=0.05 * side / 100.0, inlet_profile=2,
                 collision_model=G.MRT, curved_boundaries=1, outlet_profile=2,
                 precision=precision)
    s.set_state(None, np.ones(s.N), np.zeros(s.N), np.zeros(s.N))
    s.step(steps - 1000)
    s.check()
    s.step(1000)
    du = s.check()["du_rel"]
    out = s.fields()
    s.close()
    fluid = G.inspect_mesh(mesh)["cls"] > 0
    return out, du, fluid


def reference(side):
    if side not in _ref_cache:
        _ref_cache[side] = run(side, G.FP64, STEPS[side])
    return _ref_cache[side]


@pytest.mark.parametrize("side", [64, 254])
@pytest.mark.parametrize("precision", [G.FP32, G.FP16NEQ, G.FP16DEV, G.BF16DEV])
def test_steady_state_against_fp64(side, precision):
    ref, du, fl = reference(side)
    assert du <= 1e-8  # FP64 at (or near) its steady state
    low, _, _ = run(side, precision, STEPS[side])
    sp = np.sqrt(ref["u"] ** 2 + ref["v"] ** 2)[fl]
    e = np.sqrt((low["u"] - ref["u"]) ** 2 + (low["v"] - ref["v"]) ** 2)[fl]
    dr = (low["rho"] - ref["rho"])[fl]
    err_u = e.max() / sp.max()
    err_rho = np.abs(dr - dr.mean()).max()
    off = abs(dr.mean())
    print(f"side {side} precision {precision} after {STEPS[side]} steps (FP64 du_rel {du:.1e}): "
          f"|u| {err_u:.3e} rho de-meaned {err_rho:.3e} mean offset {off:.3e}")
    tu, tr, to = TOL[precision]
    assert err_u <= tu
    assert err_rho <= tr
    assert off <= to
