"""GPU: moment storage (LBM_FP16NEQ) against the FP64 parity mode.

The state of this storage is each node's post-collision moments: density
and momentum deviations in 24-bit fixed point, the six non-equilibrium
moments in FP16, nodes with boundary work in FP32.  Arithmetic is FP32.  It
runs every collision model (serial/CellFunctions.c:352-438) and boundary
kind of the parity cases; results are compared with the FP64 mode (itself
bit-identical to the serial reference) after each case's step count, with
the per-field tolerances below, relative to max |field|.
"""
import numpy as np
import pytest

import cases
import parallellbmcranfield_gb300 as G

pytestmark = pytest.mark.gpu

TOL_RHO = 2e-5  # max |rho - rho_FP64| / max rho
TOL_U = 2e-4    # max |(u, v) - (u, v)_FP64| / max |(u, v)_FP64|
FEQ_CASES = sorted(k for k, v in cases.ALL.items() if v[2] == "feq")


def run(name, precision, tile=0, steps=None):
    spec, params, start, nsteps = cases.ALL[name]
    mesh = cases.build_mesh(spec)
    s = G.Solver(mesh, precision=precision, pattern=G.AB, tile_variant=tile, **params)
    s.set_state(*cases.start_state(mesh, params, start))
    s.step(steps or nsteps)
    out = s.fields()
    d = s.check()
    s.close()
    return out, d


@pytest.mark.parametrize("name", FEQ_CASES)
def test_fp16neq_against_fp64(name):
    ref, dref = run(name, G.FP64)
    low, dlow = run(name, G.FP16NEQ)
    speed = np.sqrt(ref["u"] ** 2 + ref["v"] ** 2).max()
    err_u = np.sqrt((low["u"] - ref["u"]) ** 2 + (low["v"] - ref["v"]) ** 2).max() / speed
    err_rho = np.abs(low["rho"] - ref["rho"]).max() / np.abs(ref["rho"]).max()
    print(f"{name}: rho {err_rho:.3e} |u| {err_u:.3e}")
    assert err_rho <= TOL_RHO
    assert err_u <= TOL_U
    # the full-field diagnostics agree too (mass to the density tolerance)
    assert abs(dlow["mass"] - dref["mass"]) <= TOL_RHO * abs(dref["mass"])


@pytest.mark.parametrize("tile", [1, 2, 3, 4])
def test_every_tile_against_fp64(tile):
    """The four bulk tiles (34 or 64 rows per thread, source rows loaded one
    or two rows ahead, 4 or 5 blocks per SM) do the same arithmetic per node, but the
    compiler may fuse multiply-adds differently in each; a
    last-bit difference can move a dithered fixed-point code by one step, so
    the tiles are not bitwise equal: each meets the FP64 tolerances."""
    ref, _ = run("cavity_mrt_curved", G.FP64)
    low, _ = run("cavity_mrt_curved", G.FP16NEQ, tile=tile)
    speed = np.sqrt(ref["u"] ** 2 + ref["v"] ** 2).max()
    assert np.abs(low["rho"] - ref["rho"]).max() <= TOL_RHO * np.abs(ref["rho"]).max()
    assert np.sqrt((low["u"] - ref["u"]) ** 2 + (low["v"] - ref["v"]) ** 2).max() <= TOL_U * speed


def test_autotune_and_bytes():
    spec, params, start, _ = cases.ALL["cavity_mrt_curved"]
    mesh = cases.build_mesh(spec)
    s = G.Solver(mesh, precision=G.FP16NEQ, **params)
    rep = s.autotune(3)
    assert 0 <= rep["variant"] < 4 and len(rep["ms"]) == 4
    assert s.info()["bytes_per_node_step"] == 42
    s.close()


def test_aa_pattern_is_refused():
    spec, params, _, _ = cases.ALL["cavity_mrt_curved"]
    with pytest.raises(G.LbmError, match="A-B"):
        G.Solver(cases.build_mesh(spec), precision=G.FP16NEQ, pattern=G.AA, **params)


def test_out_of_range_is_reported():
    """The reference's own start (F = 0 before the first collision) gives a
    collided state whose density is omega rho0 (here 1.89 rho0): beyond the
    fixed-point range, which the step reports instead of storing a clipped value."""
    spec, params, _, _ = cases.ALL["cavity_bgk_refstart"]
    s = G.Solver(cases.build_mesh(spec), precision=G.FP16NEQ, **params)
    with pytest.raises(G.DivergedError, match="out of range"):
        s.step(2)
    s.close()
