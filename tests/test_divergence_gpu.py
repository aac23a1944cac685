"""GPU: lbm_step reports a NaN anywhere in a reduced-precision state.

The reference stops on divergence only when its residual line is NaN
(serial/ComputeResiduals.c:47-51), and that residual visits the cells 0..m-1
only: on a cavity those are solid, so a NaN in the flow goes unseen.  The FP32
and 16-bit steps flag any node whose collision meets a NaN or an infinity, so
lbm_step returns LBM_DIVERGED without a check or a residual line.  The NaN is
planted on the host, in the density of one bulk node given to lbm_set_state.
FP64, the parity mode, keeps the reference's report: the step goes on, and
only lbm_check (full-field sums) sees the NaN.
"""
import numpy as np
import pytest

import parallellbmcranfield_gb300 as G

pytestmark = pytest.mark.gpu

SIDE = 62


def solver(precision, pattern, model, tile):
    mesh = G.Mesh.cavity(SIDE)
    return G.Solver(mesh, uavg=0.05, rho_ini=1.0, viscosity=0.05 * SIDE / 100.0,
                    collision_model=model, curved_boundaries=2, precision=precision,
                    pattern=pattern, tile_variant=tile)


def planted(s, where):
    rho = np.ones(s.N)
    rho[where] = np.nan
    s.set_state(None, rho, np.zeros(s.N), np.zeros(s.N))


@pytest.mark.parametrize("precision,pattern,model,tile", [
    (G.FP32, G.AB, G.MRT, 1), (G.FP32, G.AA, G.MRT, 2), (G.FP32, G.AB, G.BGKW, 3),
    (G.FP32, G.AB, G.TRT, 4), (G.FP16DEV, G.AB, G.MRT, 5), (G.FP16DEV, G.AA, G.MRT, 6),
    (G.FP16DEV, G.AB, G.TRT, 5), (G.BF16DEV, G.AB, G.MRT, 1), (G.FP16NEQ, G.AB, G.MRT, 1),
    (G.FP16NEQ, G.AB, G.BGKW, 3)])
def test_nan_in_a_bulk_node_is_reported(precision, pattern, model, tile):
    s = solver(precision, pattern, model, tile)
    centre = (s.m // 2) * s.n + s.n // 2
    planted(s, centre)
    with pytest.raises(G.DivergedError, match="NaN or infinity"):
        s.step(3, 0)  # no residual line asked for
    # the flag stays until a new state is set; a clean state steps again
    with pytest.raises(G.DivergedError):
        s.step(1, 0)
    s.set_state(None, np.ones(s.N), np.zeros(s.N), np.zeros(s.N))
    s.step(5, 0)
    s.close()


@pytest.mark.parametrize("precision,tile", [(G.FP16DEV, 5), (G.FP16NEQ, 2)])
def test_nan_next_to_a_wall_is_reported(precision, tile):
    s = solver(precision, G.AB, G.MRT, tile)
    planted(s, 1 * s.n + 1)  # the bottom-left fluid corner: a boundary node
    with pytest.raises(G.DivergedError):
        s.step(2, 0)
    s.close()


def test_fp64_keeps_the_reference_report():
    s = solver(G.FP64, G.AB, G.MRT, 0)
    planted(s, (s.m // 2) * s.n + s.n // 2)
    resid = s.step(4, 1)  # the reference's residual (cells 0..m-1) stays finite
    assert np.isfinite(resid).all()
    with pytest.raises(G.DivergedError):
        s.check()  # the full-field diagnostics see it
    s.close()
