"""GPU: the plain-method case over its full length -- lid-driven cavity of
125^2 fluid cells (the shipped coarse layout, 127 x 128 nodes), D2Q9 BGK,
FP64, lid u = 0.05, Re = 100 (nu = u L / Re with L = 125), rho0 = 1, f = f_eq
at rest, 20000 iterations with a residual line every 100 -- against the CPU
oracle over the whole run."""
import time

import numpy as np
import pytest

import cases
import parallellbmcranfield_gb300 as G
from oracle import oracle as O

pytestmark = pytest.mark.gpu

PARAMS = dict(uavg=0.05, vavg=0.0, rho_ini=1.0, viscosity=0.05 * 125 / 100, inlet_profile=2,
              collision_model=1, curved_boundaries=2, outlet_profile=2)
STEPS, EVERY = 20000, 100


def test_config1_full_run_matches_oracle():
    mesh = G.Mesh.cavity(125)
    st = cases.start_state(mesh, PARAMS, "feq")
    s = G.Solver(mesh, precision=G.FP64, **PARAMS)
    s.set_state(*st)
    t0 = time.perf_counter()
    res = s.step(STEPS, EVERY)
    gpu_s = time.perf_counter() - t0
    out = s.fields(f=True)
    diag = s.check()
    port = O.Port(mesh.nodes, mesh.conns, **cases.oracle_params(PARAMS))
    port.set_state(*st)
    t0 = time.perf_counter()
    _, pres = port.run(STEPS)
    cpu_s = time.perf_counter() - t0
    ps = port.state()
    print(f"config 1: GPU {gpu_s:.3f} s, oracle {cpu_s:.1f} s for {STEPS} iterations")
    assert res.shape == (STEPS // EVERY, 4)
    assert np.allclose(res, pres[EVERY - 1::EVERY], rtol=1e-12, atol=1e-300)
    for k, pk in (("rho", "rho"), ("u", "u"), ("v", "v"), ("f", "F")):
        err = np.abs(out[k] - ps[pk]).max() / np.abs(ps[pk]).max()
        assert err <= 1e-10, (k, err)
    pd = port.diagnostics()
    assert abs(diag["mass"] - pd[1]) <= 1e-12 * pd[1]
    assert abs(diag["l2_full"] - pd[0]) <= 1e-10 * pd[0]
