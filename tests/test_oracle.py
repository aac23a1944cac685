"""CPU: the oracle (C restatement) against the golden fixtures and, where the
reference sources were available at build time, against the unmodified
reference itself."""
import os

import numpy as np
import pytest

import cases
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
REF_CASES = O.REF_CASES


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))


def run_port(name):
    spec, params, start, steps = cases.ALL[name]
    mesh = cases.build_mesh(spec)
    port = O.Port(mesh.nodes, mesh.conns, **cases.oracle_params(params))
    st = cases.start_state(mesh, params, start)
    if st is not None:
        port.set_state(*st)
    status, resid = port.run(steps)
    return mesh, port, status, resid


@pytest.mark.parametrize("name", sorted(cases.ALL))
def test_port_matches_golden(name):
    g = load_golden(name)
    mesh, port, status, resid = run_port(name)
    assert status == 0
    s = port.state()
    idx = g["sample"]
    # bit-exact: the port is the reference's arithmetic in the reference's order
    assert np.array_equal(resid, g["resid"])
    for k in ("rho", "u", "v"):
        assert np.array_equal(s[k][idx], g[f"s_{k}"]), k
        assert np.allclose([s[k].sum(), (s[k] ** 2).sum()], g[f"sum_{k}"], rtol=1e-13, atol=0)
    assert np.array_equal(s["F"][idx], g["s_F"])
    assert np.array_equal(s["METAF"][idx], g["s_METAF"])
    assert np.array_equal(s["drag"][idx], g["s_drag"])
    assert np.allclose(port.diagnostics(), g["diag"], rtol=1e-12, atol=1e-300)


def test_residual_quirk_is_zero_on_cavities():
    """serial/ComputeResiduals.c:25 only visits cells 0..m-1 (solid): L2 is 0."""
    g = load_golden("cavity_bgk_bb")
    assert (g["resid"][:, :2] == 0).all()


@pytest.mark.skipif(not O.ref_available(), reason="reference harness not built here")
@pytest.mark.parametrize("case", ["coarse", "medium"])
@pytest.mark.parametrize("model,curved", [(1, 2), (2, 1), (3, 2), (3, 1)])
def test_port_matches_reference_on_shipped_meshes(case, model, curved):
    d = os.path.join(REF_CASES, case, "Mesh")
    nf, cf = os.path.join(d, "D2node.dat"), os.path.join(d, "BCconnectors.dat")
    nodes, conns = O.read_mesh(nf, cf)
    kw = dict(uavg=0.08, vavg=0.0, rho_ini=5.0, viscosity=0.03, inlet_profile=2, model=model,
              curved=curved, outlet=2)
    ref = O.Ref(nf, cf, **kw)
    port = O.Port(nodes, conns, **kw)
    ri, rr = ref.init_fields()
    pi, pr = port.init_fields()
    assert np.array_equal(ri, pi) and np.array_equal(rr, pr)
    assert np.array_equal(ref.constants(), port.constants())
    steps = 40 if case == "medium" else 100
    _, a = ref.run(steps)
    _, b = port.run(steps)
    assert np.array_equal(a, b)
    sa, sb = ref.state(), port.state()
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k


def divergence_case():
    """A tall narrow channel (m > n): cells 0..m-1, the only ones the reference's
    residual visits, reach into the fluid; a NaN planted in a fluid cell there
    shows up in the residual."""
    mesh = cases.build_mesh(("channel", 4, 20, []))
    n, m = mesh.shape
    N = n * m
    F = np.tile(cases.W, (N, 1))
    F[n + 2] = np.nan  # fluid cell (2, 1), index n + 2 < m
    return mesh, (F, np.ones(N), np.zeros(N), np.zeros(N))


def test_port_reports_divergence():
    """NaN in the residual makes the step return 1 (the reference exits(1))."""
    mesh, st = divergence_case()
    port = O.Port(mesh.nodes, mesh.conns, uavg=0.04, vavg=0.0, rho_ini=1.0, viscosity=0.05,
                  model=1, curved=2, outlet=1)
    port.set_state(*st)
    status, _ = port.run(2)
    assert status == 1
