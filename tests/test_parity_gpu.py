"""GPU parity: the CUDA library through its C ABI against the oracle.

FP64 mode must equal the serial reference within 1e-10 relative (it is
designed to be bit-identical); the AA in-place pattern must equal the A-B
pattern; reduced precisions are checked against FP64 with stated tolerances.
"""
import os

import numpy as np
import pytest

import cases
import parallellbmcranfield_gb300 as G
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
FP64_RTOL = 1e-10

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    scale = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() / scale


def run_gpu(name, precision=G.FP64, pattern=G.AB, check_every=1, steps=None):
    spec, params, start, nsteps = cases.ALL[name]
    steps = steps or nsteps
    mesh = cases.build_mesh(spec)
    s = G.Solver(mesh, precision=precision, pattern=pattern, **params)
    st = cases.start_state(mesh, params, start)
    if st is not None:
        s.set_state(*st)
    resid = s.step(steps, check_every)
    return mesh, s, resid


def run_port(name, steps=None):
    spec, params, start, nsteps = cases.ALL[name]
    mesh = cases.build_mesh(spec)
    p = O.Port(mesh.nodes, mesh.conns, **cases.oracle_params(params))
    st = cases.start_state(mesh, params, start)
    if st is not None:
        p.set_state(*st)
    _, r = p.run(steps or nsteps)
    return p, r


@pytest.mark.parametrize("pattern", [G.AB, G.AA])
@pytest.mark.parametrize("name", sorted(cases.ALL))
def test_fp64_matches_reference(name, pattern):
    g = dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))
    mesh, s, resid = run_gpu(name, G.FP64, pattern)
    port, presid = run_port(name)
    ps = port.state()
    out = s.fields(f=True, metaf=True)
    idx = g["sample"]
    # residual lines of serial/Iterate.c:301 (quirky L2 over cells 0..m-1)
    assert resid.shape == g["resid"].shape
    assert np.allclose(resid, g["resid"], rtol=1e-12, atol=1e-300)
    for k in ("rho", "u", "v"):
        assert rel_err(out[k][idx], g[f"s_{k}"]) <= FP64_RTOL, k
        assert rel_err(out[k], ps[k]) <= FP64_RTOL, k
    assert rel_err(out["f"], ps["F"]) <= FP64_RTOL
    assert rel_err(out["metaf"], ps["METAF"]) <= FP64_RTOL
    assert rel_err(out["f"][idx], g["s_F"]) <= FP64_RTOL
    d = s.check()
    pd = port.diagnostics()
    assert abs(d["l2_full"] - pd[0]) <= 1e-10 * max(pd[0], 1e-30)
    assert abs(d["mass"] - pd[1]) <= 1e-12 * pd[1]
    for i in range(2):
        assert abs(d["momentum"][i] - pd[2 + i]) <= 1e-10 * max(abs(pd[1]), 1.0)
        assert abs(d["force"][i] - pd[4 + i]) <= 1e-10 * max(abs(pd[4]), abs(pd[5]), 1e-12)
    s.close()


@pytest.mark.parametrize("name", ["cavity_mrt_curved", "chan_mrt_extrap", "chan_bgk_velout"])
def test_aa_equals_ab_bitwise(name):
    _, a, _ = run_gpu(name, G.FP64, G.AB, check_every=0)
    _, b, _ = run_gpu(name, G.FP64, G.AA, check_every=0)
    fa, fb = a.fields(f=True, metaf=True), b.fields(f=True, metaf=True)
    for k in fa:
        assert np.array_equal(fa[k], fb[k]), k


@pytest.mark.parametrize("pattern", [G.AB, G.AA])
@pytest.mark.parametrize("name", ["chan_mrt_extrap", "cavity_trt_curved"])
@pytest.mark.parametrize("tile", [2, 3, 4, 5, 6])
def test_tile_variants_bitwise(tile, pattern, name):
    """Every tile variant of the fused step computes the same FP64 state."""
    spec, params, start, steps = cases.ALL[name]
    mesh = cases.build_mesh(spec)
    out = []
    for t in (1, tile):
        s = G.Solver(mesh, precision=G.FP64, pattern=pattern, tile_variant=t, **params)
        s.set_state(*cases.start_state(mesh, params, start))
        s.step(steps)
        out.append(s.fields(f=True, metaf=True))
        s.close()
    for k in out[0]:
        assert np.array_equal(out[0][k], out[1][k]), k


MID_CASES = {
    # cases wide enough that whole warps of every tile shape see only bulk
    # nodes, so the vector / paired / TMA paths run (not only the per-node path)
    "mid_cavity": (("cavity", 300), dict(uavg=0.05, vavg=0.0, rho_ini=1.0, viscosity=0.02,
                                         inlet_profile=2, collision_model=3, curved_boundaries=1,
                                         outlet_profile=2), 120),
    "mid_channel": (("channel", 700, 90, [(150.0, 45.5, 12.0)]),
                    dict(uavg=0.04, vavg=0.0, rho_ini=1.0, viscosity=0.03, inlet_profile=1,
                         collision_model=2, curved_boundaries=1, outlet_profile=2), 120),
}


def run_mid(name, precision, pattern, tile):
    spec, params, steps = MID_CASES[name]
    mesh = cases.build_mesh(spec)
    s = G.Solver(mesh, precision=precision, pattern=pattern, tile_variant=tile, **params)
    s.set_state(*cases.start_state(mesh, params, "feq"))
    s.step(steps)
    out = s.fields(f=True)
    s.close()
    return out


@pytest.mark.parametrize("pattern", [G.AB, G.AA])
@pytest.mark.parametrize("tile", [2, 3, 4, 5, 6])
@pytest.mark.parametrize("name", sorted(MID_CASES))
def test_tile_variants_bitwise_mid(name, tile, pattern):
    """FP64 on the wider cases: every tile shape gives the bitwise-same state."""
    a = run_mid(name, G.FP64, pattern, 1)
    b = run_mid(name, G.FP64, pattern, tile)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("precision,tol", [(G.FP32, 1e-5), (G.FP16DEV, 2e-3), (G.BF16DEV, 3e-2)])
@pytest.mark.parametrize("pattern", [G.AB, G.AA])
@pytest.mark.parametrize("tile", [2, 3, 4, 5, 6])
@pytest.mark.parametrize("name", sorted(MID_CASES))
def test_tile_variants_reduced_precision(name, tile, pattern, precision, tol):
    """Every tile reproduces the default tile's state in FP32 and 16-bit
    storage.  The node arithmetic is the same, but the compiler may contract a
    different set of multiply-adds in each kernel, so the check is at rounding
    level (relative to max |field|)."""
    a = run_mid(name, precision, pattern, 1)
    b = run_mid(name, precision, pattern, tile)
    assert rel_err(b["rho"], a["rho"]) <= tol
    assert rel_err(b["f"], a["f"]) <= tol
    speed = np.sqrt(a["u"] ** 2 + a["v"] ** 2).max()
    assert np.sqrt((b["u"] - a["u"]) ** 2 + (b["v"] - a["v"]) ** 2).max() <= tol * speed


def test_autotune_picks_a_variant(tmp_path):
    spec, params, start, _ = cases.ALL["cavity_mrt_curved"]
    mesh = cases.build_mesh(spec)
    cache = tmp_path / "tune.jsonl"
    s = G.Solver(mesh, precision=G.FP32, **params)
    rep = s.autotune(3, cache)
    assert 0 <= rep["variant"] < 6 and len(rep["ms"]) == 6
    s.set_state(*cases.start_state(mesh, params, start))
    s.step(10)
    s2 = G.Solver(mesh, precision=G.FP32, **params)
    rep2 = s2.autotune(3, cache)
    assert rep2.get("cached") and rep2["variant"] == rep["variant"]
    with pytest.raises(G.LbmError):
        s.autotune(3)  # only before set_state


def test_split_calls_equal_one_call():
    """lbm_step(a) + lbm_step(b) == lbm_step(a + b), with odd splits for AA parity."""
    _, one, _ = run_gpu("chan_mrt_extrap", G.FP64, G.AA, check_every=0, steps=101)
    spec, params, start, _ = cases.ALL["chan_mrt_extrap"]
    mesh = cases.build_mesh(spec)
    two = G.Solver(mesh, precision=G.FP64, pattern=G.AA, **params)
    two.set_state(*cases.start_state(mesh, params, start))
    for k in (1, 37, 63):
        two.step(k)
    a, b = one.fields(f=True), two.fields(f=True)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("pattern", [G.AB, G.AA])
@pytest.mark.parametrize("precision,tol_rho,tol_u", [(G.FP32, 1e-5, 1e-3), (G.FP16DEV, 1e-3, 5e-2),
                                                     (G.BF16DEV, 1e-2, 3e-1)])
@pytest.mark.parametrize("name", ["cavity_mrt_curved", "chan_mrt_pressure", "cavity_trt_curved"])
def test_reduced_precision_against_fp64(name, precision, tol_rho, tol_u, pattern):
    """Per-field tolerances after the case's step count, relative to max |field|."""
    _, ref, _ = run_gpu(name, G.FP64, G.AB, check_every=0)
    _, low, _ = run_gpu(name, precision, pattern, check_every=0)
    a, b = low.fields(), ref.fields()
    speed = np.sqrt(b["u"] ** 2 + b["v"] ** 2).max()
    err_u = np.sqrt((a["u"] - b["u"]) ** 2 + (a["v"] - b["v"]) ** 2).max() / speed
    err_rho = rel_err(a["rho"], b["rho"])
    print(f"{name} prec={precision} pat={pattern}: rho {err_rho:.3e} u {err_u:.3e}")
    assert err_rho <= tol_rho
    assert err_u <= tol_u


def test_reference_start_state():
    """Without lbm_set_state the library starts like the reference: F = 0, U = Uo."""
    g = dict(np.load(os.path.join(GOLDEN, "cavity_bgk_refstart.npz")))
    mesh, s, resid = run_gpu("cavity_bgk_refstart")
    out = s.fields()
    for k in ("rho", "u", "v"):
        assert rel_err(out[k][g["sample"]], g[f"s_{k}"]) <= FP64_RTOL


def test_fields_before_first_iteration():
    spec, params, start, _ = cases.ALL["cavity_bgk_bb"]
    mesh = cases.build_mesh(spec)
    s = G.Solver(mesh, **params)
    out = s.fields()
    assert np.all(out["rho"] == np.float32(params["rho_ini"]))
    assert np.all(out["u"] == np.float32(params["uavg"]))
    with pytest.raises(G.LbmError):
        s.fields(f=True)


def test_divergence_is_reported():
    from test_oracle import divergence_case

    mesh, st = divergence_case()
    s = G.Solver(mesh, uavg=0.04, rho_ini=1.0, viscosity=0.05, collision_model=1,
                 curved_boundaries=2, outlet_profile=1)
    s.set_state(*st)
    with pytest.raises(G.DivergedError):
        s.step(2, 1)
    with pytest.raises(G.DivergedError):
        s.check()
