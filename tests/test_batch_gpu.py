"""GPU: batched stepping (lbm_batch_*) against single-domain contexts."""
import numpy as np
import pytest

import cases
import parallellbmcranfield_gb300 as G

pytestmark = pytest.mark.gpu

BASE = dict(uavg=0.05, vavg=0.0, rho_ini=1.0, inlet_profile=2, curved_boundaries=1,
            outlet_profile=2)


def batch_cases(model):
    return [
        (G.Mesh.cavity(30), dict(BASE, viscosity=0.03, collision_model=model)),
        (G.Mesh.cavity(57), dict(BASE, viscosity=0.05, collision_model=model)),
        (G.Mesh.channel(60, 20, [(15.0, 10.4, 4.0)]),
         dict(BASE, uavg=0.04, viscosity=0.04, inlet_profile=1, outlet_profile=1,
              collision_model=model)),
        (G.Mesh.cavity(131), dict(BASE, viscosity=0.02, collision_model=model)),
    ]


def single(mesh, params, precision, iterations):
    s = G.Solver(mesh, precision=precision, **params)
    n, m = mesh.shape
    N = n * m
    s.set_state(None, np.full(N, float(np.float32(params["rho_ini"]))), np.zeros(N), np.zeros(N))
    s.step(iterations)
    out = s.fields()
    s.close()
    return out


@pytest.mark.parametrize("model", [1, 2, 3])
def test_batch_equals_single_contexts_fp64(model):
    """FP64: each case of a batch is bitwise the single-domain result."""
    cs = batch_cases(model)
    b = G.Batch(cs, precision="fp64")
    b.set_rest()
    r = b.run(60, check_every=20, tol=-1.0)  # tol < 0: nobody converges
    assert (r["steps"] == 60).all()
    for c, (mesh, params) in enumerate(cs):
        got = b.fields(c)
        want = single(mesh, params, G.FP64, 61)  # set_rest + 60 fused steps = 61 iterations
        for k in got:
            assert np.array_equal(got[k], want[k]), (c, k)
    b.close()


@pytest.mark.parametrize("precision", ["fp32", "fp16dev"])
def test_batch_tiles_and_autotune(precision):
    cs = batch_cases(2)
    ref = None
    rep = G.Batch(cs, precision=precision).autotune(2)
    assert 0 <= rep["variant"] < 4 and len(rep["ms"]) == 4
    assert rep["special_blocks_per_sm"] in (0, 2, 4, 8) and len(rep["special_ms"]) == 4
    assert rep["bulk_prefetch"] in (0, 1) and len(rep["prefetch_ms"]) == 2
    for tile in range(4):
        b = G.Batch(cs, precision=precision)
        b.set_tile(tile)
        b.set_rest()
        r = b.run(40, check_every=40, tol=-1.0)
        assert (r["steps"] == 40).all()
        f = b.fields(3)
        if ref is None:
            ref = f
        else:
            assert np.abs(f["u"] - ref["u"]).max() < 1e-3 * np.abs(ref["u"]).max()
        b.close()


def test_batch_convergence_freezes_cases():
    """Low-Re cavities converge at different times; a converged case stops."""
    cs = [(G.Mesh.cavity(side), dict(BASE, viscosity=nu, collision_model=2))
          for side, nu in ((16, 0.2), (24, 0.2), (40, 0.3))]
    b = G.Batch(cs, precision="fp32")
    r = b.run(200000, check_every=100, tol=1e-8)  # relative change per step
    assert (r["converged"] == 1).all(), r
    assert (r["du_rel"] <= 1e-8).all()
    # a smaller cavity converges in fewer steps than a larger one at similar Re
    assert r["steps"][0] < r["steps"][2]
    # frozen cases keep their converged state
    f1 = b.fields(0)
    b.close()
    assert np.isfinite(f1["u"]).all()


@pytest.mark.parametrize("precision", ["fp32", "fp16dev"])
def test_batch_matches_single_contexts_reduced(precision):
    """FP32 / FP16-dev: the per-tile bulk kernel and the boundary-node pass do
    the single-domain arithmetic per node (same operators, same storage)."""
    cs = batch_cases(3)
    b = G.Batch(cs, precision=precision)
    b.set_rest()
    b.run(60, check_every=20, tol=-1.0)
    for c, (mesh, params) in enumerate(cs):
        got = b.fields(c)
        want = single(mesh, params, G.PRECISIONS[precision], 61)
        speed = np.sqrt(want["u"] ** 2 + want["v"] ** 2).max()
        err = np.sqrt((got["u"] - want["u"]) ** 2 + (got["v"] - want["v"]) ** 2).max() / speed
        assert err <= 1e-5, (c, err)
        assert np.abs(got["rho"] - want["rho"]).max() <= 1e-6
    b.close()


@pytest.mark.parametrize("precision", ["fp32", "fp16dev"])
def test_batch_outlet_kinds_match_single_contexts(precision):
    """Channels with each outlet kind (velocity outlet, second-order
    extrapolation, constant pressure) and a curved cylinder in one batch: the
    boundary-node pass takes its neighbours from the side arrays or from the
    planes by kind, the extrapolating outlet takes the full treatment, and
    every plane another node reads is written; the fields match single
    contexts as in the cavity batches."""
    cs = [(G.Mesh.channel(60, 20, [(15.0, 10.4, 4.0)]),
           dict(BASE, uavg=0.04, viscosity=0.04, inlet_profile=1, outlet_profile=o, rho_out=1.0,
                collision_model=3))
          for o in (1, 2, 4)]
    b = G.Batch(cs, precision=precision)
    b.set_rest()
    b.run(60, check_every=20, tol=-1.0)
    for c, (mesh, params) in enumerate(cs):
        got = b.fields(c)
        want = single(mesh, params, G.PRECISIONS[precision], 61)
        speed = np.sqrt(want["u"] ** 2 + want["v"] ** 2).max()
        err = np.sqrt((got["u"] - want["u"]) ** 2 + (got["v"] - want["v"]) ** 2).max() / speed
        assert err <= 1e-5, (c, err)
        assert np.abs(got["rho"] - want["rho"]).max() <= 1e-6
    b.close()


@pytest.mark.parametrize("precision", ["fp32", "fp16dev"])
def test_launch_options_do_not_change_results(precision):
    """The boundary-node pass walks its list grid-stride (one thread per entry
    or a few blocks per multiprocessor) and the bulk pass's L2 prefetch is a
    hint: the arithmetic per node is the same, so the fields are bitwise equal."""
    cs = batch_cases(3)
    ref = None
    for bps, pf in ((0, False), (1, False), (2, True), (8, True), (0, True)):
        b = G.Batch(cs, precision=precision)
        b.set_tile(1)
        b.set_launch(bps, pf)
        b.set_rest()
        r = b.run(60, check_every=30, tol=-1.0)
        assert (r["steps"] == 60).all()
        f = [b.fields(c) for c in range(len(cs))]
        b.close()
        if ref is None:
            ref = f
            continue
        for c in range(len(cs)):
            for k in ("rho", "u", "v"):
                assert np.array_equal(f[c][k], ref[c][k]), (bps, pf, c, k)
