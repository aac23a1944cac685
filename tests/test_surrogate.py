"""The warm-start network: the FP64 oracle against torch autograd (CPU), and
the library's BF16 tensor-core forward/backward against the oracle (GPU)."""
import numpy as np
import pytest

from oracle import sg_oracle as SO

CIN, COUT, BASE, H = 4, 3, 8, 16


def sample(seed=1, B=2, h=H, cin=CIN):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(B, h, h, cin))
    t = rng.normal(size=(B, h, h, COUT)) * 0.5
    m = (rng.random((B, h, h)) > 0.2).astype(np.float64)
    return x, t, m


def torch_grads(params, x, t, m, coarse=None):
    torch = pytest.importorskip("torch")
    F = torch.nn.functional
    P = torch.tensor(params, dtype=torch.float64, requires_grad=True)
    off, layers = 0, []
    for ci, co, taps, relu in SO.layer_table(CIN, COUT, BASE):
        kp = SO.rup(taps * ci, 32)
        W = P[off:off + co * kp].reshape(co, kp)[:, :taps * ci]
        off += co * kp
        b = P[off:off + co]
        off += co
        k = 3 if taps == 9 else 1
        Wt = W.reshape(co, k, k, ci).permute(0, 3, 1, 2)
        layers.append((Wt, b, k, relu))

    def conv(i, X):
        Wt, b, k, relu = layers[i]
        Y = F.conv2d(X, Wt, b, padding=k // 2)
        return F.relu(Y) if relu else Y

    X = torch.tensor(x).permute(0, 3, 1, 2)
    pool = lambda a: F.avg_pool2d(a, 2)
    up = lambda a: F.interpolate(a, scale_factor=2, mode="nearest")
    e0 = conv(1, conv(0, X))
    e1 = conv(3, conv(2, pool(e0)))
    e2 = conv(5, conv(4, pool(e1)))
    e3 = conv(7, conv(6, pool(e2)))
    d2 = conv(9, conv(8, torch.cat([up(e3), e2], 1)))
    d1 = conv(11, conv(10, torch.cat([up(d2), e1], 1)))
    d0 = conv(13, conv(12, torch.cat([up(d1), e0], 1)))
    y = conv(14, d0).permute(0, 2, 3, 1)
    M = torch.tensor(m)[..., None]
    T = torch.tensor(t)
    loss = (M * (y - T) ** 2).sum() / (M.sum() * COUT)
    if coarse is not None:
        lam, s = coarse
        B, Hh, Ww, C = y.shape
        blk = lambda a: a.reshape(B, Hh // s, s, Ww // s, s, -1).sum(dim=(2, 4))
        w = blk(M)
        ok = (w > 0).squeeze(-1)
        D = (blk(M * y) - blk(M * T)) / torch.where(w > 0, w, torch.ones_like(w))
        loss = loss + lam * (D[ok] ** 2).sum() / (ok.sum() * C)
    loss.backward()
    return loss.item(), y.detach().numpy(), P.grad.numpy()


def test_oracle_matches_torch_autograd():
    params = SO.init_params(CIN, COUT, BASE, seed=3)
    x, t, m = sample()
    loss, y, g = SO.Net(params, CIN, COUT, BASE).loss_grads(x, t, m)
    tl, ty, tg = torch_grads(params, x, t, m)
    assert abs(loss - tl) <= 1e-12 * abs(tl)
    assert np.abs(y - ty).max() <= 1e-12 * np.abs(ty).max()
    assert np.abs(g - tg).max() <= 1e-10 * np.abs(tg).max()


def test_oracle_coarse_term_matches_torch_autograd():
    """The block-mean loss term of the oracle (mirrored by the GPU kernels)."""
    params = SO.init_params(CIN, COUT, BASE, seed=4)
    x, t, m = sample(seed=5)
    m[0, :4, :4] = 0.0  # one block without fluid
    loss, y, g = SO.Net(params, CIN, COUT, BASE).loss_grads(x, t, m, coarse=(2.0, 4))
    tl, ty, tg = torch_grads(params, x, t, m, coarse=(2.0, 4))
    assert abs(loss - tl) <= 1e-12 * abs(tl)
    assert np.abs(g - tg).max() <= 1e-10 * np.abs(tg).max()


def test_bf16_rounding_helper():
    v = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 0.0])
    r = SO.to_bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0  # tie to even
    assert r[2] == 1.0078125
    assert abs(r[3] - -3.140625) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("products", ["tcgen05", "mma"])
@pytest.mark.parametrize("cin,base,h,coarse", [(CIN, BASE, H, 0.0), (7, 32, 32, 0.0),
                                               (8, 32, 32, 0.0), (CIN, BASE, H, 2.0),
                                               (8, 32, 64, 0.0)])
def test_gpu_gradients_match_oracle(cin, base, h, coarse, products):
    """4 or 7 input channels: the first layer's products use an explicit im2col
    in memory; every layer with a multiple of 8 channels (all of them at 8
    inputs) uses the implicit-im2col forward/input-gradient products and the
    pixel-split weight-gradient kernel, including K padded beyond taps*C.
    products="tcgen05" runs those on the 5th-generation tensor cores (tensor
    memory accumulators, 128 x N x 16 MMAs), "mma" on mma.sync."""
    import parallellbmcranfield_gb300 as G

    s = G.Surrogate(height=h, width=h, in_channels=cin, out_channels=COUT, base=base, max_batch=2,
                    seed=5, coarse_weight=coarse, coarse_block=4, products=products)
    params = s.params().astype(np.float64)
    x, t, m = sample(seed=2, h=h, cin=cin)
    loss, g = s.loss_grads(x, t, m)
    oloss, oy, og = SO.Net(params, cin, COUT, base, bf16=True).loss_grads(
        x, t, m, coarse=(coarse, 4) if coarse else None)
    y = s.forward(x)
    assert np.abs(y - oy).max() <= 2e-2 * np.abs(oy).max()
    assert abs(loss - oloss) <= 2e-2 * oloss
    # per-layer relative L2 error of the weight gradients
    off = 0
    for ci, co, taps, relu in SO.layer_table(cin, COUT, base):
        n = co * SO.rup(taps * ci, 32) + co
        a, b = g[off:off + n], og[off:off + n]
        off += n
        err = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        # BF16 values are rounded in a different accumulation order on the GPU
        # than in the oracle, so rounding decisions differ and the difference
        # grows along the backward chain (1-3 % in the deepest layers); a wrong
        # product gives O(1) errors
        assert err <= 5e-2, (ci, co, err)
    s.close()


@pytest.mark.gpu
def test_gpu_training_reduces_loss():
    import parallellbmcranfield_gb300 as G

    s = G.Surrogate(height=32, width=32, in_channels=CIN, out_channels=COUT, base=BASE,
                    max_batch=4, lr=3e-3, seed=1)
    rng = np.random.default_rng(0)
    x = rng.normal(size=(16, 32, 32, CIN)).astype(np.float32)
    # a smooth target that depends on the input: learnable
    t = np.stack([np.tanh(x[..., 0]), 0.5 * x[..., 1], x[..., 2] * x[..., 3] * 0.1], -1)
    m = np.ones((16, 32, 32), np.float32)
    s.set_dataset(x, t, m)
    first = s.train(np.arange(16), 4)
    for _ in range(60):
        last = s.train(rng.permutation(16), 4)
    assert last < 0.5 * first, (first, last)
    s.close()


@pytest.mark.gpu
def test_pipeline_small(tmp_path):
    """Data generation -> training -> warm/cold comparison end to end, tiny."""
    from parallellbmcranfield_gb300 import surrogate as S

    rep = S.main(["--cavities", "3", "--channels", "3", "--max-steps", "30000",
                  "--check-every", "100", "--gen-tol", "2e-4", "--tol", "2e-4", "--epochs", "2",
                  "--batch", "2", "--eval", "2", "--out", str(tmp_path / "r.json")])
    assert rep["cases"] == 6 and rep["steady"] == 6, rep
    assert np.isfinite(rep["training"]["loss_last"])
    assert rep["training"]["cases"] == 5  # 6 cases: 5 train, 1 test
    ev = rep["warm_vs_cold"]
    assert ev["cases"] == 1 and ev["converged_cold"] == 1 and ev["converged_warm"] == 1


@pytest.mark.gpu
def test_warm_start_gains_over_cold_start(tmp_path):
    """What the trained network gains: cavities at Re 100-400 (steady within a
    few 10^4 steps), trained on the GPU, then the held-out cases iterated to
    the same tolerance from rest and from the prediction.  The warm starts must
    converge in clearly fewer steps, to fields as close to the reference."""
    from parallellbmcranfield_gb300 import surrogate as S

    rep = S.main(["--cavities", "30", "--channels", "0", "--cavity-re-max", "400",
                  "--epochs", "300", "--batch", "4", "--eval", "8", "--lr", "2e-3",
                  "--out", str(tmp_path / "r.json")])
    ev = rep["warm_vs_cold"]
    assert ev["cases"] >= 4 and ev["converged_cold"] == ev["converged_warm"] == ev["cases"], ev
    assert ev["work_ratio"] >= 1.2, ev  # about 1.25 after 80 epochs
    # at the same tolerance the warm results sit closer to the converged fields
    assert ev["err_warm_median"] <= ev["err_cold_median"], ev


def test_pipeline_host_logic():
    """Case draws, input maps and the prediction -> initial-field mapping (CPU)."""
    from parallellbmcranfield_gb300 import surrogate as S

    cases = S.make_cases(4, 4, seed=3)
    assert [c["kind"] for c in cases] == ["cavity"] * 4 + ["channel"] * 4
    for c in cases:
        assert 0.05 <= c["U"] <= 0.1
        assert c["params"]["viscosity"] > 0
        if c["kind"] == "cavity":
            assert 100 <= c["re"] <= 5000
            assert abs(c["params"]["viscosity"] - c["U"] * S.SIDE / c["re"]) < 1e-12
        else:
            assert 0.05 <= c["params"]["viscosity"] <= 0.4
            assert 1 <= len(c["spec"][3]) <= 3
    for c in (cases[0], cases[4]):
        mesh = S.build_mesh(c["spec"])
        n, m = mesh.shape
        x, mask = S.features(c, mesh)
        assert x.shape == (S.GRID, S.GRID, S.IN_CH) and mask.shape == (S.GRID, S.GRID)
        assert set(np.unique(mask)) <= {0.0, 1.0}
        # distance map: zero on solid cells, >= 1/32 on fluid cells
        assert (x[..., 6][mask == 0] == 0).all() and (x[..., 6][mask == 1] >= 1 / 32 - 1e-7).all()
        assert x[0, 5, 4] == np.float32(5 / 256) and x[7, 0, 5] == np.float32(7 / 256)
        g = x[..., 7]
        if c["kind"] == "cavity":
            assert (g == 0).all()
        else:
            # zero on solid cells; in every column the gaps carry the inlet flow rate
            assert (g[mask == 0] == 0).all()
            q = g * c["U"]
            flux = q.sum(axis=0)
            assert np.allclose(flux[1:-1], c["params"]["uavg"] * mask[:, 1].sum(), rtol=1e-3)
        # targets -> prediction -> fields round trip on fluid cells
        rng = np.random.default_rng(0)
        f = {k: rng.normal(size=n * m) * 0.01 for k in ("rho", "u", "v")}
        f["rho"] = 1.0 + f["rho"] * c["U"] ** 2  # (rho - 1) / U^2 within the clip
        y = S.targets(c, f, n, m, x)
        rho, u, v = S.fields_from_prediction(c, y, n, m, mask, x)
        fl = np.zeros((m, n), bool)
        fl[:S.GRID, :S.GRID] = mask > 0
        # float32 targets of O(1) magnitude: absolute round-off ~1e-7 U
        assert np.allclose(u.reshape(m, n)[fl], f["u"].reshape(m, n)[fl], rtol=1e-5, atol=1e-7)
        assert np.allclose(v.reshape(m, n)[fl], f["v"].reshape(m, n)[fl], rtol=1e-5, atol=1e-7)
        r = rho.reshape(m, n)[fl]
        if c["kind"] == "cavity":  # closed box: mean density shifted to the cold start's 1
            assert abs(r.mean() - 1.0) < 1e-12
        else:
            assert np.allclose(r, f["rho"].reshape(m, n)[fl], rtol=0, atol=1e-6)
        assert (u.reshape(m, n)[~fl] == 0).all() and (rho.reshape(m, n)[~fl] == 1).all()
    # mirrored channel: twice is the identity, v changes sign, position maps stay
    rng = np.random.default_rng(1)
    x = rng.normal(size=(S.GRID, S.GRID, S.IN_CH)).astype(np.float32)
    y = rng.normal(size=(S.GRID, S.GRID, 3)).astype(np.float32)
    m = (rng.random((S.GRID, S.GRID)) > 0.5).astype(np.float32)
    xf, yf, mf = S.flip_channel(x, y, m)
    assert (xf[..., 4:6] == x[..., 4:6]).all() and (xf[3, :, 0] == x[S.GRID - 4, :, 0]).all()
    assert (yf[3, :, 2] == -y[S.GRID - 4, :, 2]).all() and (mf[3] == m[S.GRID - 4]).all()
    x2, y2, m2 = S.flip_channel(xf, yf, mf)
    assert (x2 == x).all() and (y2 == y).all() and (m2 == m).all()
    assert S.cosine_lr(1e-3, 2e-5, 0, 10) == 1e-3
    assert abs(S.cosine_lr(1e-3, 2e-5, 10, 10) - 2e-5) < 1e-12


def test_config_validation_on_the_host():
    """Bad network shapes are refused before any device work (CPU)."""
    import parallellbmcranfield_gb300 as G

    bad = [dict(height=30, width=32), dict(base=12), dict(out_channels=9),
           dict(coarse_weight=1.0, coarse_block=5), dict(coarse_weight=-1.0)]
    for kw in bad:
        args = dict(height=32, width=32, in_channels=4, out_channels=3, base=8, max_batch=2)
        args.update(kw)
        with pytest.raises(G.LbmError) as e:
            G.Surrogate(**args)
        assert e.value.status == G.LBM_INVALID, kw


def test_gap_flow_of_an_empty_channel_is_the_inlet_parabola():
    """Without cylinders every column is one gap of the full width: the
    estimate is the parabolic profile with peak 1.5 x the mean speed (CPU)."""
    from parallellbmcranfield_gb300 import surrogate as S

    umax = 0.08
    case = dict(kind="channel", U=umax, params=dict(uavg=umax / 1.5))
    fl = np.zeros((S.GRID, S.GRID), np.float32)
    fl[1:-1, 1:-1] = 1.0
    g = S.gap_flow(case, fl)
    h = S.GRID - 2
    s = (np.arange(h) + 0.5) / h
    want = 6.0 * (umax / 1.5) * s * (1 - s) / umax
    assert np.allclose(g[1:-1, 128], want, rtol=1e-6)
    assert abs(g[1:-1, 128].max() - 1.0) < 1e-3  # peak = umax
    assert (g[0] == 0).all() and (g[:, 0] == 0).all()


@pytest.mark.gpu
@pytest.mark.parametrize("tc", ["tcgen05", "tcgen05-1seg", "tcgen05-gather"])
@pytest.mark.parametrize("h,B", [(64, 2), (256, 1)])
def test_tcgen05_and_mma_products_agree(tc, h, B):
    """The tcgen05 product paths against mma.sync at base width 32: at 64 x 64
    every layer takes the im2col gather (tile widths 32, 64, 128, several K
    tiles); at 256 x 256 the 3x3 layers of levels 0 and 1 (W 256 and 128, C a
    multiple of 32, N 32 or 64) take the TMA-fed halo-tile form with
    "tcgen05" (four row segments per convolution block) and "tcgen05-1seg"
    (one), the gather with "tcgen05-gather".  Forward outputs and gradients
    agree to the BF16 rounding of the activations."""
    import parallellbmcranfield_gb300 as G

    x, t, m = sample(seed=9, B=B, h=h, cin=8)
    out = {}
    for products in (tc, "mma"):
        s = G.Surrogate(height=h, width=h, in_channels=8, out_channels=COUT, base=32,
                        max_batch=B, seed=11, products=products)
        loss, g = s.loss_grads(x, t, m)
        out[products] = (s.forward(x), loss, g)
        s.close()
    (ya, la, ga), (yb, lb, gb) = out[tc], out["mma"]
    assert np.abs(ya - yb).max() <= 1e-2 * np.abs(yb).max()
    assert abs(la - lb) <= 1e-2 * lb
    assert np.linalg.norm(ga - gb) <= 3e-2 * np.linalg.norm(gb)
