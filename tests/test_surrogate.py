"""The warm-start network: the FP64 oracle against torch autograd (CPU), and
the library's BF16 tensor-core forward/backward against the oracle (GPU)."""
import numpy as np
import pytest

from oracle import sg_oracle as SO

CIN, COUT, BASE, H = 4, 3, 8, 16


def sample(seed=1, B=2):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(B, H, H, CIN))
    t = rng.normal(size=(B, H, H, COUT)) * 0.5
    m = (rng.random((B, H, H)) > 0.2).astype(np.float64)
    return x, t, m


def torch_grads(params, x, t, m):
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
    loss = (M * (y - torch.tensor(t)) ** 2).sum() / (M.sum() * COUT)
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


def test_bf16_rounding_helper():
    v = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 0.0])
    r = SO.to_bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0  # tie to even
    assert r[2] == 1.0078125
    assert abs(r[3] - -3.140625) < 1e-12


@pytest.mark.gpu
def test_gpu_gradients_match_oracle():
    import parallellbmcranfield_gb300 as G

    s = G.Surrogate(height=H, width=H, in_channels=CIN, out_channels=COUT, base=BASE, max_batch=2,
                    seed=5)
    params = s.params().astype(np.float64)
    x, t, m = sample(seed=2)
    loss, g = s.loss_grads(x, t, m)
    oloss, oy, og = SO.Net(params, CIN, COUT, BASE, bf16=True).loss_grads(x, t, m)
    y = s.forward(x)
    assert np.abs(y - oy).max() <= 2e-2 * np.abs(oy).max()
    assert abs(loss - oloss) <= 2e-2 * oloss
    # per-layer relative L2 error of the weight gradients
    off = 0
    for ci, co, taps, relu in SO.layer_table(CIN, COUT, BASE):
        n = co * SO.rup(taps * ci, 32) + co
        a, b = g[off:off + n], og[off:off + n]
        off += n
        err = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        assert err <= 3e-2, (ci, co, err)
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

    rep = S.main(["--cavities", "3", "--channels", "3", "--max-steps", "3000",
                  "--check-every", "500", "--epochs", "2", "--batch", "2", "--eval", "2",
                  "--out", str(tmp_path / "r.json")])
    assert rep["cases"] == 6
    assert np.isfinite(rep["training"]["loss_last"])
    assert rep["warm_vs_cold"]["cases"] == 1  # 6 cases: 5 train, 1 test
