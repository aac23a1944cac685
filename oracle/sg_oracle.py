"""TEST INFRASTRUCTURE ONLY: FP64 numpy restatement of the surrogate network
(liblbm_gb300's lbm_sg_*), forward and backward, with the library's parameter
layout, for the GPU gradient checks.

With ``bf16=True`` it rounds exactly where the GPU stores BF16 (weights,
layer outputs, upsampled/pooled tensors, gradients handed between layers), so
the remaining difference is only the order of the FP32 accumulations.
"""
import numpy as np

GBK = 32


def rup(x, a):
    return (x + a - 1) // a * a


def to_bf16(x):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    f = np.asarray(x, np.float32)
    b = f.view(np.uint32).astype(np.uint64)
    rounded = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    out = rounded.astype(np.uint32).view(np.float32).astype(np.float64)
    return np.where(np.isnan(f), np.nan, out)


def layer_table(cin, cout, b):
    """(cin, cout, taps, relu) of the 15 layers in forward order."""
    return [(cin, b, 9, 1), (b, b, 9, 1), (b, 2 * b, 9, 1), (2 * b, 2 * b, 9, 1),
            (2 * b, 4 * b, 9, 1), (4 * b, 4 * b, 9, 1), (4 * b, 4 * b, 9, 1),
            (4 * b, 4 * b, 9, 1), (8 * b, 4 * b, 9, 1), (4 * b, 4 * b, 9, 1),
            (6 * b, 2 * b, 9, 1), (2 * b, 2 * b, 9, 1), (3 * b, b, 9, 1), (b, b, 9, 1),
            (b, cout, 1, 0)]


def unpack(params, cin, cout, b):
    out, off = [], 0
    for ci, co, taps, relu in layer_table(cin, cout, b):
        kp = rup(taps * ci, GBK)
        W = params[off:off + co * kp].reshape(co, kp)[:, :taps * ci]
        off += co * kp
        bias = params[off:off + co]
        off += co
        out.append((W.reshape(co, taps, ci), bias, taps, relu))
    return out


def pack_grads(grads, cin, cout, b):
    flat = []
    for (gW, gb), (ci, co, taps, relu) in zip(grads, layer_table(cin, cout, b)):
        kp = rup(taps * ci, GBK)
        full = np.zeros((co, kp))
        full[:, :taps * ci] = gW.reshape(co, taps * ci)
        flat += [full.ravel(), gb]
    return np.concatenate(flat)


def im2col(X, taps):
    if taps == 1:
        return X[:, :, :, None, :]
    B, H, W, C = X.shape
    P = np.pad(X, ((0, 0), (1, 1), (1, 1), (0, 0)))
    cols = [P[:, 1 + dy:1 + dy + H, 1 + dx:1 + dx + W, :] for dy in (-1, 0, 1) for dx in (-1, 0, 1)]
    return np.stack(cols, axis=3)  # B,H,W,9,C with tap r = (dy+1)*3 + (dx+1)


def col2im(G, taps, shape):
    """Adjoint of im2col: scatter-add G[B,H,W,taps,C] back to X's shape."""
    if taps == 1:
        return G[:, :, :, 0, :]
    B, H, W, C = shape
    P = np.zeros((B, H + 2, W + 2, C))
    r = 0
    for dy in (-1, 0, 1):
        for dx in (-1, 0, 1):
            P[:, 1 + dy:1 + dy + H, 1 + dx:1 + dx + W, :] += G[:, :, :, r, :]
            r += 1
    return P[:, 1:H + 1, 1:W + 1, :]


def pool(X):
    B, H, W, C = X.shape
    return X.reshape(B, H // 2, 2, W // 2, 2, C).mean(axis=(2, 4))


def pool_back(G, shape):
    return np.repeat(np.repeat(G, 2, axis=1), 2, axis=2) * 0.25


def up(X):
    return np.repeat(np.repeat(X, 2, axis=1), 2, axis=2)


def up_back(G):
    B, H, W, C = G.shape
    return G.reshape(B, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4))


class Net:
    def __init__(self, params, cin, cout, base, bf16=False):
        self.cin, self.cout, self.base = cin, cout, base
        self.rb = to_bf16 if bf16 else (lambda a: np.asarray(a, np.float64))
        self.L = unpack(np.asarray(params, np.float64), cin, cout, base)

    def conv(self, i, X):
        W, b, taps, relu = self.L[i]
        A = im2col(X, taps)
        Z = np.einsum("bhwrc,orc->bhwo", A, self.rb(W), optimize=True) + b
        Y = self.rb(np.maximum(Z, 0) if relu else Z)
        self.cache[i] = (X, Y)
        return Y

    def forward(self, x):
        rb = self.rb
        self.cache = {}
        X = rb(x)
        e0 = self.conv(1, self.conv(0, X))
        e1 = self.conv(3, self.conv(2, rb(pool(e0))))
        e2 = self.conv(5, self.conv(4, rb(pool(e1))))
        e3 = self.conv(7, self.conv(6, rb(pool(e2))))
        d2 = self.conv(9, self.conv(8, np.concatenate([up(e3), e2], axis=3)))
        d1 = self.conv(11, self.conv(10, np.concatenate([up(d2), e1], axis=3)))
        d0 = self.conv(13, self.conv(12, np.concatenate([up(d1), e0], axis=3)))
        return self.conv(14, d0)

    def conv_back(self, i, G, need_dx=True):
        W, b, taps, relu = self.L[i]
        X, Y = self.cache[i]
        if relu:
            G = np.where(Y > 0, G, 0.0)
        gb = G.sum(axis=(0, 1, 2))
        A = im2col(X, taps)
        gW = np.einsum("bhwo,bhwrc->orc", G, A, optimize=True)
        gX = None
        if need_dx:
            gX = self.rb(col2im(np.einsum("bhwo,orc->bhwrc", G, self.rb(W), optimize=True), taps, X.shape))
        return gX, (gW, gb)

    def loss_grads(self, x, t, m=None, coarse=None):
        """Loss, output and flat gradients; coarse = (weight, block) adds the
        block-mean term of lbm_sg_loss_grads."""
        rb = self.rb
        y = self.forward(x)
        B, H, W, C = y.shape
        m = np.ones((B, H, W)) if m is None else np.asarray(m, np.float64)
        inv = 1.0 / (m.sum() * C)
        d = y - t
        loss = float((m[..., None] * d * d).sum() * inv)
        G = rb(2 * inv * m[..., None] * d)
        if coarse is not None and coarse[0] > 0:
            lam, s = coarse
            blk = lambda a: a.reshape(B, H // s, s, W // s, s, *a.shape[3:]).sum(axis=(2, 4))
            w = blk(m)
            ok = w > 0
            D = np.where(ok[..., None], (blk(m[..., None] * y) - blk(m[..., None] * t)) /
                         np.where(ok, w, 1)[..., None], 0.0)
            nb = ok.sum()
            loss += float(lam * (D[ok] ** 2).sum() / (nb * C))
            up = lambda a: np.repeat(np.repeat(a, s, axis=1), s, axis=2)
            g = lam * 2 * up(D) * m[..., None] / up(np.where(ok, w, 1))[..., None] / (nb * C)
            G = rb(G + np.where(up(ok)[..., None], g, 0.0))
        grads = [None] * 15
        b = self.base
        G, grads[14] = self.conv_back(14, G)
        G, grads[13] = self.conv_back(13, G)
        G, grads[12] = self.conv_back(12, G)
        g_d1, g_e0 = rb(up_back(G[..., :2 * b])), G[..., 2 * b:]
        G, grads[11] = self.conv_back(11, g_d1)
        G, grads[10] = self.conv_back(10, G)
        g_d2, g_e1 = rb(up_back(G[..., :4 * b])), G[..., 4 * b:]
        G, grads[9] = self.conv_back(9, g_d2)
        G, grads[8] = self.conv_back(8, G)
        g_e3, g_e2 = rb(up_back(G[..., :4 * b])), G[..., 4 * b:]
        G, grads[7] = self.conv_back(7, g_e3)
        G, grads[6] = self.conv_back(6, G)
        g_e2 = rb(g_e2 + pool_back(G, None))
        G, grads[5] = self.conv_back(5, g_e2)
        G, grads[4] = self.conv_back(4, G)
        g_e1 = rb(g_e1 + pool_back(G, None))
        G, grads[3] = self.conv_back(3, g_e1)
        G, grads[2] = self.conv_back(2, G)
        g_e0 = rb(g_e0 + pool_back(G, None))
        G, grads[1] = self.conv_back(1, g_e0)
        _, grads[0] = self.conv_back(0, G, need_dx=False)
        return loss, y, pack_grads(grads, self.cin, self.cout, self.base)


def init_params(cin, cout, base, seed=0):
    """He-normal weights in the library's layout (zero padding and biases)."""
    rng = np.random.default_rng(seed)
    flat = []
    for ci, co, taps, relu in layer_table(cin, cout, base):
        kp = rup(taps * ci, GBK)
        W = np.zeros((co, kp))
        W[:, :taps * ci] = rng.normal(0, np.sqrt(2.0 / (taps * ci)), (co, taps * ci))
        flat += [W.ravel(), np.zeros(co)]
    return np.concatenate(flat)
