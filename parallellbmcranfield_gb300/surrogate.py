"""Surrogate warm start: steady fields generated by the batched solver, the
encoder-decoder trained on them with the library's own BF16 kernels, and a
warm-vs-cold comparison of the wall time to du_rel <= tol (du_rel: relative
change of (u, v) per step over the check interval).

Cases (256 x 256 node grids, MRT, FP32 storage, curved/half-way walls):
  * lid-driven cavities of 254^2 fluid cells, Re log-uniform in [100, 5000],
    lid speed U uniform in [0.05, 0.1] (nu = U * 254 / Re);
  * channels of 254 x 254 fluid cells with 1-3 non-overlapping cylinders of
    diameter 16-64, parabolic inlet (peak U uniform in [0.05, 0.1]),
    constant-pressure outlet, nu log-uniform in [0.05, 0.4] (Re on the mean
    inlet speed and the largest diameter: about 1-90).
Network input (8 maps): fluid mask, velocity-boundary cells, log(Re)/log(5000),
U / 0.1, x / 256, y / 256, the distance to the nearest solid cell / 32 (these
three give every cell its position, which 3x3 convolutions with zero padding do
not see beyond their receptive field) and a gap-flow estimate g / U (channels:
the inlet flow rate split over the fluid gaps of each column in proportion to
gap width cubed, each gap carrying a parabolic profile; cavities: 0).  Output
(3 maps): clip((rho - 1) / U^2, -8, 8) / 10, (u - g) / U, v / U on fluid cells
(the clip keeps the pressure peaks at the lid corners from dominating the loss
and the factor 1/10 weights the squared error towards the velocity, which sets
the warm start's slow modes; the network corrects the gap-flow estimate rather
than rebuilding it).

The training targets are run to a tighter tolerance (gen_tol) than the
comparison (tol) and serve as the converged reference against which both the
cold and the warm result are measured.  Cases whose generation run does not
reach gen_tol (unsteady wakes, the slowest cavities) neither train nor enter
the comparison: they have no steady field to predict or to reach.

    python -m parallellbmcranfield_gb300.surrogate --cavities 700 --channels 1300 --out report.json
"""
import argparse
import json
import math
import time

import numpy as np

import parallellbmcranfield_gb300 as G

GRID = 256
SIDE = GRID - 2
IN_CH = 8
RHO_CLIP, RHO_SCALE = 8.0, 0.1


def make_cases(n_cav, n_ch, seed, cavity_re=(100.0, 5000.0)):
    rng = np.random.default_rng(seed)
    cases = []
    for _ in range(n_cav):
        re = float(np.exp(rng.uniform(np.log(cavity_re[0]), np.log(cavity_re[1]))))
        U = float(rng.uniform(0.05, 0.1))
        nu = U * SIDE / re
        cases.append(dict(kind="cavity", re=re, U=U, spec=("cavity", SIDE),
                          params=dict(uavg=U, vavg=0.0, rho_ini=1.0, viscosity=nu,
                                      inlet_profile=2, collision_model=3, curved_boundaries=1,
                                      outlet_profile=2)))
    for _ in range(n_ch):
        k = int(rng.integers(1, 4))
        cyl = []
        while len(cyl) < k:
            d = float(rng.uniform(16, 64))
            cx = float(rng.uniform(50, 200))
            cy = float(rng.uniform(d / 2 + 10, SIDE - d / 2 - 10))
            if all((cx - a) ** 2 + (cy - b) ** 2 > (d / 2 + r + 6) ** 2 for a, b, r in cyl):
                cyl.append((cx, cy + 0.37, d / 2))
        umax = float(rng.uniform(0.05, 0.1))
        nu = float(np.exp(rng.uniform(np.log(0.05), np.log(0.4))))
        dmax = 2 * max(r for _, _, r in cyl)
        re = (umax / 1.5) * dmax / nu
        cases.append(dict(kind="channel", re=re, U=umax, spec=("channel", SIDE, SIDE, cyl),
                          params=dict(uavg=umax / 1.5, vavg=0.0, rho_ini=1.0, viscosity=nu,
                                      inlet_profile=1, collision_model=3, curved_boundaries=1,
                                      outlet_profile=4, rho_out=1.0)))
    return cases


def build_mesh(spec):
    if spec[0] == "cavity":
        return G.Mesh.cavity(spec[1])
    return G.Mesh.channel(spec[1], spec[2], spec[3])


def gap_flow(case, fl):
    """Gap-flow estimate of u / U on a GRID x GRID fluid mask (rows = y)."""
    g = np.zeros((GRID, GRID), np.float32)
    if case["kind"] != "channel":
        return g
    u_mean = case["params"]["uavg"]
    q = u_mean * float(fl[:, 1].sum())  # inlet flow rate per unit depth
    for x in range(GRID):
        col = fl[:, x] > 0
        if not col.any():
            continue
        edges = np.flatnonzero(np.diff(np.concatenate(([0], col.astype(np.int8), [0]))))
        starts, ends = edges[0::2], edges[1::2]
        h = (ends - starts).astype(np.float64)
        share = q * h ** 3 / (h ** 3).sum()
        for y0, hh, qq in zip(starts, h, share):
            s = (np.arange(int(hh)) + 0.5) / hh
            g[y0:y0 + int(hh), x] = 6.0 * (qq / hh) * s * (1.0 - s) / case["U"]
    return g


def features(case, mesh):
    """Input maps (GRID, GRID, IN_CH) and the fluid mask (GRID, GRID)."""
    from scipy.ndimage import distance_transform_edt
    n, m = mesh.shape
    fluid = np.zeros((m, n), np.float32)
    ij = mesh.nodes[:, :2].astype(np.int64)
    fluid[ij[:, 1], ij[:, 0]] = mesh.nodes[:, 4]
    bc = np.zeros((m, n), np.float32)
    vel = mesh.conns[mesh.conns[:, 3] == 2]
    bc[vel[:, 1].astype(np.int64), vel[:, 0].astype(np.int64)] = 1.0
    fl = fluid[:GRID, :GRID]
    x = np.zeros((GRID, GRID, IN_CH), np.float32)
    x[..., 0] = fl
    x[..., 1] = bc[:GRID, :GRID]
    x[..., 2] = np.log(case["re"]) / np.log(5000.0)
    x[..., 3] = case["U"] / 0.1
    x[..., 4] = (np.arange(GRID, dtype=np.float32) / GRID)[None, :]
    x[..., 5] = (np.arange(GRID, dtype=np.float32) / GRID)[:, None]
    x[..., 6] = distance_transform_edt(fl > 0) / 32.0
    x[..., 7] = gap_flow(case, fl)
    return x, fl.copy()


def targets(case, fields, n, m, x):
    """Network targets of a steady field; x: the case's input maps (the u
    target is relative to the gap-flow estimate x[..., 7])."""
    U = case["U"]
    t = np.zeros((GRID, GRID, 3), np.float32)
    rho = (fields["rho"].reshape(m, n)[:GRID, :GRID] - 1.0) / (U * U)
    t[..., 0] = np.clip(rho, -RHO_CLIP, RHO_CLIP) * RHO_SCALE
    t[..., 1] = fields["u"].reshape(m, n)[:GRID, :GRID] / U - x[..., 7]
    t[..., 2] = fields["v"].reshape(m, n)[:GRID, :GRID] / U
    return t


def fields_from_prediction(case, y, n, m, mask, x):
    """rho, u, v arrays of the case's n*m grid from a network output (x: the
    case's input maps).  In a closed cavity the mass is conserved, so the
    predicted density is shifted to the mean the cold start has (1); open
    channels keep the prediction."""
    U = case["U"]
    rho, u, v = np.ones((m, n)), np.zeros((m, n)), np.zeros((m, n))
    fl = mask > 0
    r = 1.0 + y[..., 0][fl].astype(np.float64) * (U * U / RHO_SCALE)
    if case["kind"] == "cavity":
        r += 1.0 - r.mean()
    rho[:GRID, :GRID][fl] = r
    u[:GRID, :GRID][fl] = (y[..., 1][fl] + x[..., 7][fl]) * U
    v[:GRID, :GRID][fl] = y[..., 2][fl] * U
    return rho.ravel(), u.ravel(), v.ravel()


def run_batch(cases, meshes, max_steps, check_every, tol, init=None):
    b = G.Batch([(m, c["params"]) for c, m in zip(cases, meshes)], precision="fp32")
    b.autotune(3)
    b.set_rest()
    if init is not None:
        for i, (rho, u, v) in enumerate(init):
            b.set_state(i, rho, u, v)
    r = b.run(max_steps, check_every, tol, raise_on_nan=False)
    return b, r


def generate(cases, max_steps, check_every, tol):
    meshes = [build_mesh(c["spec"]) for c in cases]
    t0 = time.perf_counter()
    b, r = run_batch(cases, meshes, max_steps, check_every, tol)
    gen_s = time.perf_counter() - t0
    X, Y, M = [], [], []
    for i, (c, mesh) in enumerate(zip(cases, meshes)):
        x, mask = features(c, mesh)
        n, m = mesh.shape
        f = b.fields(i)
        X.append(x)
        Y.append(targets(c, f, n, m, x))
        M.append(mask)
    b.close()
    return meshes, np.stack(X), np.stack(Y), np.stack(M), r, gen_s


def flip_channel(x, y, m):
    """The channel mirrored top to bottom (rows j -> GRID-1-j; walls on rows 0
    and GRID-1 map onto each other): geometry maps flip, the position maps stay,
    v changes sign."""
    xf, yf = x[::-1].copy(), y[::-1].copy()
    xf[..., 4:6] = x[..., 4:6]
    yf[..., 2] = -yf[..., 2]
    return xf, yf, m[::-1].copy()


def training_set(cases, X, Y, M, train_idx, augment=True):
    """Training samples: the cases train_idx plus, with augment, every channel
    mirrored top to bottom."""
    xs, ys, ms = [X[i] for i in train_idx], [Y[i] for i in train_idx], [M[i] for i in train_idx]
    if augment:
        for i in train_idx:
            if cases[i]["kind"] == "channel":
                a, b, c = flip_channel(X[i], Y[i], M[i])
                xs.append(a)
                ys.append(b)
                ms.append(c)
    return np.stack(xs), np.stack(ys), np.stack(ms)


def cosine_lr(lr, lr_min, epoch, epochs):
    return lr_min + 0.5 * (lr - lr_min) * (1.0 + math.cos(math.pi * epoch / max(1, epochs)))


def train(X, Y, M, train_idx, epochs, batch, lr, seed, lr_min=None, weight_decay=0.0,
          coarse_weight=0.0, coarse_block=32, base=32, products="tcgen05"):
    """Adam with a cosine learning-rate schedule over the samples train_idx of
    (X, Y, M); returns the network, the mean loss of every epoch and the time."""
    if len(train_idx) == 0:
        raise ValueError("no training samples (no case reached the generation tolerance)")
    net = G.Surrogate(height=GRID, width=GRID, in_channels=X.shape[-1], out_channels=3, base=base,
                      max_batch=batch, lr=lr, seed=seed, weight_decay=weight_decay,
                      coarse_weight=coarse_weight, coarse_block=coarse_block, products=products)
    net.set_dataset(X, Y, M)
    rng = np.random.default_rng(seed)
    lr_min = lr * 0.02 if lr_min is None else lr_min
    hist = []
    t0 = time.perf_counter()
    for e in range(epochs):
        net.set_lr(cosine_lr(lr, lr_min, e, epochs))
        hist.append(net.train(rng.permutation(train_idx), batch))
    return net, hist, time.perf_counter() - t0


def masked_mse(net, X, Y, M, idx):
    y = net.forward(X[idx])
    w = M[idx][..., None]
    return float((w * (y - Y[idx]) ** 2).sum() / (w.sum() * 3)), y


def velocity_error(case, fields, n, m, y_ref, mask, x):
    """Relative L2 error of (u, v) / U against the reference target maps."""
    U = case["U"]
    fl = mask > 0
    u = (fields["u"].reshape(m, n)[:GRID, :GRID] / U)[fl]
    v = (fields["v"].reshape(m, n)[:GRID, :GRID] / U)[fl]
    ur, vr = y_ref[..., 1][fl] + x[..., 7][fl], y_ref[..., 2][fl]
    return float(np.sqrt(((u - ur) ** 2 + (v - vr) ** 2).sum() / (ur ** 2 + vr ** 2).sum()))


def evaluate(net, cases, meshes, X, Y, M, idx, max_steps, check_every, tol):
    """Cold start (rest) against warm start (network prediction) on the cases
    idx, both to du_rel <= tol in one batch each; the error of each result is
    measured against the reference targets Y.  With net None the warm start
    is seeded with the reference fields themselves (the best any prediction
    can do when it seeds f = f_eq)."""
    if len(idx) == 0:
        return dict(cases=0)
    sub = [cases[i] for i in idx]
    sub_m = [meshes[i] for i in idx]
    t0 = time.perf_counter()
    bc, rc = run_batch(sub, sub_m, max_steps, check_every, tol)
    cold_s = time.perf_counter() - t0
    err_cold = [velocity_error(cases[i], bc.fields(j), *meshes[i].shape, Y[i], M[i], X[i])
                for j, i in enumerate(idx)]
    bc.close()
    t0 = time.perf_counter()
    y = net.forward(X[idx]) if net is not None else Y[idx]
    infer_s = time.perf_counter() - t0
    init, err_pred = [], []
    for j, i in enumerate(idx):
        n, m = meshes[i].shape
        rho, u, v = fields_from_prediction(cases[i], y[j], n, m, M[i], X[i])
        init.append((rho, u, v))
        err_pred.append(velocity_error(cases[i], dict(u=u, v=v), n, m, Y[i], M[i], X[i]))
    t0 = time.perf_counter()
    bw, rw = run_batch(sub, sub_m, max_steps, check_every, tol, init=init)
    warm_s = time.perf_counter() - t0
    err_warm = [velocity_error(cases[i], bw.fields(j), *meshes[i].shape, Y[i], M[i], X[i])
                for j, i in enumerate(idx)]
    bw.close()
    both = (rc["converged"] == 1) & (rw["converged"] == 1)
    sc, sw = rc["steps"].astype(np.float64), rw["steps"].astype(np.float64)
    per_case = [dict(kind=cases[i]["kind"], re=cases[i]["re"], U=cases[i]["U"],
                     steps_cold=int(rc["steps"][j]), steps_warm=int(rw["steps"][j]),
                     conv_cold=int(rc["converged"][j]), conv_warm=int(rw["converged"][j]),
                     err_pred=err_pred[j], err_cold=err_cold[j], err_warm=err_warm[j])
                for j, i in enumerate(idx)]
    ratio = sc[both] / np.maximum(sw[both], 1) if both.any() else np.zeros(0)
    return dict(
        cases=len(idx), converged_cold=int((rc["converged"] == 1).sum()),
        converged_warm=int((rw["converged"] == 1).sum()),
        steps_cold_total=float(sc.sum()), steps_warm_total=float(sw.sum()),
        work_ratio=float(sc.sum() / max(sw.sum(), 1.0)),
        steps_ratio_mean=float(ratio.mean()) if ratio.size else None,
        steps_ratio_median=float(np.median(ratio)) if ratio.size else None,
        err_pred_median=float(np.median(err_pred)),
        err_cold_median=float(np.median(err_cold)), err_warm_median=float(np.median(err_warm)),
        err_cold_max=float(np.max(err_cold)), err_warm_max=float(np.max(err_warm)),
        wall_cold_s=cold_s, wall_warm_s=warm_s + infer_s, inference_s=infer_s,
        wall_speedup=cold_s / (warm_s + infer_s), per_case=per_case)


def train_throughput(batch=8, samples=16, epochs=3, seed=1, products="tcgen05", base=32):
    """Training samples per second of the warm-start network on random
    256 x 256 inputs (the cost does not depend on the values)."""
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(samples, GRID, GRID, IN_CH)).astype(np.float32)
    t = rng.normal(size=(samples, GRID, GRID, 3)).astype(np.float32)
    m = np.ones((samples, GRID, GRID), np.float32)
    net = G.Surrogate(height=GRID, width=GRID, in_channels=IN_CH, out_channels=3, base=base,
                      max_batch=batch, seed=seed, products=products)
    net.set_dataset(x, t, m)
    net.train(np.arange(samples), batch)  # warm-up
    t0 = time.perf_counter()
    for _ in range(epochs):
        net.train(np.arange(samples), batch)
    rate = epochs * samples / (time.perf_counter() - t0)
    net.close()
    return rate


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--cavities", type=int, default=700)
    p.add_argument("--cavity-re-max", type=float, default=5000.0)
    p.add_argument("--channels", type=int, default=1300)
    p.add_argument("--max-steps", type=int, default=600000)
    p.add_argument("--check-every", type=int, default=100)
    p.add_argument("--tol", type=float, default=1e-6, help="du_rel of the warm/cold comparison")
    p.add_argument("--gen-tol", type=float, default=1e-7, help="du_rel of the training targets")
    p.add_argument("--epochs", type=int, default=200)
    p.add_argument("--batch", type=int, default=8)
    p.add_argument("--lr", type=float, default=1e-3)
    p.add_argument("--weight-decay", type=float, default=0.01, help="AdamW decay")
    p.add_argument("--coarse-weight", type=float, default=0.0,
                   help="weight of the block-mean loss term (large-scale error)")
    p.add_argument("--coarse-block", type=int, default=32)
    p.add_argument("--eval", type=int, default=400, help="test cases in the warm/cold comparison")
    p.add_argument("--no-augment", action="store_true", help="no mirrored channels in training")
    p.add_argument("--seed", type=int, default=20240601)
    p.add_argument("--out", default=None)
    p.add_argument("--throughput", action="store_true",
                   help="only time training on random inputs (samples/s)")
    p.add_argument("--reference-start", action="store_true",
                   help="no network: seed the warm starts with the reference fields")
    p.add_argument("--products", default="tcgen05", choices=["tcgen05", "tcgen05-gather", "tcgen05-1seg", "mma"],
                   help="tensor-core path of the network's convolution products")
    p.add_argument("--base", type=int, default=32, help="channels of the first level")
    a = p.parse_args(argv)
    if a.throughput:
        rate = train_throughput(batch=a.batch, products=a.products, base=a.base)
        print(json.dumps({"train_samples_per_s": rate, "batch": a.batch, "grid": GRID,
                          "products": a.products, "base": a.base}))
        return {"train_samples_per_s": rate}
    cases = make_cases(a.cavities, a.channels, a.seed, cavity_re=(100.0, a.cavity_re_max))
    meshes, X, Y, M, gen, gen_s = generate(cases, a.max_steps, a.check_every, a.gen_tol)
    rng = np.random.default_rng(a.seed + 1)
    order = rng.permutation(len(cases))
    ntr = int(round(0.8 * len(cases)))
    tr, te = np.sort(order[:ntr]), np.sort(order[ntr:])
    steady = gen["converged"] == 1
    tr, te = tr[steady[tr]], te[steady[te]]
    if a.reference_start:
        ev = evaluate(None, cases, meshes, X, Y, M, te[: a.eval], a.max_steps, a.check_every, a.tol)
        report = dict(cases=len(cases), steady=int(steady.sum()), reference_start=True, tol=a.tol,
                      warm_vs_cold=ev)
        print(json.dumps({k: v for k, v in ev.items() if k != "per_case"}))
        if a.out:
            with open(a.out, "w") as f:
                json.dump(report, f, indent=1)
        return report
    Xt, Yt, Mt = training_set(cases, X, Y, M, tr, augment=not a.no_augment)
    n_samples = len(Xt)
    net, hist, train_s = train(Xt, Yt, Mt, np.arange(len(Xt)), a.epochs, a.batch, a.lr, a.seed,
                               weight_decay=a.weight_decay, coarse_weight=a.coarse_weight,
                               coarse_block=a.coarse_block, base=a.base, products=a.products)
    del Xt, Yt, Mt
    test_mse = masked_mse(net, X, Y, M, te)[0] if len(te) else None
    ev = evaluate(net, cases, meshes, X, Y, M, te[: a.eval], a.max_steps, a.check_every, a.tol)
    report = dict(
        cases=len(cases), cavities=a.cavities, channels=a.channels, steady=int(steady.sum()),
        generation=dict(seconds=gen_s, converged=int(steady.sum()),
                        steps_mean=float(gen["steps"].mean()), max_steps=a.max_steps,
                        check_every=a.check_every, tol=a.gen_tol),
        training=dict(cases=len(tr), samples=n_samples, epochs=a.epochs, batch=a.batch,
                      lr=a.lr, weight_decay=a.weight_decay, coarse_weight=a.coarse_weight,
                      coarse_block=a.coarse_block,
                      seconds=train_s, loss_first=hist[0], loss_last=hist[-1],
                      params=net.num_params, history=hist),
        test_mse=test_mse, tol=a.tol, warm_vs_cold=ev)
    short = {k: v for k, v in report.items() if k not in ("warm_vs_cold", "training")}
    short["training"] = {k: v for k, v in report["training"].items() if k != "history"}
    short["warm_vs_cold"] = {k: v for k, v in ev.items() if k != "per_case"}
    print(json.dumps(short))
    if a.out:
        with open(a.out, "w") as f:
            json.dump(report, f, indent=1)
    net.close()
    return report


if __name__ == "__main__":
    main()
