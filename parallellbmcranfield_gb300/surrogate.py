"""Surrogate warm start: steady fields generated by the batched solver, the
encoder-decoder trained on them with the library's own BF16 kernels, and a
warm-vs-cold comparison of the wall time to du_rel <= tol.

Cases (256 x 256 node grids, MRT, FP32 storage, curved/half-way walls):
  * lid-driven cavities of 254^2 fluid cells, Re log-uniform in [100, 5000],
    lid speed U uniform in [0.03, 0.06] (nu = U * 254 / Re);
  * channels of 254 x 254 fluid cells with 1-3 non-overlapping cylinders of
    diameter 16-64, parabolic inlet (peak U in [0.03, 0.06]), constant-pressure
    outlet, Re on the largest diameter uniform in [5, 40] (steady wakes).
Network input (4 maps): fluid mask, velocity-boundary cells, log(Re)/log(5000),
U / 0.05.  Output (3 maps): 100 (rho - 1), u / U, v / U on fluid cells.

    python -m parallellbmcranfield_gb300.surrogate --cavities 1000 --channels 1000 --out report.json
"""
import argparse
import json
import time

import numpy as np

import parallellbmcranfield_gb300 as G

GRID = 256
SIDE = GRID - 2


def make_cases(n_cav, n_ch, seed):
    rng = np.random.default_rng(seed)
    cases = []
    for _ in range(n_cav):
        re = float(np.exp(rng.uniform(np.log(100), np.log(5000))))
        U = float(rng.uniform(0.03, 0.06))
        nu = max(U * SIDE / re, 0.0017)
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
        umax = float(rng.uniform(0.03, 0.06))
        re = float(rng.uniform(5, 40))
        dmax = 2 * max(r for _, _, r in cyl)
        nu = max((umax / 1.5) * dmax / re, 0.0017)
        cases.append(dict(kind="channel", re=re, U=umax, spec=("channel", SIDE, SIDE, cyl),
                          params=dict(uavg=umax / 1.5, vavg=0.0, rho_ini=1.0, viscosity=nu,
                                      inlet_profile=1, collision_model=3, curved_boundaries=1,
                                      outlet_profile=4, rho_out=1.0)))
    return cases


def build_mesh(spec):
    if spec[0] == "cavity":
        return G.Mesh.cavity(spec[1])
    return G.Mesh.channel(spec[1], spec[2], spec[3])


def features(case, mesh):
    """Input maps (GRID, GRID, 4) and the fluid mask (GRID, GRID)."""
    n, m = mesh.shape
    fluid = np.zeros((m, n), np.float32)
    ij = mesh.nodes[:, :2].astype(np.int64)
    fluid[ij[:, 1], ij[:, 0]] = mesh.nodes[:, 4]
    bc = np.zeros((m, n), np.float32)
    vel = mesh.conns[mesh.conns[:, 3] == 2]
    bc[vel[:, 1].astype(np.int64), vel[:, 0].astype(np.int64)] = 1.0
    x = np.zeros((GRID, GRID, 4), np.float32)
    x[..., 0] = fluid[:GRID, :GRID]
    x[..., 1] = bc[:GRID, :GRID]
    x[..., 2] = np.log(case["re"]) / np.log(5000.0)
    x[..., 3] = case["U"] / 0.05
    return x, fluid[:GRID, :GRID].copy()


def targets(case, fields, n, m):
    U = case["U"]
    t = np.zeros((GRID, GRID, 3), np.float32)
    for c, (k, scale, shift) in enumerate((("rho", 100.0, 1.0), ("u", 1.0 / U, 0.0),
                                           ("v", 1.0 / U, 0.0))):
        t[..., c] = ((fields[k].reshape(m, n) - shift) * scale)[:GRID, :GRID]
    return t


def fields_from_prediction(case, y, n, m, mask):
    """rho, u, v arrays of the case's n*m grid from a network output."""
    U = case["U"]
    rho, u, v = np.ones((m, n)), np.zeros((m, n)), np.zeros((m, n))
    fl = mask > 0
    rho[:GRID, :GRID][fl] = 1.0 + y[..., 0][fl] / 100.0
    u[:GRID, :GRID][fl] = y[..., 1][fl] * U
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
        Y.append(targets(c, f, n, m))
        M.append(mask)
    b.close()
    return meshes, np.stack(X), np.stack(Y), np.stack(M), r, gen_s


def train(X, Y, M, train_idx, epochs, batch, lr, seed):
    net = G.Surrogate(height=GRID, width=GRID, in_channels=4, out_channels=3, base=32,
                      max_batch=batch, lr=lr, seed=seed)
    net.set_dataset(X, Y, M)
    rng = np.random.default_rng(seed)
    hist = []
    t0 = time.perf_counter()
    for _ in range(epochs):
        hist.append(net.train(rng.permutation(train_idx), batch))
    return net, hist, time.perf_counter() - t0


def masked_mse(net, X, Y, M, idx):
    y = net.forward(X[idx])
    w = M[idx][..., None]
    return float((w * (y - Y[idx]) ** 2).sum() / (w.sum() * 3)), y


def evaluate(net, cases, meshes, X, M, idx, max_steps, check_every, tol):
    sub = [cases[i] for i in idx]
    sub_m = [meshes[i] for i in idx]
    t0 = time.perf_counter()
    bc, rc = run_batch(sub, sub_m, max_steps, check_every, tol)
    cold_s = time.perf_counter() - t0
    bc.close()
    t0 = time.perf_counter()
    y = net.forward(X[idx])
    infer_s = time.perf_counter() - t0
    init = []
    for j, i in enumerate(idx):
        n, m = meshes[i].shape
        init.append(fields_from_prediction(cases[i], y[j], n, m, M[i]))
    t0 = time.perf_counter()
    bw, rw = run_batch(sub, sub_m, max_steps, check_every, tol, init=init)
    warm_s = time.perf_counter() - t0
    bw.close()
    both = (rc["converged"] == 1) & (rw["converged"] == 1)
    return dict(
        cases=len(idx), converged_cold=int((rc["converged"] == 1).sum()),
        converged_warm=int((rw["converged"] == 1).sum()),
        steps_cold_mean=float(rc["steps"][both].mean()) if both.any() else None,
        steps_warm_mean=float(rw["steps"][both].mean()) if both.any() else None,
        steps_ratio_mean=float((rc["steps"][both] / np.maximum(rw["steps"][both], 1)).mean())
        if both.any() else None,
        wall_cold_s=cold_s, wall_warm_s=warm_s + infer_s, inference_s=infer_s,
        wall_speedup=cold_s / (warm_s + infer_s))


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--cavities", type=int, default=1000)
    p.add_argument("--channels", type=int, default=1000)
    p.add_argument("--max-steps", type=int, default=150000)
    p.add_argument("--check-every", type=int, default=500)
    p.add_argument("--tol", type=float, default=1e-6)
    p.add_argument("--epochs", type=int, default=30)
    p.add_argument("--batch", type=int, default=8)
    p.add_argument("--lr", type=float, default=1e-3)
    p.add_argument("--eval", type=int, default=400, help="test cases in the warm/cold comparison")
    p.add_argument("--seed", type=int, default=20240601)
    p.add_argument("--out", default=None)
    a = p.parse_args(argv)
    cases = make_cases(a.cavities, a.channels, a.seed)
    meshes, X, Y, M, gen, gen_s = generate(cases, a.max_steps, a.check_every, a.tol)
    rng = np.random.default_rng(a.seed + 1)
    order = rng.permutation(len(cases))
    ntr = int(round(0.8 * len(cases)))
    tr, te = np.sort(order[:ntr]), np.sort(order[ntr:])
    net, hist, train_s = train(X, Y, M, tr, a.epochs, a.batch, a.lr, a.seed)
    test_mse, _ = masked_mse(net, X, Y, M, te[: max(1, min(len(te), 64))])
    ev = evaluate(net, cases, meshes, X, M, te[: a.eval], a.max_steps, a.check_every, a.tol)
    report = dict(
        cases=len(cases), cavities=a.cavities, channels=a.channels,
        generation=dict(seconds=gen_s, converged=int((gen["converged"] == 1).sum()),
                        steps_mean=float(gen["steps"].mean()), max_steps=a.max_steps,
                        check_every=a.check_every, tol=a.tol),
        training=dict(samples=len(tr), epochs=a.epochs, batch=a.batch, seconds=train_s,
                      loss_first=hist[0], loss_last=hist[-1], params=net.num_params),
        test_mse=test_mse, warm_vs_cold=ev)
    print(json.dumps(report))
    if a.out:
        with open(a.out, "w") as f:
            json.dump(report, f, indent=1)
    net.close()
    return report


if __name__ == "__main__":
    main()
