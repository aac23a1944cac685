"""Reference workloads of the time-step path, runnable end to end on one GPU.

    python -m parallellbmcranfield_gb300.workloads cylinder   [--out r.json]
    python -m parallellbmcranfield_gb300.workloads steady     [--out r.json]
    python -m parallellbmcranfield_gb300.workloads cavities   [--out r.json]
    python -m parallellbmcranfield_gb300.workloads batch      [--cases N --steps K]

cylinder: channel of 2048 x 512 nodes, MRT, parabolic inlet (u_max 0.04),
  constant-pressure outlet, a cylinder of diameter 64 centred at (400, 257)
  (one node off the axis), Re 200 on the mean inlet speed, 200k steps in FP64,
  FP32 and FP16-deviation storage.  The wake sheds vortices, so the comparison
  is on the statistics of the last 100k steps: mean drag coefficient,
  drag and lift amplitudes, Strouhal number (lift spectrum peak).
steady: steady flows: FP64 runs to du_rel <= 1e-10 (or a step cap), every other
  precision the same number of steps; velocity and de-meaned density errors
  against FP64.
cavities: 256 lid-driven cavities in one batch, sides log-uniform in
  [64, 1024], Re uniform in [100, 3200], lid 0.05, TRT (magic parameter 3/16),
  FP32, autotuned tile, run until every case reaches du_rel <= 1e-6 or stops
  on NaN.
batch: throughput of the batched step alone: N lid-driven cavities of 256^2
  nodes, MRT, Re 1000, FP32, K steps with no case converging (tol < 0).
"""
import argparse
import json
import time

import numpy as np

import parallellbmcranfield_gb300 as G


def cylinder_stats(fx, fy, every, u_mean, diameter):
    cd = 2 * fx / (u_mean * u_mean * diameter)
    cl = 2 * fy / (u_mean * u_mean * diameter)
    y = cl - cl.mean()
    spec = np.abs(np.fft.rfft(y * np.hanning(len(y))))
    k = float(np.argmax(spec[1:]) + 1)
    i = int(k)
    if 1 <= i < len(spec) - 1:  # parabolic refinement of the peak
        a, b, c = spec[i - 1], spec[i], spec[i + 1]
        k = i + 0.5 * (a - c) / (a - 2 * b + c)
    period = len(y) * every / k
    return dict(cd_mean=float(cd.mean()), cd_amp=float(cd.std() * np.sqrt(2)),
                cl_amp=float(cl.std() * np.sqrt(2)), cl_mean=float(cl.mean()),
                strouhal=float(diameter / (u_mean * period)))


def cylinder(precisions=("fp64", "fp32", "fp16dev"), steps=200000, sample_from=100000, every=50):
    u_max, d, re = 0.04, 64, 200
    u_mean = u_max / 1.5
    out = {}
    fields = {}
    for prec in precisions:
        mesh = G.Mesh.channel(2046, 510, [(400.0, 257.0, d / 2)])
        s = G.Solver(mesh, uavg=u_mean, viscosity=u_mean * d / re, inlet_profile=1,
                     collision_model=G.MRT, curved_boundaries=1, outlet_profile=4, rho_out=1.0,
                     drag_lift_id=5, precision=prec)
        s.set_state(None, np.ones(s.N), np.zeros(s.N), np.zeros(s.N))
        t0 = time.perf_counter()
        s.step(sample_from)
        fx, fy = [], []
        for _ in range((steps - sample_from) // every):
            s.step(every)
            dg = s.check()
            fx.append(dg["force"][0])
            fy.append(dg["force"][1])
        el = time.perf_counter() - t0
        fields[prec] = s.fields()
        s.close()
        out[prec] = dict(cylinder_stats(np.array(fx), np.array(fy), every, u_mean, d), seconds=el)
    ref = fields.get("fp64")
    if ref is not None:
        sp = np.sqrt(ref["u"] ** 2 + ref["v"] ** 2).max()
        for prec in precisions:
            if prec != "fp64":
                f = fields[prec]
                out[prec]["pointwise_max_rel_at_end"] = float(
                    np.sqrt((f["u"] - ref["u"]) ** 2 + (f["v"] - ref["v"]) ** 2).max() / sp)
    return out


def run_steady(mesh, kw, prec, max_steps, tol=1e-10, chunk=1000, fixed=False):
    """Steps in chunks until du_rel <= tol or max_steps (fixed: exactly max_steps)."""
    s = G.Solver(mesh, precision=prec, **kw)
    s.set_state(None, np.ones(s.N), np.zeros(s.N), np.zeros(s.N))
    s.step(chunk)
    d = s.check()
    it = chunk
    while it < max_steps:
        s.step(chunk)
        it += chunk
        d = s.check()
        if not fixed and d["du_rel"] <= tol:
            break
    f = s.fields()
    s.close()
    return f, it, d["du_rel"]


STEADY_CASES = {
    "cavity254_re100": (lambda: G.Mesh.cavity(254),
                        dict(uavg=0.05, viscosity=0.05 * 254 / 100, inlet_profile=2,
                             collision_model=G.MRT, curved_boundaries=1, outlet_profile=2), 400000),
    "channel512x128_cyl16_re20": (lambda: G.Mesh.channel(510, 126, [(100.0, 64.5, 8.0)]),
                                  dict(uavg=0.04 / 1.5, viscosity=(0.04 / 1.5) * 16 / 20,
                                       inlet_profile=1, collision_model=G.MRT, curved_boundaries=1,
                                       outlet_profile=4, rho_out=1.0), 1500000),
}


def steady(precisions=("fp32", "fp16neq", "fp16dev", "bf16dev")):
    """Every precision runs exactly as many steps as FP64 needed to reach
    du_rel <= 1e-10, so the comparison is at the same iteration (the cavity's
    lid treatment adds mass every step, so its mean density keeps rising)."""
    out = {}
    for name, (mk, kw, mx) in STEADY_CASES.items():
        mesh = mk()
        fluid = G.inspect_mesh(mesh, **{k: v for k, v in kw.items() if k != "rho_out"})["cls"] > 0
        ref, it, du = run_steady(mesh, kw, "fp64", mx)
        r = {"fp64": dict(steps=it, du_rel=du)}
        sp = np.sqrt(ref["u"] ** 2 + ref["v"] ** 2)[fluid]
        for prec in precisions:
            f, _, dup = run_steady(mesh, kw, prec, it, fixed=True)
            e = np.sqrt((f["u"] - ref["u"]) ** 2 + (f["v"] - ref["v"]) ** 2)[fluid]
            dr = (f["rho"] - ref["rho"])[fluid]
            r[prec] = dict(steps=it, du_rel=dup, vel_err_max_rel=float(e.max() / sp.max()),
                           vel_err_l2_rel=float(np.sqrt((e ** 2).sum() / (sp ** 2).sum())),
                           rho_err_demeaned_max=float(np.abs(dr - dr.mean()).max()),
                           rho_mean_offset=float(dr.mean()))
        out[name] = r
    return out


def cavities(n=256, max_steps=2000000, seed=20240603):
    rng = np.random.default_rng(seed)
    sides = np.round(np.exp(rng.uniform(np.log(64), np.log(1024), n))).astype(int)
    res = rng.uniform(100, 3200, n)
    cs = [(G.Mesh.cavity(int(side) - 2),
           dict(uavg=0.05, vavg=0.0, rho_ini=1.0, viscosity=0.05 * (int(side) - 2) / re,
                inlet_profile=2, collision_model=G.TRT, curved_boundaries=1, outlet_profile=2))
          for side, re in zip(sides, res)]
    t0 = time.perf_counter()
    b = G.Batch(cs, precision="fp32")
    tune = b.autotune(5)
    b.set_rest()
    setup = time.perf_counter() - t0
    info = b.info()
    r = b.run(max_steps, check_every=100, tol=1e-6, raise_on_nan=False)
    b.close()
    nodes = np.array([c[0].shape[0] * c[0].shape[1] for c in cs], float)
    node_steps = float((nodes * r["steps"]).sum())
    nu = np.array([c[1]["viscosity"] for c in cs])
    conv = r["converged"]
    return dict(cases=n, info=info, tune=tune, setup_s=setup, seconds=r["seconds"],
                converged=int((conv == 1).sum()), diverged=int((conv == -1).sum()),
                steps_median=float(np.median(r["steps"][conv == 1])) if (conv == 1).any() else None,
                steps_max=int(r["steps"].max()), node_steps=node_steps,
                glups=node_steps / r["seconds"] / 1e9, hbm_gbs=node_steps * 72 / r["seconds"] / 1e9,
                max_cell_re_converged=float((0.05 / nu[conv == 1]).max()) if (conv == 1).any() else None,
                min_cell_re_diverged=float((0.05 / nu[conv == -1]).min()) if (conv == -1).any() else None)


def batch(n=256, steps=2000, side=254):
    cs = [(G.Mesh.cavity(side), dict(uavg=0.05, vavg=0.0, rho_ini=1.0, viscosity=0.05 * side / 1000,
                                      inlet_profile=2, collision_model=G.MRT, curved_boundaries=1,
                                      outlet_profile=2)) for _ in range(n)]
    b = G.Batch(cs, precision="fp32")
    tune = b.autotune(5)
    b.set_rest()
    b.run(200, check_every=100, tol=-1.0)  # warm-up
    r = b.run(steps, check_every=100, tol=-1.0)
    info = b.info()
    b.close()
    node_steps = float(info["nodes"]) * steps
    return dict(cases=n, nodes=info["nodes"], steps=steps, seconds=r["seconds"], tune=tune,
                glups=node_steps / r["seconds"] / 1e9,
                hbm_gbs=node_steps * 72 / r["seconds"] / 1e9)


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("workload", choices=["cylinder", "steady", "cavities", "batch"])
    p.add_argument("--cases", type=int, default=256)
    p.add_argument("--steps", type=int, default=2000)
    p.add_argument("--out", default=None)
    a = p.parse_args(argv)
    if a.workload == "batch":
        r = batch(a.cases, a.steps)
    else:
        r = {"cylinder": cylinder, "steady": steady, "cavities": cavities}[a.workload]()
    print(json.dumps(r))
    if a.out:
        with open(a.out, "w") as f:
            json.dump(r, f, indent=1)
    return r


if __name__ == "__main__":
    main()
