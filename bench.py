"""Benchmark of the fused D2Q9 step on one GB300 (MLUPS and HBM roofline).

Workload (the large single cavity): a lid-driven cavity of 16382^2 fluid
cells in a 16384 x 16385 node array (268.4 M nodes), lid u = 0.05,
Re = 10000 (nu = u L / Re), MRT collision, FP32 populations, A-B pattern,
started from f = f_eq at rest.  A step is one iteration of the reference's
loop body over the whole array: the fused step kernel plus the reference's
residual line (serial/Iterate.c:263-307).

  value   MLUPS = nodes x steps / device time of the timed steps (CUDA events
          on the solver's stream; state resident in HBM; 19.3 GB of
          populations per step, far above the 129 MB L2, so no flush is needed)
  e2e     the same job through the C ABI with host buffers: lbm_set_state
          from pinned host rho/u/v, K x lbm_step(1) with the reference's
          per-step residual line copied back, lbm_get_fields to host
  roofline  algorithmic bytes per node and step (FP32: 9 loads + 9 stores of
          4 bytes = 72 B) x nodes / average duration of the step kernel alone
          (a second timed run without residual lines), against the measured
          HBM copy peak
  variants  the other storages and patterns of the same cavity (AA, 16-bit)

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]
  torchrun --nproc-per-node N bench.py --gpus N ...   (N replicas, one per GPU)
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

W9 = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4)
PREC_NAME = {0: "fp64", 1: "fp32", 2: "fp16dev", 3: "bf16dev", 4: "fp16neq"}
DTYPE = {0: "f64", 1: "f32", 2: "f16 storage, f32 compute", 3: "bf16 storage, f32 compute",
         4: "24-bit fixed rho/j + f16 non-equilibrium moments, f32 compute"}
BYTES = {0: 144, 1: 72, 2: 36, 3: 36, 4: 42}
CPU_SAMPLE_SIDE = 1022  # 1024 x 1025 node cavity for the CPU legs
VARIANTS = (("fp32", "aa"), ("fp16neq", "ab"), ("fp16dev", "ab"), ("fp16dev", "aa"),
            ("bf16dev", "ab"), ("bf16dev", "aa"))


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--side", type=int, default=16382, help="fluid cells per cavity side")
    p.add_argument("--precision", default="fp32", choices=list(PREC_NAME.values()))
    p.add_argument("--pattern", default="ab", choices=["ab", "aa"])
    p.add_argument("--model", type=int, default=3)
    p.add_argument("--cpu-seconds", type=float, default=12.0)
    p.add_argument("--cpu-side", type=int, default=CPU_SAMPLE_SIDE,
                   help="fluid cells per side of the CPU sample cavity")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--tile", type=int, default=0,
                   help="fused-step tile variant 1..6; 0 = autotune")
    p.add_argument("--no-variants", action="store_true",
                   help="skip the AA and 16-bit storage variants of the cavity")
    return p.parse_args()


def host_info():
    """CPU model string and logical core count of this host."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.split(":")[0].strip() in ("Model name", "Model"):
                val = line.split(":", 1)[1].strip()
                if val and not val.isdigit():
                    model = val
                    break
    except (OSError, subprocess.SubprocessError):
        pass
    if model is None:
        try:
            with open("/proc/cpuinfo") as fh:
                for line in fh:
                    if line.lower().startswith(("model name", "cpu part")):
                        model = line.split(":", 1)[1].strip()
                        break
        except OSError:
            pass
    return {"cpu_model": model or "unknown", "nproc": os.cpu_count()}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl" if os.environ.get("LBM_BENCH_GLOO") is None else "gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def job_mlups(ws, nodes, steps, ms_max):
    """Whole-job throughput of ws replicas of `nodes` nodes each, `steps`
    steps, timed by the slowest rank (ms_max)."""
    return ws * nodes * steps / (ms_max / 1e3) / 1e6


def median_pass(passes):
    """The median of the timed end-to-end passes, each (job time over ranks,
    set_state, steps, get_fields) in seconds: the middle one by job time."""
    return sorted(passes)[len(passes) // 2]


def max_over_ranks(ws, x, device):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-i", str(self.idx), "-lms", "100"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            self.p.wait()

    def summary(self):
        self.f.flush()
        rows = []
        try:
            with open(self.f.name) as fh:
                for line in fh:
                    parts = [x.strip() for x in line.split(",")]
                    if len(parts) >= 9:
                        rows.append(parts)
        finally:
            os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


def feq_rest(rho0, N):
    return np.tile(rho0 * W9, (N, 1))


def _port_sample(side, model):
    """The oracle port on a side^2 cavity at rest, after its first collision.
    The mesh comes from numpy (oracle.meshgen): no GPU library is loaded."""
    from oracle import meshgen
    from oracle import oracle as O

    nodes, conns, (n, m) = meshgen.cavity(side)
    nu = 0.05 * side / 10000.0
    port = O.Port(nodes, conns, uavg=0.05, vavg=0.0, rho_ini=1.0, viscosity=nu,
                  inlet_profile=2, model=model, curved=1, outlet=2)
    N = n * m
    port.set_state(feq_rest(1.0, N), np.ones(N), np.zeros(N), np.zeros(N))
    port.run(1, want_resid=False)
    return port, N


def cpu_port_mlups(side, model, seconds, steps=None):
    """The oracle (C restatement of the serial reference, 1 thread) on a cavity
    sample, one step and the reference's residual line at a time."""
    from oracle import oracle as O

    O.build(ref=False)
    port, N = _port_sample(side, model)
    done, t0 = 0, time.perf_counter()
    while True:
        port.run(1, want_resid=True)
        done += 1
        el = time.perf_counter() - t0
        if (steps is not None and done >= steps) or (steps is None and el >= seconds):
            break
    port.close()
    return N * done / el / 1e6, N, done, el


def _replica(job):
    """One CPU core's share of the reference arm: warm-up, then the timed steps."""
    side, model, warmup, steps = job
    port, N = _port_sample(side, model)
    port.run(warmup, want_resid=True)
    t0 = time.perf_counter()
    port.run(steps, want_resid=True)
    el = time.perf_counter() - t0
    port.close()
    return N, el


def reference_arm(args):
    """The reference's own CPU arithmetic (the oracle port, bit-identical to the
    serial code) on every host core: one independent cavity per core, as the
    serial program is single-threaded.  It loads nothing of the GPU library."""
    import multiprocessing as mp

    ws, rank, _ = dist_setup()
    if rank != 0:
        return
    from oracle import oracle as O

    O.build(ref=False)
    host = host_info()
    cores = host["nproc"] or 1
    side = args.cpu_side
    with mp.get_context("spawn").Pool(cores) as pool:
        res = pool.map(_replica, [(side, args.model, args.warmup, args.steps)] * cores)
    N = res[0][0]
    el_max = max(el for _, el in res)
    mlups = cores * N * args.steps / el_max / 1e6
    n, m = side + 2, side + 3
    sample = (f"oracle port (the serial reference's arithmetic, bit-identical; 528-byte cells, five "
              f"sweeps) on {cores} independent {n}x{m}-node cavities, one per host core "
              f"({host['cpu_model']}, nproc {host['nproc']}), {args.steps} steps each after "
              f"{args.warmup} warm-up, per-step residual line as the serial loop; whole-host MLUPS "
              f"timed by the slowest core")
    line = {
        "impl": "reference", "metric": "MLUPS", "value": round(mlups, 3), "unit": "MLUPS",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(el_max / args.steps * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"lid-driven cavity {n}x{m} nodes ({side}^2 fluid), lid u=0.05, "
                               f"Re=10000, D2Q9 MRT, FP64 as the serial reference, x{cores} "
                               f"(one per host core); CPU sample of the GPU arm's "
                               f"{args.side + 2}x{args.side + 3} cavity, which does not fit "
                               f"the reference's 528-byte cells in host memory",
                   "nodes": n * m * cores, "fluid_nodes": side * side * cores,
                   "precision": "fp64", "collision_model": args.model, "replicas": cores,
                   "l2_flush": f"CPU run: each cavity holds {n * m * 528 / 1e9:.3f} GB of "
                               f"528-byte cells"},
        "cpu_baseline": {"value": round(mlups, 3), "unit": "MLUPS", "cores": cores,
                         "kind": "port", "sample": sample, "host": host},
        "e2e": {"value": round(mlups, 3), "unit": "MLUPS", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


ELEM_BYTES = {"fp64": 8, "fp32": 4, "fp16dev": 2, "bf16dev": 2, "fp16neq": 21 / 9}


def workload_config(args, side):
    n, m = side + 2, side + 3
    pop_gb = n * m * 9 * ELEM_BYTES[args.precision] * (2 if args.pattern == "ab" else 1) / 1e9
    return {"workload": f"lid-driven cavity {n}x{m} nodes ({side}^2 fluid), lid u=0.05, Re=10000, "
                        f"D2Q9 MRT, {args.precision} {args.pattern.upper()}",
            "nodes": n * m, "fluid_nodes": side * side, "precision": args.precision,
            "pattern": args.pattern, "collision_model": args.model,
            "l2_flush": f"inputs larger than L2 (populations {pop_gb:.2f} GB, L2 0.13 GB)"
                        if pop_gb > 0.129 else "inputs fit in L2: no flush (small case)"}


def load_traffic(precision, pattern, model):
    """Per-launch DRAM bytes from the committed ncu summary of this kernel, if any."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as fh:
            t = json.load(fh)
        return t.get(f"{precision}_{pattern}_m{model}")
    except (OSError, ValueError):
        return None


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback"


def cavity_solver(G, side, prec_name, pat_name, model, local, stream, tile=0):
    mesh = G.Mesh.cavity(side)
    s = G.Solver(mesh, uavg=0.05, vavg=0.0, rho_ini=1.0, viscosity=0.05 * side / 10000.0,
                 inlet_profile=2, collision_model=model, curved_boundaries=1, outlet_profile=2,
                 precision=G.PRECISIONS[prec_name], pattern=G.PATTERNS[pat_name], device=local,
                 stream=stream.cuda_stream, tile_variant=tile)
    del mesh
    return s


def timed_steps(torch, dev, stream, solver, steps, check_every, local=0, clocks=False):
    """Device time (ms) of `steps` lbm_step iterations on the solver's stream,
    with nvidia-smi sampling the clocks meanwhile when asked."""
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clk = ClockSampler(local) if clocks else None
    if clk:
        clk.__enter__()
    try:
        torch.cuda.synchronize(dev)
        ev0.record(stream)
        solver.step(steps, check_every)
        ev1.record(stream)
        torch.cuda.synchronize(dev)
    finally:
        if clk:
            clk.__exit__()
    return ev0.elapsed_time(ev1), (clk.summary() if clk else None)


E2E_PASSES = 3  # timed end-to-end passes; the median is reported


def run_gpu(args):
    import torch

    import parallellbmcranfield_gb300 as G

    ws, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    prec = G.PRECISIONS[args.precision]
    side = args.side
    t_setup = time.perf_counter()
    stream = torch.cuda.Stream(device=dev)
    solver = cavity_solver(G, side, args.precision, args.pattern, args.model, local, stream,
                           args.tile)
    N = solver.N
    tune = solver.autotune(10) if args.tile == 0 else {"variant": args.tile - 1, "fixed": True}
    # pinned host state: f = f_eq at rest is formed on the device from rho/u/v
    rho_h = torch.ones(N, dtype=torch.float64, pin_memory=True)
    u_h = torch.zeros(N, dtype=torch.float64, pin_memory=True)
    v_h = torch.zeros(N, dtype=torch.float64, pin_memory=True)
    solver.set_state(None, rho_h.numpy(), u_h.numpy(), v_h.numpy())
    setup_s = time.perf_counter() - t_setup

    # ---- device-resident throughput: the loop body of the reference (fused
    # step + residual line every step)
    solver.step(args.warmup, 1)
    torch.cuda.synchronize(dev)
    barrier(ws)
    ms, clocks = timed_steps(torch, dev, stream, solver, args.steps, 1, local, clocks=True)
    barrier(ws)
    ms_max = max_over_ranks(ws, ms, dev)
    launches = 2 * args.steps  # per step: the fused step kernel and the residual kernel
    mlups = job_mlups(ws, N, args.steps, ms_max)
    # ---- the step kernel alone (roofline)
    ms_k, _ = timed_steps(torch, dev, stream, solver, args.steps, 0)
    per_launch_s = ms_k / 1e3 / args.steps
    bpn = BYTES[prec]
    achieved = bpn * N / per_launch_s / 1e9
    peak, peak_kind = measured_peak()
    traffic = load_traffic(args.precision, args.pattern, args.model)
    diag = solver.check()

    # ---- end to end through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        res_h = np.zeros((args.steps, 4))
        rho_o = torch.empty(N, dtype=torch.float64, pin_memory=True).numpy()
        u_o = torch.empty(N, dtype=torch.float64, pin_memory=True).numpy()
        v_o = torch.empty(N, dtype=torch.float64, pin_memory=True).numpy()
        # one untimed pass of the same calls first: the first device access to
        # freshly pinned host pages and the first launch of each kernel cost
        # once per process (3-4x the steady set_state time on the GB300 host)
        solver.set_state(None, rho_h.numpy(), u_h.numpy(), v_h.numpy())
        solver.step(1, 1)
        assert solver.L.lbm_get_fields(solver.h, rho_o.ctypes.data, u_o.ctypes.data,
                                       v_o.ctypes.data, None, None) == 0
        # three timed passes, the median reported: the host link of a shared
        # box is occasionally slower for one pass (set_state 33 ms in most
        # passes, up to 128 ms in a few)
        passes = []
        for _ in range(E2E_PASSES):
            barrier(ws)
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            solver.set_state(None, rho_h.numpy(), u_h.numpy(), v_h.numpy())
            t1 = time.perf_counter()
            for i in range(args.steps):
                res_h[i] = solver.step(1, 1)[0]
            t2 = time.perf_counter()
            out = solver.L.lbm_get_fields(solver.h, rho_o.ctypes.data, u_o.ctypes.data,
                                          v_o.ctypes.data, None, None)
            torch.cuda.synchronize(dev)
            t3 = time.perf_counter()
            assert out == 0
            passes.append((max_over_ranks(ws, t3 - t0, dev), t1 - t0, t2 - t1, t3 - t2))
        el, p1, p2, p3 = median_pass(passes)
        e2e = {"value": round(ws * N * args.steps / el / 1e6, 1), "unit": "MLUPS",
               "h2d_bytes_per_step": int(3 * 8 * N / args.steps),
               "d2h_bytes_per_step": int(32 + 3 * 8 * N / args.steps),
               "what": "lbm_set_state(host rho,u,v) + steps x lbm_step(1, residual line) + "
                       "lbm_get_fields(host rho,u,v), wall clock, median of "
                       f"{E2E_PASSES} passes after one untimed pass of the same calls",
               "phases_ms": {"set_state": round(p1 * 1e3, 2), "steps": round(p2 * 1e3, 2),
                             "get_fields": round(p3 * 1e3, 2)},
               "passes_ms": [round(q[0] * 1e3, 1) for q in passes]}
    solver.close()

    variants = {}
    if not args.no_variants:
        for vp, vpat in VARIANTS:
            if (vp, vpat) != (args.precision, args.pattern):
                variants[f"{vp}_{vpat}"] = time_variant(args, G, torch, dev, stream, local, vp,
                                                        vpat)
        base = variants.get("fp32_ab") if args.precision != "fp32" else None
        ref_ms = base["ms_per_step"] if base else (ms_k / args.steps
                                                   if args.precision == "fp32" and
                                                   args.pattern == "ab" else None)
        if ref_ms:
            for v in variants.values():
                v["speedup_vs_fp32_ab"] = round(ref_ms / v["ms_per_step"], 3)

    if rank != 0:
        return
    cpu_mlups, cpu_N, cpu_steps, cpu_s = cpu_port_mlups(args.cpu_side, args.model,
                                                        args.cpu_seconds)
    host = host_info()
    line = {
        "metric": "MLUPS", "value": round(mlups, 1), "unit": "MLUPS", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_max / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": DTYPE[prec], "data": "synthetic",
        "config": workload_config(args, side),
        "what": "value: per step the fused step kernel and the reference's residual line "
                "(serial/Iterate.c:263-307), state resident on the device; roofline: the step "
                "kernel alone",
        "fluid_mlups": round(ws * args.side ** 2 * args.steps / (ms_max / 1e3) / 1e6, 1),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic,
                     "peak_kind": peak_kind, "bytes_per_node_step": bpn,
                     "kernel_ms": round(ms_k / args.steps, 4),
                     "kernel": "lbm::k_step (fused pull-stream + BC + moments + collision)"},
        "cpu_baseline": {"value": round(cpu_mlups, 3), "unit": "MLUPS", "cores": 1, "kind": "port",
                         "sample": f"oracle port (serial reference restated, bit-identical), cavity "
                                   f"{args.cpu_side + 2}x{args.cpu_side + 3} MRT FP64, "
                                   f"{cpu_steps} steps in {cpu_s:.1f} s, 1 thread of "
                                   f"{host['nproc']} ({host['cpu_model']})",
                         "host": host},
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clocks,
        "diagnostics": {"mass": diag["mass"], "max_speed": diag["max_speed"]},
        "setup_s": round(setup_s, 1),
        "tile": tune,
    }
    if variants:
        line["variants"] = variants
    print(json.dumps(line), flush=True)


def time_variant(args, G, torch, dev, stream, local, prec_name, pat_name):
    """MLUPS, HBM fraction and clocks of another storage / pattern on the same
    cavity (autotuned tile), the step kernel alone."""
    steps = max(10, args.steps // 2)
    s = cavity_solver(G, args.side, prec_name, pat_name, args.model, local, stream)
    N = s.N
    tune = s.autotune(10)
    s.set_state(None, np.ones(N), np.zeros(N), np.zeros(N))
    s.step(max(3, args.warmup), 0)
    ms, clocks = timed_steps(torch, dev, stream, s, steps, 0, local, clocks=True)
    s.close()
    prec = G.PRECISIONS[prec_name]
    per = ms / 1e3 / steps
    peak, _ = measured_peak()
    return {"mlups": round(N / per / 1e6, 1),
            "ms_per_step": round(ms / steps, 4), "steps": steps,
            "bytes_per_node_step": BYTES[prec],
            "hbm_frac": round(BYTES[prec] * N / per / 1e9 / peak, 4), "tile": tune,
            "clocks": clocks}


def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
