"""Build recipe of liblbm_gb300.so (in-tree, no CMake).

Every CUDA translation unit is compiled for sm_103a only; the FP64 kernels
are compiled with --fmad=false so that their arithmetic keeps the serial
reference's roundings.  Objects go to _build/, the library next to this file.
Translation units compile in parallel.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "liblbm_gb300.so")
SOLVER = os.path.join(HERE, "bin", "lbm_solver")  # drop-in for the serial program
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblbm_gb300.so")


INST = "lbm_kernels_inst.cu"  # compiled once per (precision, part)
BATCH_INST = "lbm_batch_inst.cu"  # compiled once per batch precision (FP64, FP32, FP16-dev)
PRECS = ["f64", "f32", "f16", "b16"]


def sources():
    """(object name, source, extra flags) for every translation unit."""
    units = []
    for f in sorted(os.listdir(CSRC)):
        if f == INST:
            for p, name in enumerate(PRECS):
                for part in range(4):
                    flags = [f"-DLBM_PREC={p}", f"-DLBM_PART={part}"]
                    if name == "f64":
                        flags.append("--fmad=false")
                    units.append((f"lbm_kernels_{name}_{part}", f, flags))
        elif f == BATCH_INST:
            for p in range(3):
                flags = [f"-DLBM_PREC={p}"] + (["--fmad=false"] if p == 0 else [])
                units.append((f"lbm_batch_{PRECS[p]}", f, flags))
        elif f.endswith((".cu", ".cpp")) and not f.endswith("_main.cpp"):
            units.append((os.path.splitext(f)[0], f, []))
    return units


def _cmd(obj, src, flags):
    nvcc = _nvcc()
    out = os.path.join(OBJ, obj + ".o")
    path = os.path.join(CSRC, src)
    if src.endswith(".cu"):
        cmd = [nvcc, *ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
               "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr", *flags,
               "-c", path, "-o", out]
        if os.environ.get("LBM_PTXAS_VERBOSE"):
            cmd.insert(1, "-Xptxas=-v")
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off",
               "-I", "/usr/local/cuda/include", "-c", path, "-o", out]
    return cmd, out, path


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, jobs=None):
    os.makedirs(OBJ, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "lbm_gb300.h"))
    jobs_ = []
    objs = []
    for obj, src, flags in sources():
        cmd, out, path = _cmd(obj, src, flags)
        objs.append(out)
        if _stale(out, [path, *headers, __file__]):
            jobs_.append((obj, cmd))
    # objects of sources that no longer exist must not be linked
    for f in os.listdir(OBJ):
        if f.endswith(".o") and os.path.join(OBJ, f) not in objs:
            os.remove(os.path.join(OBJ, f))
    errors = []

    def run(item):
        src, cmd = item
        if verbose:
            print(" ".join(cmd), flush=True)
        t0 = time.time()
        p = subprocess.run(cmd, capture_output=True, text=True)
        if verbose:
            print(f"  {src}: {time.time() - t0:.1f} s", flush=True)
        return src, p

    with cf.ThreadPoolExecutor(max_workers=jobs or min(24, os.cpu_count() or 4)) as ex:
        for src, p in ex.map(run, jobs_):
            if p.returncode != 0:
                errors.append(f"--- {src}\n{p.stdout}\n{p.stderr}")
            elif verbose and (p.stderr.strip()):
                print(p.stderr, file=sys.stderr)
    if errors:
        raise RuntimeError("build failed:\n" + "\n".join(errors))
    if jobs_ or not os.path.exists(LIB):
        cmd = [_nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart_static", "-lrt",
               "-ldl", "-lpthread"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.check_call(cmd)
    main = os.path.join(CSRC, "lbm_solver_main.cpp")
    if _stale(SOLVER, [main, LIB, os.path.join(os.path.dirname(HERE), "include", "lbm_gb300.h")]):
        os.makedirs(os.path.dirname(SOLVER), exist_ok=True)
        cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", main, "-o", SOLVER,
               "-L", HERE, "-llbm_gb300", "-Wl,-rpath,$ORIGIN/.."]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.check_call(cmd)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
