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

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "liblbm_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblbm_gb300.so")


def sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cu, cpp


def _cmd(src):
    nvcc = _nvcc()
    out = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    if src.endswith(".cu"):
        cmd = [nvcc, *ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
               "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr",
               "-c", path, "-o", out]
        if src.endswith("_f64.cu"):
            cmd.insert(1, "--fmad=false")
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
    cu, cpp = sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "lbm_gb300.h"))
    jobs_ = []
    objs = []
    for src in cu + cpp:
        cmd, out, path = _cmd(src)
        objs.append(out)
        if _stale(out, [path, *headers, __file__]):
            jobs_.append((src, cmd))
    errors = []

    def run(item):
        src, cmd = item
        if verbose:
            print(" ".join(cmd), flush=True)
        p = subprocess.run(cmd, capture_output=True, text=True)
        return src, p

    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
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
    return LIB


if __name__ == "__main__":
    build(verbose=True)
