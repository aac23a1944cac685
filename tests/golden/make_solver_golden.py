"""Writes tests/golden/solver/<case>/: the output files of the UNMODIFIED
serial reference program (oracle/_ref/LBMSolver, built by ``make -C oracle
ref-main`` from mate-szoke/ParallelLbmCranfield serial/) on small generated
cases, gzip-compressed, plus the SetUpData.ini it ran with.  The meshes are
rebuilt by the library's generator (tests/solver_cases.py), so they are not
stored.

    python tests/golden/make_solver_golden.py
"""
import gzip
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import solver_cases  # noqa: E402

REF_BIN = os.path.join(ROOT, "oracle", "_ref", "LBMSolver")


def main():
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref-main"])
    for name, case in solver_cases.CASES.items():
        out = os.path.join(HERE, "solver", name)
        shutil.rmtree(out, ignore_errors=True)
        os.makedirs(out)
        with tempfile.TemporaryDirectory() as td:
            solver_cases.write_case(case, td)
            subprocess.run([REF_BIN], cwd=td, check=True, stdout=subprocess.DEVNULL)
            shutil.copy(os.path.join(td, "SetUpData.ini"), os.path.join(out, "SetUpData.ini"))
            res = os.path.join(td, "Results")
            for f in sorted(os.listdir(res)):
                if f == "SerialTimeMeasuerment.dat":
                    continue  # wall-clock figures
                with open(os.path.join(res, f), "rb") as src, \
                        gzip.open(os.path.join(out, f + ".gz"), "wb", compresslevel=9) as dst:
                    dst.write(src.read())
        print(name, sorted(os.listdir(out)))


if __name__ == "__main__":
    main()
