"""GPU: the drop-in program (bin/lbm_solver) writes the same files as the
serial reference program on the same case directory.

Fixtures: tests/golden/solver/<case>/*.gz, the reference program's own output
(tests/golden/make_solver_golden.py).  FP64 mode is bit-identical, so the text
files must match exactly, except the two log lines the reference corrupts
(its CompDataConn float/double mismatch) and the wall-clock timing lines.
"""
import gzip
import os
import subprocess

import pytest

import solver_cases
from parallellbmcranfield_gb300 import build as B

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "solver")


def run_solver(case, tmp_path, *extra):
    solver_cases.write_case(solver_cases.CASES[case], str(tmp_path))
    with open(os.path.join(GOLDEN, case, "SetUpData.ini")) as f:
        assert f.read() == open(tmp_path / "SetUpData.ini").read()
    p = subprocess.run([B.SOLVER, "--dir", str(tmp_path), *extra], capture_output=True, text=True,
                       timeout=300)
    assert p.returncode == 0, p.stderr
    return tmp_path / "Results", p.stdout


def golden(case, name):
    with gzip.open(os.path.join(GOLDEN, case, name + ".gz"), "rt") as f:
        return f.read()


def log_lines_to_compare(text):
    keep = []
    for line in text.splitlines():
        if "InletCoordY" in line or " took " in line:
            continue
        if line.startswith(":::: Iterations done"):
            break
        keep.append(line)
    return keep


@pytest.mark.parametrize("case", sorted(solver_cases.CASES))
def test_solver_outputs_match_reference_program(case, tmp_path):
    res, out = run_solver(case, tmp_path)
    names = sorted(f[:-3] for f in os.listdir(os.path.join(GOLDEN, case)) if f.endswith(".gz"))
    for name in names:
        mine = open(res / name).read()
        ref = golden(case, name)
        if name == "logFile.log":
            assert log_lines_to_compare(mine) == log_lines_to_compare(ref)
        else:
            assert mine == ref, name
    assert "Iterations: 00100/" in out


def test_solver_chunked_residual_lines(tmp_path):
    """--check-every K writes every K-th line of the per-step file, same values."""
    case = "cavity30_bgk_csv"
    res, _ = run_solver(case, tmp_path, "--check-every", "25")
    mine = open(res / "residuals.dat").read().splitlines()
    ref = golden(case, "residuals.dat").splitlines()
    assert mine[0] == ref[0]
    wanted = [ref[0]] + [l for l in ref[1:] if (int(l.split()[0]) + 1) % 25 == 0]
    assert mine == wanted


def test_solver_fields_final_data(tmp_path):
    """--final-data both also writes every cell (the reference repeats row 0)."""
    res, _ = run_solver("cavity30_bgk_csv", tmp_path, "--final-data", "both")
    compat = open(res / "FinalData.csv").read().splitlines()
    fields = open(res / "FinalDataFields.csv").read().splitlines()
    assert len(compat) == len(fields)
    assert len(set(compat[1:])) < len(set(fields[1:]))
