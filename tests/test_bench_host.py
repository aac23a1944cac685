"""bench.py host helpers on CPU: the clock record, the workload description,
the committed traffic figures."""
import os
import sys
import types

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_clock_summary_flags_throttle_reasons(tmp_path):
    c = bench.ClockSampler(0)
    c.f.write("0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active\n"
              "0, 2055, 2070, 1400.0, 0x4, Not Active, Not Active, Not Active, Active\n"
              "0, 2070, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active\n")
    r = c.summary()
    assert r["sm_mhz"] == 2070.0 and r["sm_max_mhz"] == 2070.0 and r["samples"] == 3
    assert r["reasons"] == ["sw_power_cap"]


def test_workload_config_and_traffic():
    a = types.SimpleNamespace(precision="fp32", pattern="ab", model=3)
    cfg = bench.workload_config(a, 16382)
    assert cfg["nodes"] == 16384 * 16385 and cfg["fluid_nodes"] == 16382 ** 2
    assert "19.33 GB" in cfg["l2_flush"]
    a.precision = "fp16dev"
    assert "9.66 GB" in bench.workload_config(a, 16382)["l2_flush"]
    t = bench.load_traffic("fp32", "ab", 3)
    # measured DRAM bytes of one full-size launch: the algorithmic 72 B/node plus
    # the class byte (1.4 %), no re-reads
    assert 1.0 < t / (72 * 16384 * 16385) < 1.03
    assert bench.load_traffic("fp64", "aa", 1) is None


def test_reference_arm_loads_no_gpu_library():
    """The reference arm times the oracle port on every host core and states
    the workload it timed; neither it nor its workers load liblbm_gb300.so."""
    import json
    import subprocess

    code = ("import sys, runpy; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '2', "
            "'--warmup', '1', '--cpu-side', '30']; runpy.run_path('bench.py', run_name='__main__'); "
            "maps = open('/proc/self/maps').read(); "
            "print('LOADED' if 'liblbm_gb300' in maps or 'parallellbmcranfield_gb300' in sys.modules "
            "else 'CLEAN')")
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True,
                         timeout=600)
    assert out.returncode == 0, out.stderr
    lines = out.stdout.strip().splitlines()
    assert lines[-1] == "CLEAN"
    line = json.loads(lines[-2])
    assert line["impl"] == "reference" and line["unit"] == "MLUPS" and line["value"] > 0
    assert "32x33 nodes" in line["config"]["workload"] and "FP64" in line["config"]["workload"]
    cb = line["cpu_baseline"]
    assert cb["cores"] == os.cpu_count() and cb["kind"] == "port"
    assert cb["host"]["nproc"] == os.cpu_count() and cb["host"]["cpu_model"]


def test_host_info():
    h = bench.host_info()
    assert h["nproc"] == os.cpu_count() and isinstance(h["cpu_model"], str)


def test_e2e_median_pass():
    """The end-to-end figure is the middle one of the timed passes by job time,
    with that pass's phases (one slow pass on a shared host link does not set it)."""
    passes = [(0.132, 0.033, 0.059, 0.040), (0.228, 0.128, 0.060, 0.040), (0.131, 0.033, 0.058, 0.040)]
    assert bench.median_pass(passes) == passes[0]
    assert bench.median_pass(passes[:1]) == passes[0]
    assert bench.E2E_PASSES >= 3 and bench.E2E_PASSES % 2 == 1
