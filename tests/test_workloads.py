"""Host logic of the workload runner (CPU): the wake statistics."""
import numpy as np

from parallellbmcranfield_gb300 import workloads as W


def test_cylinder_stats_recovers_a_known_wake():
    u_mean, d, every = 0.04 / 1.5, 64, 50
    period = 9000.0  # steps: St = d / (u_mean * period)
    t = np.arange(2000) * every
    cd, cl_amp, cd_amp = 1.37, 0.8, 0.05
    scale = u_mean * u_mean * d / 2
    fx = (cd + cd_amp * np.sin(4 * np.pi * t / period)) * scale
    fy = cl_amp * np.sin(2 * np.pi * t / period + 0.3) * scale
    r = W.cylinder_stats(fx, fy, every, u_mean, d)
    assert abs(r["cd_mean"] - cd) < 1e-3
    assert abs(r["cl_amp"] - cl_amp) < 2e-2 and abs(r["cd_amp"] - cd_amp) < 2e-3
    assert abs(r["strouhal"] - d / (u_mean * period)) < 5e-3 * d / (u_mean * period)
