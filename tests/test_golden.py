"""Committed golden fixtures: setups written by the reference's own Python builder and the
oracle's per-step outputs for them (tests/golden/make_golden.py).

CPU: the oracle reproduces the committed numbers (regression pin, 1e-12).
GPU: the CUDA library reproduces them within the hot path's bar (1e-5 relative).
"""
import os

import numpy as np
import pytest

from stormbird_gb300.setups import GustyWind
from tests.helpers import rel_inf, rel_vec

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["dynamic", "quasi_steady"]


def load(case):
    js = open(os.path.join(HERE, f"setup_stormbird_setup_{case}.json")).read()
    g = np.load(os.path.join(HERE, f"golden_stormbird_setup_{case}.npz"))
    return js, g


def replay(sim, g):
    wind = GustyWind(seed=int(g["seed"]))
    dt = float(g["dt"])
    n = sim.nr_freestream_points
    for k in range(int(g["steps"])):
        t = k * dt
        yield k, sim.do_step(time=t, time_step=dt, freestream_velocity=wind.freestream(t, n))


@pytest.mark.parametrize("case", CASES)
def test_oracle_reproduces_golden(oracle_mod, case):
    js, g = load(case)
    sim = oracle_mod.OracleSimulation(js)
    for k, r in replay(sim, g):
        assert rel_inf(r.circulation_strength, g["gamma"][k]) < 1e-12
        assert rel_vec(r.integrated_forces_sum(), g["force"][k]) < 1e-12
        assert r.iterations == g["iterations"][k]


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_gpu_reproduces_golden(gpu_lib, case):
    from stormbird_gb300 import Simulation

    js, g = load(case)
    sim = Simulation(js)
    for k, r in replay(sim, g):
        assert rel_inf(r.circulation_strength, g["gamma"][k]) <= 1e-5, f"step {k}"
        assert rel_vec(r.integrated_forces_sum(), g["force"][k]) <= 1e-5, f"step {k}"
        assert rel_vec(r.integrated_moments_sum(), g["moment"][k]) <= 1e-5, f"step {k}"
