"""Failure path of the bounded device-side waits, and of device allocation.

A kernel that waits on an asynchronous copy polls its mbarrier a bounded number of times;
when the polls run out it records a timeout in the launch's error word, waits (bounded
again) for its own copies still in flight, and returns, so the call fails with
SB_ERR_TIMEOUT and the device context stays usable. These tests make waits run out without
faulting or hanging anything: a wait on an mbarrier armed for bytes no copy delivers, and
Biot-Savart sweeps whose tile waits are given no polls at all (their copies are in flight
and land while the CTA drains them). Afterwards the same sweeps run to the oracle's result.
"""
import json

import numpy as np
import pytest

from stormbird_gb300 import SbError, Simulation
from stormbird_gb300 import setups as S
from tests.helpers import rel_inf

SB_ERR_CUDA, SB_ERR_TIMEOUT = -4, -6


def _sweep_case():
    corners, strengths, cores, pts = S.synthetic_sail_row_wake(2, 16, 40, seed=4)
    return corners, strengths, cores, pts[::3]


@pytest.mark.gpu
def test_wait_on_a_barrier_no_copy_completes_runs_out(gpu_lib):
    for polls in (0, 8, 256):
        rc = gpu_lib.sb_wait_timeout_self_test(0, polls)
        assert rc == SB_ERR_TIMEOUT, gpu_lib.sb_last_error().decode()
        assert "bounded device-side wait ran out" in gpu_lib.sb_last_error().decode()


@pytest.mark.gpu
def test_sweep_leaves_when_its_waits_run_out_and_the_context_stays_usable(gpu_lib, oracle_mod):
    from stormbird_gb300.simulation import panel_sweep

    corners, strengths, cores, targets = _sweep_case()
    ref = oracle_mod.bs_sweep(corners, cores, strengths, 5.0, targets, nthreads=8)
    gpu_lib.sb_set_sweep_wait_polls(0)
    try:
        for mode in ("kahan", "fp32", "fp64"):
            with pytest.raises(SbError) as e:
                panel_sweep(corners, strengths, cores, targets, far_field_ratio=5.0, precision=mode)
            assert e.value.code == SB_ERR_TIMEOUT
    finally:
        gpu_lib.sb_set_sweep_wait_polls(-1)
    for mode in ("kahan", "fp32", "fp64"):
        got = panel_sweep(corners, strengths, cores, targets, far_field_ratio=5.0, precision=mode)
        assert rel_inf(got, ref) <= 1e-5, mode


@pytest.mark.gpu
def test_step_reports_a_timeout_and_a_new_simulation_runs(gpu_lib, oracle_mod):
    setup = S.wing_sail_row(nr_sails=2, panels_per_sail=8, wake_rows=12)
    wind = S.GustyWind(seed=0)
    sim = Simulation(setup)
    n = sim.nr_freestream_points
    for k in range(4):  # the roll-up sweep starts after three steps
        sim.do_step(time=0.05 * k, time_step=0.05, freestream_velocity=wind.freestream(0.05 * k, n))
    gpu_lib.sb_set_sweep_wait_polls(0)
    try:
        with pytest.raises(SbError) as e:
            sim.do_step(time=0.2, time_step=0.05, freestream_velocity=wind.freestream(0.2, n))
        assert e.value.code == SB_ERR_TIMEOUT
    finally:
        gpu_lib.sb_set_sweep_wait_polls(-1)
    sim.close()
    g, o = Simulation(setup), oracle_mod.OracleSimulation(setup)
    for k in range(5):
        fs = wind.freestream(0.05 * k, n)
        rg = g.do_step(time=0.05 * k, time_step=0.05, freestream_velocity=fs)
        ro = o.do_step(time=0.05 * k, time_step=0.05, freestream_velocity=fs)
        assert rel_inf(rg.circulation_strength, ro.circulation_strength) <= 1e-5


@pytest.mark.gpu
def test_device_allocation_failure_is_reported(gpu_lib):
    """A wake whose buffers exceed the GPU's memory: sb_sim_new returns NULL with SB_ERR_CUDA
    (cudaMalloc's out-of-memory error, released cleanly), and the next simulation builds."""
    d = json.loads(S.wing_sail_row(nr_sails=4, panels_per_sail=64, wake_rows=12))
    d["simulation_settings"]["Dynamic"]["wake"]["nr_panels_per_line_element"] = 100_000_000  # ~0.6 TB of wake points
    h = gpu_lib.sb_sim_new(json.dumps(d).encode(), 0)
    assert not h
    assert gpu_lib.sb_last_status() == SB_ERR_CUDA
    assert "cudaMalloc" in gpu_lib.sb_last_error().decode()
    sim = Simulation(S.wing_sail_row(nr_sails=1, panels_per_sail=8, wake_rows=5))
    r = sim.do_step(time=0.0, time_step=0.05, freestream_velocity=np.tile([10.0, 0.0, 0.0], (sim.nr_freestream_points, 1)))
    assert np.all(np.isfinite(r.circulation_strength))


def test_sim_new_without_a_usable_gpu_reports_a_cuda_error(gpu_lib):
    """On a machine without a GPU, a valid setup gets NULL and SB_ERR_CUDA (the first CUDA call
    fails), not a crash; the JSON is validated before that call."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = gpu_lib.sb_sim_new(S.wing_sail_row(1, 4, 5).encode(), 0)
    assert not h and gpu_lib.sb_last_status() == SB_ERR_CUDA
    h = gpu_lib.sb_sim_new(b"{not json", 0)
    assert not h and gpu_lib.sb_last_status() == -3
