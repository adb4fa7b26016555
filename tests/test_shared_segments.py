"""Shared-segment roll-up (chain records) in the all-near-field mode.

With far_field_ratio = 1e30 every panel pair is a vortex ring, and each wake segment lies on
two adjacent rings with opposite directions. The library then evaluates each segment once
with the strength difference. Checked on the GPU through the C ABI:
  * the same dynamic run with sharing on and off, step by step (circulation, forces,
    roll-up velocities), within the FP32 sweep tolerance; about half the evaluations;
  * the shared roll-up velocities against the oracle's ring sweep over the GPU's own wake;
  * the whole run against the oracle simulation at a fixed iteration count;
  * wings with different line counts (chains of fewer than four segments) and a batch.
"""
import math

import numpy as np
import pytest

from stormbird_gb300 import setups as S
from tests.helpers import fixed_iterations, panel_corners, rel_inf, rel_vec, run_pair

pytestmark = pytest.mark.gpu

DT = 0.05


def uneven_wings(rows=14, far_field_ratio=1e30):
    """Two sails with 6 and 9 lines (partial chains), roll-up of every wake point."""
    f = S.foil(cl_initial_slope=2 * math.pi, mean_positive_stall_angle=math.radians(15.0),
               mean_negative_stall_angle=math.radians(15.0), cd_min=0.01, cdi_correction_factor=0.05)
    wings = [S.wing_builder([(0, 0, 0), (0, 0, 30)], [(10, 0, 0), (10, 0, 0)], f, nr_sections=6),
             S.wing_builder([(40, 0, 0), (40, 0, 24)], [(8, 0, 0), (8, 0, 0)], f, nr_sections=9)]
    lfm = S.line_force_model(wings, 8, local_wing_angles=[math.radians(37.0), math.radians(37.0)])
    wake = S.dynamic_wake(nr_panels_per_line_element=rows, viscous_core_length={"Absolute": 1.0},
                          first_panel_relative_length=0.06, ratio_of_wake_affected_by_induced_velocities=1.0,
                          far_field_ratio=far_field_ratio)
    return S.simulation(lfm, dynamic=True, solver=S.simple_iterative(), wake=wake)


def test_shared_segments_match_rings(gpu_lib):
    from stormbird_gb300 import Simulation

    js = fixed_iterations(uneven_wings(rows=14), 20)
    on, off = Simulation(js), Simulation(js)
    off.set_segment_sharing(False)
    assert on.segment_sharing_active and not off.segment_sharing_active
    wind = S.GustyWind(seed=4)
    n = on.nr_freestream_points
    for k in range(20):  # past the wake length: every row carries circulation
        fs = wind.freestream(k * DT, n)
        a = on.do_step(time=k * DT, time_step=DT, freestream_velocity=fs)
        b = off.do_step(time=k * DT, time_step=DT, freestream_velocity=fs)
        assert rel_inf(a.circulation_strength, b.circulation_strength) <= 2e-6, k
        assert rel_vec(a.integrated_forces_sum(), b.integrated_forces_sum()) <= 2e-6, k
    _, _, va = on.wake_state()
    _, _, vb = off.wake_state()
    assert rel_inf(va, vb) <= 2e-6
    ca, cb = on.last_step_counters(), off.last_step_counters()
    assert ca["rollup_targets"] == cb["rollup_targets"]
    assert ca["rollup_segments"] < 0.6 * cb["rollup_segments"]


def test_shared_segments_match_oracle_sweep(gpu_lib, oracle_mod):
    from stormbird_gb300 import Simulation

    sails, panels, rows = 3, 16, 40
    g = Simulation(S.wing_sail_row(sails, panels, rows, far_field_ratio=1e30))
    assert g.segment_sharing_active
    wind = S.GustyWind(seed=2)
    n = g.nr_freestream_points
    for k in range(rows + 3):
        g.do_step(time=k * DT, time_step=DT, freestream_velocity=wind.freestream(k * DT, n))
    # the stored wake points and strengths are the inputs of the last step's roll-up, the
    # stored velocities its output (freestream + induced, update_data.rs:125-141)
    pts, strengths, vel = g.wake_state()
    corners = panel_corners(pts, sails * (panels + 1), [(i * panels, (i + 1) * panels) for i in range(sails)], rows)
    rng = np.random.default_rng(3)
    idx = np.sort(rng.choice(len(pts) - 1, 160, replace=False))
    uo = oracle_mod.bs_sweep(corners, np.full(len(strengths), 1.0), strengths, 1e30, pts[idx], nthreads=8)
    u_fs = wind.velocity((rows + 2) * DT)
    assert rel_inf(vel[idx], uo + u_fs) <= 1e-6


def test_shared_segments_dynamic_run_matches_oracle(gpu_lib, oracle_mod):
    from stormbird_gb300 import Simulation

    js = fixed_iterations(uneven_wings(rows=10), 15)
    g = Simulation(js)
    o = oracle_mod.OracleSimulation(js)
    assert g.segment_sharing_active
    for k, rg, ro in run_pair(g, o, S.GustyWind(seed=6), 14, DT):
        assert rel_inf(rg.circulation_strength, ro.circulation_strength) <= 1e-5, k
        assert rel_vec(rg.integrated_forces_sum(), ro.integrated_forces_sum()) <= 1e-5, k


def test_batch_with_shared_segments_matches_single(gpu_lib):
    from stormbird_gb300 import Batch, Simulation

    cases = S.uneven_cases(4, 31, sails=(1, 3), panels=(3, 10), wake_rows=(5, 12), far_field_ratio=1e30)
    cases = [(fixed_iterations(js, 12), w) for js, w in cases]
    b = Batch([js for js, _ in cases])
    sims = [Simulation(js) for js, _ in cases]
    winds = [w for _, w in cases]
    for k in range(14):
        b.do_step(time=k * DT, time_step=DT, freestream_velocity=S.batch_freestream(b, winds, k * DT))
        g = b.circulation()
        for i, (s, w) in enumerate(zip(sims, winds)):
            r = s.do_step(time=k * DT, time_step=DT, freestream_velocity=w.freestream(k * DT, s.nr_freestream_points))
            assert rel_inf(g[b.case_slice(i)], r.circulation_strength) <= 2e-6, (k, i)
