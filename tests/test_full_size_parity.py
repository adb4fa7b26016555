"""Full-size parity against the f64 oracle, from a shared state.

The oracle cannot shed a full wake in test time: its all-near-field roll-up of the 4 sail x
64 panel, 300-row case is 2.4e10 segment evaluations per step. So the GPU sheds the wake,
its state (wake points, velocity at the points, strengths, previous circulation and
flow-derivative history; sb_sim_get_state) is loaded into the oracle, and both take the next
step from that same state with the same freestream. Bar: relative circulation error
max|dGamma| / max|Gamma| <= 1e-5 and relative total-force error |dF| / |F| <= 1e-5, the
hot path's stated tolerance; where the oracle runs its roll-up too (far-field ratio 5), the
induced velocity at every wake point within 1e-5 of the largest (_check_rollup_velocities).
"""
import numpy as np
import pytest

from stormbird_gb300 import Batch, Simulation
from stormbird_gb300 import setups as S
from stormbird_gb300.warm_start import tight_solver
from tests.helpers import panel_corners, rel_inf, rel_vec, row_wing_ranges

pytestmark = pytest.mark.gpu

TOL = 1e-5
DT = 0.05


def _step_both(setup, state, t, fs, oracle_mod, with_rollup):
    g = Simulation(setup)
    g.set_state(state)
    o = oracle_mod.OracleSimulation(setup)
    o.set_state(state)
    assert np.array_equal(g.state(), state) and np.array_equal(o.state(), state)
    if not with_rollup:
        o.skip_next_rollup()
    rg = g.do_step(time=t, time_step=DT, freestream_velocity=fs)
    ro = o.do_step(time=t, time_step=DT, freestream_velocity=fs)
    return g, o, rg, ro


@pytest.mark.parametrize("far_field_ratio", [1e30, 5.0])
def test_wing_sail_row_full_size_step_from_shared_state(gpu_lib, oracle_mod, far_field_ratio):
    rows = 300
    bench_setup = S.wing_sail_row(4, 64, rows, time_step=DT, far_field_ratio=far_field_ratio)
    wind = S.GustyWind(seed=0)
    g = Simulation(bench_setup)
    n = g.nr_freestream_points
    for k in range(rows + 2):
        g.do_step(time=k * DT, time_step=DT, freestream_velocity=wind.freestream(k * DT, n))
    state = g.state()
    _, strengths, _ = g.wake_state()
    assert np.count_nonzero(strengths) == 4 * 64 * rows
    t = (rows + 2) * DT
    fs = wind.freestream(t, n)
    # the benchmark's own solver settings, and the same solve run to a tight residual
    for setup in (bench_setup, tight_solver(bench_setup, max_iterations=3000, residual_tolerance=1e-11)):
        gg, oo, rg, ro = _step_both(setup, state, t, fs, oracle_mod, with_rollup=far_field_ratio < 1e15)
        eg = rel_inf(rg.circulation_strength, ro.circulation_strength)
        ef = rel_vec(rg.integrated_forces_sum(), ro.integrated_forces_sum())
        assert eg <= TOL and ef <= TOL, f"circulation error {eg:.3e}, force error {ef:.3e}"
        assert abs(rg.iterations - ro.iterations) <= 1
        if far_field_ratio < 1e15:
            pts, strengths, vg = gg.wake_state()
            _, _, vo = oo.wake_state()
            ind_g, ind_o = vg - fs[64 * 4:], vo - fs[64 * 4:]
            _check_rollup_velocities(ind_g, ind_o, pts, strengths, far_field_ratio)
        gg.close()


def _check_rollup_velocities(ind_g, ind_o, pts, strengths, ratio):
    """Induced velocity at every wake point within 1e-5 of the largest. The near/far decision
    (|x - c|^2 <= far-field radius^2, panel.rs:53-57) is the f64 reference's at every pair: a
    pair whose FP32 distance lies in the narrow band FP32 cannot resolve is decided in f64,
    so no point takes the ring where the oracle takes the point doublet (which would differ by
    up to a few percent of that panel's contribution). On a miss, the message says whether a
    panel sits at the threshold."""
    err = np.linalg.norm(ind_g - ind_o, axis=1) / np.max(np.linalg.norm(ind_o, axis=1))
    bad = np.nonzero(err > TOL)[0]
    if bad.size:
        corners = panel_corners(pts, 4 * 65, row_wing_ranges(4, 64), 300)
        c = 0.25 * (((corners[:, 0] + corners[:, 1]) + corners[:, 2]) + corners[:, 3])
        la = np.linalg.norm(corners[:, 1] - corners[:, 0], axis=1)
        lb = np.linalg.norm(corners[:, 2] - corners[:, 1], axis=1)
        ff2 = (np.maximum(la, lb) * ratio) ** 2
        live = strengths != 0.0
        i = bad[np.argmax(err[bad])]
        gap = np.min(np.abs(np.sum((pts[i] - c[live]) ** 2, axis=1) / ff2[live] - 1.0))
        raise AssertionError(f"{bad.size} wake points beyond {TOL}; worst {i}: {err[i]:.2e}, nearest panel "
                             f"at the near/far threshold within {gap:.1e} relative")


def test_filled_uneven_case_in_a_batch_from_shared_state(gpu_lib, oracle_mod):
    """A config-3-sized case (3 sails x 48 panels, 120 wake rows, far-field ratio 5) filled
    inside a batch with two other uneven cases, stepped by graph replay; then one more batched
    step against the oracle's step from the batch's state of that case."""
    specs = [(3, 48, 120, 60.0, 9.0), (1, 20, 60, 140.0, 15.0), (5, 30, 80, 35.0, 6.0)]
    cases = [tight_solver(S.wing_sail_row(s, p, w, time_step=DT, wind_speed=u, apparent_wind_angle_deg=a),
                          residual_tolerance=1e-10)
             for s, p, w, a, u in specs]
    winds = [S.GustyWind(wind_speed=u, apparent_wind_angle_deg=a, seed=i) for i, (_, _, _, a, u) in enumerate(specs)]
    b = Batch(cases)
    steps = 122
    for k in range(steps):
        b.do_step(time=k * DT, time_step=DT, freestream_velocity=S.batch_freestream(b, winds, k * DT))
    assert b.info()["graph"] == 1.0
    state = b.case_state(0)
    o = oracle_mod.OracleSimulation(cases[0])
    o.set_state(state)
    t = steps * DT
    b.do_step(time=t, time_step=DT, freestream_velocity=S.batch_freestream(b, winds, t))
    rb = b.read_case_output(0, t)
    ro = o.do_step(time=t, time_step=DT, freestream_velocity=winds[0].freestream(t, o.nr_freestream_points))
    eg = rel_inf(rb.circulation_strength, ro.circulation_strength)
    ef = rel_vec(rb.integrated_forces_sum(), ro.integrated_forces_sum())
    assert eg <= TOL and ef <= TOL, f"circulation error {eg:.3e}, force error {ef:.3e}"
    b.close()


def test_state_round_trip_continues_like_the_original(gpu_lib):
    """A state moved to a second simulation of the same setup continues bit-identically."""
    setup = S.wing_sail_row(2, 8, 20, time_step=DT)
    wind = S.GustyWind(seed=5)
    a = Simulation(setup)
    n = a.nr_freestream_points
    for k in range(12):
        a.do_step(time=k * DT, time_step=DT, freestream_velocity=wind.freestream(k * DT, n))
    c = Simulation(setup)
    c.set_state(a.state())
    for k in range(12, 16):
        fs = wind.freestream(k * DT, n)
        ra = a.do_step(time=k * DT, time_step=DT, freestream_velocity=fs)
        rc = c.do_step(time=k * DT, time_step=DT, freestream_velocity=fs)
        assert np.array_equal(ra.circulation_strength, rc.circulation_strength)
        assert np.array_equal(ra.integrated_forces_sum(), rc.integrated_forces_sum())
    assert np.array_equal(a.state(), c.state())
