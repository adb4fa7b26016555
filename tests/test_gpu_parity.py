"""GPU parity: the CUDA library (through its C ABI) against the f64 oracle.

Tolerance (the hot path's stated bar): relative circulation error
max|Gamma_gpu - Gamma_ref| / max|Gamma_ref| <= 1e-5 and relative total-force error
|F_gpu - F_ref| / |F_ref| <= 1e-5 per step, with the Biot-Savart sweeps in FP32 with
compensated accumulation. Cases run the solver for a fixed number of iterations where the
convergence test would otherwise be the only difference (tolerances set to 0), and with
the reference's own tolerances elsewhere.
"""
import json
import math

import numpy as np
import pytest

from stormbird_gb300 import Simulation, SbError
from stormbird_gb300 import setups as S
from tests.helpers import fixed_iterations, panel_corners, rel_inf, rel_vec, row_wing_ranges, run_pair, small_row

pytestmark = pytest.mark.gpu

TOL = 1e-5


def pair(setup, oracle_mod):
    return Simulation(setup), oracle_mod.OracleSimulation(setup)


def check_step(k, rg, ro, tol=TOL):
    eg = rel_inf(rg.circulation_strength, ro.circulation_strength)
    ef = rel_vec(rg.integrated_forces_sum(), ro.integrated_forces_sum())
    assert eg <= tol, f"step {k}: circulation error {eg:.3e}"
    assert ef <= tol, f"step {k}: force error {ef:.3e}"
    return eg, ef


def test_dynamic_row_fixed_iterations(gpu_lib, oracle_mod):
    setup = fixed_iterations(small_row(2, 8, 20), 25)
    g, o = pair(setup, oracle_mod)
    wind = S.GustyWind(seed=1)
    worst = 0.0
    for k, rg, ro in run_pair(g, o, wind, steps=12, dt=0.05):
        assert rg.iterations == ro.iterations == 25
        worst = max(worst, *check_step(k, rg, ro))
    assert worst < TOL


def test_dynamic_row_reference_tolerances(gpu_lib, oracle_mod):
    setup = small_row(3, 12, 30)
    g, o = pair(setup, oracle_mod)
    wind = S.GustyWind(seed=2, apparent_wind_angle_deg=60.0)
    for k, rg, ro in run_pair(g, o, wind, steps=10, dt=0.05):
        check_step(k, rg, ro)
        assert abs(rg.iterations - ro.iterations) <= 1


def test_wake_state_matches_oracle(gpu_lib, oracle_mod):
    setup = fixed_iterations(small_row(2, 6, 15), 20)
    g, o = pair(setup, oracle_mod)
    wind = S.GustyWind(seed=3)
    for _ in run_pair(g, o, wind, steps=9, dt=0.05):
        pass
    pg, sg, vg = g.wake_state()
    po, so, vo = o.wake_state()
    # positions are integrated in f64 from FP32 induced velocities: ~1 um on a 50 m wake
    assert rel_inf(pg, po) < 1e-7, "wake points"
    assert rel_inf(sg, so) < TOL, "wake strengths"
    assert rel_inf(vg, vo) < TOL, "wake point velocities"


def test_freestream_points_match_oracle(gpu_lib, oracle_mod):
    setup = small_row(2, 8, 12)
    g, o = pair(setup, oracle_mod)
    assert rel_inf(g.get_freestream_velocity_points(), o.get_freestream_velocity_points()) < 1e-12


@pytest.mark.parametrize("mode,tol", [("kahan", 1e-6), ("fp32", 5e-6), ("fp64", 1e-12)])
def test_induced_velocities_precision_modes(gpu_lib, oracle_mod, mode, tol):
    """The sweep kernel alone: GPU induced velocities on the GPU's own wake state against
    the oracle's sweep (induced_velocity_calc.rs:111-126) over the same panels."""
    sails, panels, rows = 2, 8, 25
    setup = fixed_iterations(small_row(sails, panels, rows), 20)
    g = Simulation(setup)
    wind = S.GustyWind(seed=4)
    n = g.nr_freestream_points
    for k in range(8):
        g.do_step(time=0.05 * k, time_step=0.05, freestream_velocity=wind.freestream(0.05 * k, n))
    g.set_precision(mode)
    pts, strengths, _ = g.wake_state()
    corners = panel_corners(pts, sails * (panels + 1), row_wing_ranges(sails, panels), rows)
    rng = np.random.default_rng(0)
    targets = np.concatenate([pts[::3], rng.uniform([-20, -20, -5], [60, 40, 35], (200, 3))])
    ug = g.induced_velocities(targets)
    uo = oracle_mod.bs_sweep(corners, np.full(len(strengths), 1.0), strengths, 5.0, targets, nthreads=4)
    assert rel_inf(ug, uo) < tol


@pytest.mark.parametrize("ffr", [5.0, 1e30])
def test_full_size_wing_sail_row_sampled(gpu_lib, oracle_mod, ffr):
    """Full-size dynamic case (4 sails x 64 panels, 300 wake rows, 76,800 panels): after the
    wake is fully shed, the GPU sweep at sampled targets matches the oracle's sweep over the
    GPU's own wake, and the stored roll-up velocities equal freestream + induced velocity.
    With far_field_ratio 1e30 (the benchmark's setting) the roll-up runs on shared-segment
    chains and is checked against the ring sweep and the oracle the same way."""
    sails, panels, rows = 4, 64, 300
    g = Simulation(S.wing_sail_row(sails, panels, rows, far_field_ratio=ffr))
    wind = S.GustyWind(seed=8)
    n = g.nr_freestream_points
    for k in range(rows + 5):
        r = g.do_step(time=0.05 * k, time_step=0.05, freestream_velocity=wind.freestream(0.05 * k, n))
    assert np.all(np.isfinite(r.circulation_strength)) and r.iterations > 0
    pts, strengths, vel = g.wake_state()
    assert np.count_nonzero(strengths) == sails * panels * rows
    corners = panel_corners(pts, sails * (panels + 1), row_wing_ranges(sails, panels), rows)
    rng = np.random.default_rng(1)
    idx = np.sort(rng.choice(len(pts) - 1, 192, replace=False))
    targets = pts[idx]
    ug = g.induced_velocities(targets)
    uo = oracle_mod.bs_sweep(corners, np.full(len(strengths), 1.0), strengths, ffr, targets, nthreads=8)
    # FP32 sweep against f64: 307,200 segment evaluations per target when every pair is
    # near-field; with the default far-field ratio most pairs are point doublets instead
    tol = 2e-6 if ffr < 1e15 else 4e-6
    assert rel_inf(ug, uo) < tol
    # velocity_at_points = freestream + induced (update_data.rs:125-141), last step's freestream
    u_fs = wind.velocity(0.05 * (rows + 4))
    assert rel_inf(vel[idx], ug + u_fs) < tol / 2


def test_quasi_steady_simple_iterative_single_wing(gpu_lib, oracle_mod):
    setup, u = S.quasi_steady_single_wing()
    g, o = pair(setup, oracle_mod)
    n = g.nr_freestream_points
    rg = g.do_step(time=0.0, time_step=1.0, freestream_velocity=np.tile(u, (n, 1)))
    ro = o.do_step(time=0.0, time_step=1.0, freestream_velocity=np.tile(u, (n, 1)))
    check_step(0, rg, ro)
    assert rg.iterations == ro.iterations


def test_quasi_steady_simple_iterative_four_rows_per_thread(gpu_lib, oracle_mod):
    """2,400 span lines: each CTA of the 8-CTA cluster owns 300 (> 256) lines, so the solve
    runs the four-rows-per-thread variant; 30 fixed iterations against the oracle (the
    double-float matrix-vector product keeps the f64 result to ~1e-13)."""
    setup, u = S.quasi_steady_single_wing(nr_panels=2400)
    g, o = pair(fixed_iterations(setup, 30), oracle_mod)
    n = g.nr_freestream_points
    rg = g.do_step(time=0.0, time_step=1.0, freestream_velocity=np.tile(u, (n, 1)))
    ro = o.do_step(time=0.0, time_step=1.0, freestream_velocity=np.tile(u, (n, 1)))
    check_step(0, rg, ro, tol=1e-9)
    assert rg.iterations == ro.iterations == 30


def test_quasi_steady_linearized_default(gpu_lib, oracle_mod):
    lfm = S.rectangular_wing(5.0, 1.2, math.radians(2.0), 64)
    setup = S.simulation(lfm, dynamic=False)
    g, o = pair(setup, oracle_mod)
    v = np.array([1.2, 0.0, 0.0])
    rg = g.do_step(time=0.0, time_step=0.2, freestream_velocity=np.tile(v, (g.nr_freestream_points, 1)))
    ro = o.do_step(time=0.0, time_step=0.2, freestream_velocity=np.tile(v, (o.nr_freestream_points, 1)))
    check_step(0, rg, ro, tol=1e-9)


def test_translation_equals_inflow_on_gpu(gpu_lib):
    """Reference test right_force_magnitude_with_steady_forward_motion
    (stormbird/src/lifting_line/tests/dynamic_simulation.rs:23-114), tolerance 1e-5."""
    vm, AR = 5.2, 5.0
    lfm = S.rectangular_wing(AR, 0.5, 0.0, 20, negative_span_orientation=True)
    js = S.simulation(lfm, True)
    st, si = Simulation(js), Simulation(js)
    n = si.nr_freestream_points
    for i in range(1, 20):
        t = i * 0.1
        st.set_translation_and_rotation_with_finite_difference_for_the_velocity(0.1, [-vm * t, 0, 0], [0, 0, 0])
        rt = st.do_step(time=t, time_step=0.1, freestream_velocity=np.zeros((n, 3)))
        ri = si.do_step(time=t, time_step=0.1, freestream_velocity=np.tile([vm, 0, 0], (n, 1)))
        d = abs(rt.integrated_forces_sum()[1] - ri.integrated_forces_sum()[1]) / abs(ri.integrated_forces_sum()[1])
        assert d < 1e-5


def test_elliptic_wing_dynamic_on_gpu(gpu_lib):
    """Reference test steady_lift (stormbird/src/lifting_line/tests/compare_models.rs:28-168):
    dynamic CL within 7 % and CD within 6 % of elliptic wing theory."""
    AR, cl0, aoa = 5.0, 1.2, math.radians(2.0)
    cl2d = cl0 + 2 * math.pi * aoa
    clt = cl2d / (1 + 2 / AR)
    cdt = clt ** 2 / (math.pi * AR)
    sim = Simulation(S.simulation(S.rectangular_wing(AR, cl0, aoa, 64), True))
    v = np.array([1.2, 0.0, 0.0])
    dt = 0.25 / 1.2
    fs = np.tile(v, (sim.nr_freestream_points, 1))
    for i in range(200):
        r = sim.do_step(time=i * dt, time_step=dt, freestream_velocity=fs)
    ff = 0.5 * 13.2 * 1.2 ** 2 * AR
    f = r.integrated_forces_sum()
    assert abs(f[1] / ff - clt) / clt < 0.07
    assert abs(f[0] / ff - cdt) / cdt < 0.06


@pytest.mark.parametrize("variant", ["symmetry_z", "neglect_self", "damping", "freestream_dir", "actual_dir",
                                     "sin_core", "single_row"])
def test_wake_options_match_oracle(gpu_lib, oracle_mod, variant):
    d = json.loads(fixed_iterations(small_row(2, 6, 12), 15))
    w = d["simulation_settings"]["Dynamic"]["wake"]
    if variant == "symmetry_z":
        w["symmetry_condition"] = "Z"
        for wb in d["line_force_model"]["wing_builders"]:
            for p in wb["section_points"]:
                p["z"] += 1.0
    elif variant == "neglect_self":
        w["neglect_self_induced_velocities"] = True
    elif variant == "damping":
        w["shape_damping_factor"] = 0.3
    elif variant == "freestream_dir":
        w["first_wake_points_direction"] = "Freestream"
    elif variant == "actual_dir":
        w["first_wake_points_direction"] = "ActualVelocity"
    elif variant == "sin_core":
        w["viscous_core_length_evolution"] = {"SinIncrease": {"last_panel_value": {"Relative": 0.5}}}
    elif variant == "single_row":
        w["nr_panels_per_line_element"] = 1
    setup = json.dumps(d)
    g, o = pair(setup, oracle_mod)
    wind = S.GustyWind(seed=5)
    for k, rg, ro in run_pair(g, o, wind, steps=7, dt=0.05):
        check_step(k, rg, ro)


def test_motion_and_wing_angles_match_oracle(gpu_lib, oracle_mod):
    setup = fixed_iterations(small_row(2, 8, 15), 20)
    g, o = pair(setup, oracle_mod)

    def motion(gs, os_, t):
        tr = [0.3 * math.sin(t), 0.1 * t, 0.0]
        ro = [0.02 * math.sin(2 * t), 0.0, 0.05 * t]
        for s in (gs, os_):
            s.set_translation_and_rotation_with_finite_difference_for_the_velocity(0.05, tr, ro)
            s.set_local_wing_angles([math.radians(37.0 + 3 * math.sin(t)), math.radians(35.0)])

    for k, rg, ro in run_pair(g, o, S.GustyWind(seed=6), steps=8, dt=0.05, motion=motion):
        check_step(k, rg, ro)


def test_body_frame_output_matches_oracle(gpu_lib, oracle_mod):
    d = json.loads(fixed_iterations(small_row(2, 8, 10), 20))
    d["line_force_model"]["output_coordinate_system"] = "Body"
    d["line_force_model"]["rotation"] = {"x": 0.1, "y": 0.0, "z": 0.3}
    setup = json.dumps(d)
    g, o = pair(setup, oracle_mod)
    for k, rg, ro in run_pair(g, o, S.GustyWind(seed=7), steps=5, dt=0.05):
        check_step(k, rg, ro)
        assert rel_vec(rg.integrated_moments_sum(), ro.integrated_moments_sum()) < TOL


def test_error_codes(gpu_lib):
    g = Simulation(small_row(1, 4, 5))
    with pytest.raises(SbError) as e:
        g.do_step(time=0.0, time_step=0.1, freestream_velocity=np.zeros((3, 3)))
    assert e.value.code == -2
    fs = np.ones((g.nr_freestream_points, 3))
    fs[5, 1] = np.nan
    with pytest.raises(SbError) as e:
        g.do_step(time=0.0, time_step=0.1, freestream_velocity=fs)
    assert e.value.code == -5
    q = Simulation(S.simulation(S.rectangular_wing(), False))
    with pytest.raises(SbError) as e:
        q.induced_velocities([[0.0, 0.0, 0.0]])
    assert e.value.code == -8


@pytest.mark.parametrize("symmetry", [0, 2])
@pytest.mark.parametrize("ffr", [5.0, 1e30])
def test_standalone_panel_sweep_matches_oracle(gpu_lib, oracle_mod, symmetry, ffr):
    """sb_panel_sweep against the oracle's sweep over the same caller-given panels."""
    from stormbird_gb300.simulation import panel_sweep

    corners, strengths, cores, pts = S.synthetic_sail_row_wake(2, 12, 20, seed=3)
    rng = np.random.default_rng(2)
    targets = np.concatenate([pts[::5], rng.uniform([-10, -10, 1], [80, 60, 29], (100, 3))])
    if symmetry:
        targets[:, 1] += 5.0
    uo = oracle_mod.bs_sweep(corners, cores, strengths, ffr, targets, nthreads=4) if symmetry == 0 else None
    ug = panel_sweep(corners, strengths, cores, targets, far_field_ratio=ffr, symmetry=symmetry)
    u64 = panel_sweep(corners, strengths, cores, targets, far_field_ratio=ffr, symmetry=symmetry, precision="fp64")
    if uo is not None:
        assert rel_inf(u64, uo) < 1e-12
    assert rel_inf(ug, u64) < 2e-6


@pytest.mark.parametrize("precision", ["kahan", "fp32"])
def test_near_far_decision_at_the_threshold_is_the_f64_one(gpu_lib, oracle_mod, precision):
    """panel.rs:53-57 decides ring or point doublet by |x - c|^2 <= far-field radius^2 in f64.
    Targets at relative offsets 1e-9 .. 3e-5 on both sides of that radius, around a panel
    400 m from the origin (where FP32 coordinates alone are off by ~3e-5 m): the sweep takes
    the oracle's side at every one. The two sides differ by about a percent of the panel's
    velocity there, far above the FP32 evaluation error allowed below."""
    from stormbird_gb300.simulation import panel_sweep

    rng = np.random.default_rng(7)
    c0 = np.array([412.3, 287.9, 17.1])
    corners = c0 + np.array([[-0.25, -0.31, 0.0], [0.26, -0.3, 0.01], [0.24, 0.3, 0.0], [-0.25, 0.29, -0.01]])
    c = 0.25 * (((corners[0] + corners[1]) + corners[2]) + corners[3])
    r = 5.0 * max(np.linalg.norm(corners[1] - corners[0]), np.linalg.norm(corners[2] - corners[1]))
    offsets = np.array([s * d for d in (1e-9, 1e-8, 1e-7, 1e-6, 1e-5, 3e-5) for s in (-1.0, 1.0)])
    dirs = rng.normal(size=(16, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    targets = np.array([c + r * np.sqrt(1.0 + o) * d for d in dirs for o in offsets])
    core = 0.1
    uo = np.array([oracle_mod.panel_unit_velocity(corners, 5.0, core, x) for x in targets])
    ring = np.array([oracle_mod.panel_unit_velocity(corners, 5.0, core, x, mode=1) for x in targets])
    dbl = np.array([oracle_mod.panel_unit_velocity(corners, 5.0, core, x, mode=2) for x in targets])
    scale = np.linalg.norm(uo, axis=1)
    side_gap = np.linalg.norm(ring - dbl, axis=1) / scale
    assert side_gap.min() > 1e-3
    near = np.sum((targets - c) ** 2, axis=1) <= r * r
    assert np.array_equal(np.linalg.norm(uo - ring, axis=1) == 0.0, near)
    ug = panel_sweep(corners.reshape(1, 12), [1.0], [core], targets, far_field_ratio=5.0, precision=precision)
    err = np.linalg.norm(ug - uo, axis=1) / scale
    assert err.max() < 1e-4, f"worst target {np.argmax(err)}: {err.max():.2e} (side gap {side_gap.min():.1e})"


def test_step_timing_on_both_step_paths(gpu_lib):
    """sb_sim_enable_timing: phase and kernel times after a step with the freestream in host
    memory and after one with it in device memory (both paths read the step's events)."""
    torch = pytest.importorskip("torch")
    dt = 0.05
    sim = Simulation(S.wing_sail_row(2, 8, 12, time_step=dt))
    wind = S.GustyWind(seed=1)
    n = sim.nr_freestream_points
    for k in range(4):
        sim.do_step(time=k * dt, time_step=dt, freestream_velocity=wind.freestream(k * dt, n))
    sim.enable_timing(True)
    sim.do_step(time=4 * dt, time_step=dt, freestream_velocity=wind.freestream(4 * dt, n))
    t_host = sim.last_step_timing()
    fs = torch.from_numpy(np.ascontiguousarray(wind.freestream(5 * dt, n))).cuda()
    torch.cuda.synchronize()
    sim.do_step_device(time=5 * dt, time_step=dt, freestream_device_ptr=fs.data_ptr())
    t_dev = sim.last_step_timing()
    for t in (t_host, t_dev):
        for key in ("step", "solve", "wake_advect_kernel", "wake_panels_kernel", "rollup_sweep_kernel"):
            assert t[key] > 0.0, (key, t)
    sim.close()
