"""The reference's own tests on the lifting-line path, run against the f64 oracle.

These pin the oracle (a C++ restatement; the Rust reference cannot be compiled here) to
the reference's known answers and tolerances. Each test names the reference test it
ports. CPU only.
"""
import math

import numpy as np
import pytest

from stormbird_gb300 import setups as S


def test_default_lift_coefficient(oracle_mod):
    """section_models/tests/foil.rs:22-36: Cl(5 deg) = 2 pi sin(alpha) within 1e-5."""
    a = math.radians(5.0)
    r = oracle_mod.foil_eval("{}", a)
    assert abs(r["cl"] - 2 * math.pi * math.sin(a)) < 1e-5


def test_large_angle_of_attack_drag_is_finite(oracle_mod):
    """section_models/tests/foil.rs:10-20 (prints only): Cd(80 deg) of the default foil."""
    r = oracle_mod.foil_eval("{}", math.radians(80.0))
    assert np.isfinite(r["cd"]) and r["cd"] > 0.5


def test_sigmoid(oracle_mod):
    """stormath/src/transition_functions.rs:54-70."""
    x0, rr = 2.4, 1.2
    assert abs(oracle_mod.sigmoid(x0, x0, rr) - 0.5) < 1e-9
    assert abs(oracle_mod.sigmoid(x0 - rr, x0, rr) - 0.01) < 1e-6
    assert abs(oracle_mod.sigmoid(x0 + rr, x0, rr) - 0.99) < 1e-6


def test_compare_near_and_far_field(oracle_mod):
    """singularity_elements/tests/vortex_panel.rs:19-74: ring vs point doublet within 2 %."""
    p0 = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], float)
    rot = [math.radians(45.0), math.radians(-10.0), 0.0]
    P = np.array([oracle_mod.rotate(p, rot) for p in p0])
    x = oracle_mod.rotate([5.0, 2.0, 1.0], rot)
    assert abs(oracle_mod.quad_area(P) - 1.0) < 1e-10
    un = oracle_mod.panel_unit_velocity(P, 3.0, 0.1, x, mode=1)
    uf = oracle_mod.panel_unit_velocity(P, 3.0, 0.1, x, mode=2)
    assert np.linalg.norm(un - uf) / np.linalg.norm(un) < 0.02


def test_xyz_rotation_against_blender(oracle_mod):
    """stormath/src/spatial_vector/transformations.rs:366-388 (golden values from Blender)."""
    r = [math.radians(30.0), math.radians(21.2), math.radians(-16.1)]
    out = oracle_mod.rotate([1.0, 1.0, 1.0], r)
    assert np.allclose(out, [1.47188, -0.043868, 0.91195], atol=1e-5)


def test_compare_rotations(oracle_mod):
    """transformations.rs:302-323: Euler XYZ equals three axis rotations (exact)."""
    r = [math.radians(30.0), math.radians(21.2), math.radians(-16.1)]
    v = [1.3, 1.2, 1.5]
    a = oracle_mod.rotate(v, r, 0)
    # yaw-pitch-roll of the reversed order is a different rotation; XYZ against Rodrigues:
    c = np.array(v)
    for axis, ang in zip(np.eye(3), r):
        k = axis
        c = c * math.cos(ang) + np.cross(k, c) * math.sin(ang) + k * np.dot(k, c) * (1 - math.cos(ang))
    assert np.allclose(a, c, atol=1e-14)


def test_yaw_pitch_roll_rotation(oracle_mod):
    """transformations.rs:390-420."""
    v = [1.2, 0.0, 0.0]
    assert np.allclose(oracle_mod.rotate(v, [0, 0, math.radians(90)], 1), [0, 1.2, 0], atol=1e-12)
    assert np.allclose(oracle_mod.rotate(v, [0, math.radians(90), 0], 1), [0, 0, -1.2], atol=1e-12)
    assert np.allclose(oracle_mod.rotate(v, [0, math.radians(-90), math.radians(90)], 1), [0, 0, 1.2], atol=1e-12)


def test_vortex_line_infinite_limit(oracle_mod):
    """Property: a straight segment of half-length L at distance d induces
    |u| = 2L / (4 pi d sqrt(L^2 + d^2)) (Biot-Savart law), -> 1 / (2 pi d) as L grows."""
    for L, d in ((1.0, 0.5), (30.0, 2.0), (1e3, 1.0)):
        u = oracle_mod.line_unit_velocity([0, 0, -L], [0, 0, L], [d, 0, 0], 0.0)
        exact = 2 * L / (4 * math.pi * d * math.sqrt(L * L + d * d))
        assert abs(np.linalg.norm(u) - exact) / exact < 1e-9
    assert abs(exact - 1.0 / (2 * math.pi)) < 1e-6
    # on the segment's own line the closeness cut-off returns zero (vortex_line.rs:35)
    assert np.all(oracle_mod.line_unit_velocity([0, 0, 0], [0, 0, 1], [0, 0, 0.5], 0.0) == 0.0)


def test_far_field_converges_to_doublet(oracle_mod):
    """Property: the ring/doublet discrepancy falls as distance grows (panel.rs:82-118)."""
    P = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], float)
    errs = []
    for d in (3.0, 6.0, 12.0, 24.0):
        x = [0.5 + d, 0.5, 0.4 * d]
        un = oracle_mod.panel_unit_velocity(P, 1e9, 0.05, x, mode=1)
        uf = oracle_mod.panel_unit_velocity(P, 1e9, 0.05, x, mode=2)
        errs.append(np.linalg.norm(un - uf) / np.linalg.norm(un))
    assert all(b < a for a, b in zip(errs, errs[1:])) and errs[-1] < 1e-3


def _elliptic(AR, cl0, aoa):
    cl2d = cl0 + 2 * math.pi * aoa
    cl = cl2d / (1 + 2 / AR)
    return cl, cl ** 2 / (math.pi * AR)


def test_steady_lift_quasi_steady(oracle_mod):
    """lifting_line/tests/compare_models.rs:28-168 (quasi-steady part): CL 7 %, CD 6 %."""
    AR, cl0, aoa = 5.0, 1.2, math.radians(2.0)
    clt, cdt = _elliptic(AR, cl0, aoa)
    sim = oracle_mod.OracleSimulation(S.simulation(S.rectangular_wing(AR, cl0, aoa, 64), False))
    v = [1.2, 0.0, 0.0]
    r = sim.do_step(time=0.0, time_step=0.25 / 1.2, freestream_velocity=np.tile(v, (sim.nr_freestream_points, 1)))
    ff = 0.5 * 13.2 * 1.2 ** 2 * AR
    f = r.integrated_forces_sum()
    assert abs(clt - f[1] / ff) / clt < 0.07
    assert abs(cdt - f[0] / ff) / cdt < 0.06


def test_steady_lift_dynamic(oracle_mod):
    """compare_models.rs:28-168 (dynamic part, 200 steps): CL 7 %, CD 6 %."""
    AR, cl0, aoa = 5.0, 1.2, math.radians(2.0)
    clt, cdt = _elliptic(AR, cl0, aoa)
    sim = oracle_mod.OracleSimulation(S.simulation(S.rectangular_wing(AR, cl0, aoa, 64), True))
    v = [1.2, 0.0, 0.0]
    dt = 0.25 / 1.2
    fs = np.tile(v, (sim.nr_freestream_points, 1))
    for i in range(200):
        r = sim.do_step(time=i * dt, time_step=dt, freestream_velocity=fs)
    ff = 0.5 * 13.2 * 1.2 ** 2 * AR
    f = r.integrated_forces_sum()
    assert abs(clt - f[1] / ff) / clt < 0.07
    assert abs(cdt - f[0] / ff) / cdt < 0.06


def test_right_force_magnitude_with_steady_forward_motion(oracle_mod):
    """lifting_line/tests/dynamic_simulation.rs:23-114: translation == inflow within 1e-5."""
    vm, AR = 5.2, 5.0
    js = S.simulation(S.rectangular_wing(AR, 0.5, 0.0, 20, negative_span_orientation=True), True)
    st, si = oracle_mod.OracleSimulation(js), oracle_mod.OracleSimulation(js)
    n = si.nr_freestream_points
    for i in range(1, 20):
        t = i * 0.1
        st.set_translation_and_rotation_with_finite_difference_for_the_velocity(0.1, [-vm * t, 0, 0], [0, 0, 0])
        rt = st.do_step(time=t, time_step=0.1, freestream_velocity=np.zeros((n, 3)))
        ri = si.do_step(time=t, time_step=0.1, freestream_velocity=np.tile([vm, 0, 0], (n, 1)))
        d = abs(rt.integrated_forces_sum()[1] - ri.integrated_forces_sum()[1]) / abs(ri.integrated_forces_sum()[1])
        assert d < 1e-5


def test_right_sign_of_the_force_when_translating(oracle_mod):
    """dynamic_simulation.rs:120-182: the y force opposes the y motion (quasi-steady)."""
    js = S.simulation(S.rectangular_wing(5.0, 0.0, 0.0, 20, negative_span_orientation=True), False)
    sim = oracle_mod.OracleSimulation(js)
    fs = np.tile([1.2, 0.0, 0.0], (sim.nr_freestream_points, 1))
    dt, period, amp = 0.1, 2.0, 0.23
    w = 2 * math.pi / period
    for i in range(1, 20):
        t = i * dt
        sim.set_translation_and_rotation_with_finite_difference_for_the_velocity(
            dt, [0.0, amp * math.sin(t * w), 0.0], [0.0, 0.0, 0.0])
        r = sim.do_step(time=t, time_step=dt, freestream_velocity=fs)
        assert r.integrated_forces_sum()[1] * (amp * w * math.cos(t * w)) <= 0.0


def test_right_sign_of_the_moment_when_rotating(oracle_mod):
    """dynamic_simulation.rs:184-245: the x moment opposes the x rotation (quasi-steady)."""
    js = S.simulation(S.rectangular_wing(5.0, 0.0, 0.0, 20, negative_span_orientation=True), False)
    sim = oracle_mod.OracleSimulation(js)
    fs = np.tile([10.2, 0.0, 0.0], (sim.nr_freestream_points, 1))
    period = 2.0
    dt = period / 20
    w = 2 * math.pi / period
    amp = math.radians(5.0)
    for i in range(1, 20):
        t = i * dt
        sim.set_translation_and_rotation_with_finite_difference_for_the_velocity(
            dt, [0.0, 0.0, 0.0], [amp * math.sin(w * t), 0.0, 0.0])
        r = sim.do_step(time=t, time_step=dt, freestream_velocity=fs)
        assert r.integrated_moments_sum()[0] * (amp * w * math.cos(w * t)) <= 0.0


def test_moment_arm(oracle_mod):
    """lifting_line/tests/steady_simulation.rs:16-70: moment arm -2.5 within 1e-3."""
    sim = oracle_mod.OracleSimulation(
        S.simulation(S.rectangular_wing(5.0, 0.5, 0.0, 20, negative_span_orientation=True), False))
    r = sim.do_step(time=0.0, time_step=1.0,
                    freestream_velocity=np.tile([1.2, 0, 0], (sim.nr_freestream_points, 1)))
    f, m = r.integrated_forces_sum(), r.integrated_moments_sum()
    assert f[1] < 0.0 and m[0] < 0.0
    assert abs(-m[0] / f[1] - (-2.5)) < 1e-3


def test_coordinate_systems(oracle_mod):
    """lifting_line/tests/coordinate_systems.rs:21-137 (core of it): a translated and
    rotated model gives the same body-frame forces as the model at the origin."""
    import json

    base = json.loads(S.simulation(S.rectangular_wing(5.0, 0.5, math.radians(3.0), 20), False))
    base["line_force_model"]["output_coordinate_system"] = "Body"
    moved = json.loads(json.dumps(base))
    rot = [0.0, 0.0, math.radians(20.0)]
    moved["line_force_model"]["rotation"] = {"x": rot[0], "y": rot[1], "z": rot[2]}
    moved["line_force_model"]["translation"] = {"x": 3.0, "y": -2.0, "z": 0.0}
    a = oracle_mod.OracleSimulation(json.dumps(base))
    b = oracle_mod.OracleSimulation(json.dumps(moved))
    u = np.array([4.0, 0.0, 0.0])
    ub = oracle_mod.rotate(u, rot)
    ra = a.do_step(time=0.0, time_step=1.0, freestream_velocity=np.tile(u, (a.nr_freestream_points, 1)))
    rb = b.do_step(time=0.0, time_step=1.0, freestream_velocity=np.tile(ub, (b.nr_freestream_points, 1)))
    assert np.allclose(ra.integrated_forces_sum(), rb.integrated_forces_sum(), rtol=1e-4, atol=1e-9)


@pytest.mark.parametrize("damping", [0.0, 0.25])
def test_oracle_wake_initialisation_is_straight(oracle_mod, damping):
    """initialization.rs:12-71: after the first step's initialisation the wake rows
    2..W-1 are spaced by dt * U along the mean freestream (no damping)."""
    js = S.wing_sail_row(1, 4, 10, time_step=0.1, wind_speed=10.0, apparent_wind_angle_deg=0.0,
                         angle_of_attack_deg=0.0)
    import json

    d = json.loads(js)
    d["simulation_settings"]["Dynamic"]["wake"]["shape_damping_factor"] = damping
    sim = oracle_mod.OracleSimulation(json.dumps(d))
    n = sim.nr_freestream_points
    sim.do_step(time=0.0, time_step=0.1, freestream_velocity=np.tile([10.0, 0, 0], (n, 1)))
    p, s, v = sim.wake_state()
    p = p.reshape(11, 5, 3)
    if damping == 0.0:
        d_rows = np.diff(p[2:10, :, 0], axis=0)
        assert np.allclose(d_rows, 1.0, atol=1e-9)
    assert np.allclose(v[:, 0], 10.0)


def test_panel_corner_reconstruction_matches_oracle_wake(oracle_mod):
    """The test helper that rebuilds wake panels from wake points (used to check the GPU
    sweep on the GPU's own wake) reproduces the oracle's induced velocities exactly."""
    from tests.helpers import panel_corners, row_wing_ranges, small_row

    sails, panels, rows = 2, 5, 8
    sim = oracle_mod.OracleSimulation(small_row(sails, panels, rows))
    wind = S.GustyWind(seed=9)
    n = sim.nr_freestream_points
    for k in range(6):
        sim.do_step(time=0.05 * k, time_step=0.05, freestream_velocity=wind.freestream(0.05 * k, n))
    pts, strengths, _ = sim.wake_state()
    corners = panel_corners(pts, sails * (panels + 1), row_wing_ranges(sails, panels), rows)
    targets = pts[::2] + 0.01
    a = oracle_mod.bs_sweep(corners, np.full(len(strengths), 1.0), strengths, 5.0, targets, nthreads=2)
    b = sim.induced_velocities(targets)
    assert np.array_equal(a, b)


def test_no_self_induced_velocity_rotor_sails(oracle_mod):
    """lifting_line/tests/no_self_induced_velocity.rs:22-137: two rotor sails (rotating
    cylinders, spin ratio 2) far apart with neglect_self_induced_velocities set, 100 dynamic
    steps of 0.5 s in a uniform 1.2 m/s flow: the force coefficients equal the section table's
    values at spin ratio 2, CD 1.497 within 5e-4 and CL 4.638 within 1e-4 (relative), the
    reference's own tolerances. Rotating cylinders run in the oracle only (the GPU path takes
    foil sections); the test pins the oracle's dynamic neglect-self path, its SimpleIterative
    defaults and its force integration against the reference's tabulated numbers."""
    diameter, span, u = 1.0, 5.0, 1.2
    rps = -(u * 2.0) / (math.pi * diameter)  # -revolutions_per_second_from_spin_ratio(2, D, U)
    cylinder = {"RotatingCylinder": {
        "revolutions_per_second": rps,
        "spin_ratio_data": [0.0, 1.0, 2.0, 3.0, 4.0, 5.0],
        "cd_data": [0.554, 0.674, 1.497, 2.877, 3.556, 3.816],
        "cl_data": [0.0, 1.889, 4.638, 6.794, 7.680, 7.950],
        "wake_angle_data": [0.0, math.radians(20.0), math.radians(25.0), math.radians(35.0), math.radians(45.0),
                            math.radians(60.0)]}}
    wings = [S.wing_builder([(x, y, 0.0), (x, y, span)], [(diameter, 0, 0), (diameter, 0, 0)], cylinder)
             for x, y in ((-1.0 * span, -10.0 * span), (1.0 * span, 10.0 * span))]
    lfm = {"wing_builders": wings, "nr_sections": 10}
    setup = S.simulation(lfm, dynamic=True, wake={"neglect_self_induced_velocities": True})
    sim = oracle_mod.OracleSimulation(setup, nthreads=2)
    n = sim.nr_freestream_points
    fs = np.tile([u, 0.0, 0.0], (n, 1))
    for i in range(100):
        r = sim.do_step(time=0.5 * i, time_step=0.5, freestream_velocity=fs)
    area = 2 * diameter * span  # total_projected_area: chord x span length of every strip
    force_factor = 0.5 * 1.225 * u ** 2 * area
    f = r.integrated_forces_sum()
    cd, cl = f[0] / force_factor, f[1] / force_factor
    assert abs(cd - 1.497) / 1.497 < 0.0005, cd
    assert abs(cl - 4.638) / 4.638 < 0.0001, cl


def test_rotating_cylinder_is_rejected_by_the_gpu_path_but_read_by_the_oracle(oracle_mod, gpu_lib):
    """The setup schema reads rotating cylinders for the oracle; the GPU library's setup
    rejects them as valid reference input outside its path (SB_ERR_UNSUPPORTED)."""
    wings = [S.wing_builder([(0, 0, 0), (0, 0, 5)], [(1, 0, 0), (1, 0, 0)], {"RotatingCylinder": {}})]
    setup = S.simulation({"wing_builders": wings, "nr_sections": 4}, dynamic=True)
    oracle_mod.OracleSimulation(setup)
    assert not gpu_lib.sb_sim_new(setup.encode(), 0) and gpu_lib.sb_last_status() == -7
