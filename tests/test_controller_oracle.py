"""The oracle's restatement of the reference's sail controller (controller/set_points.rs,
measurements.rs, input.rs; CompleteSailModel::apply_controller_based_on_freestream,
complete_sail_model/mod.rs:259-288), checked on the CPU against a numpy statement of the
same rules built on the oracle's own wind freestream:

  * geometric set points: new wing angle = measured apparent wind direction - loading x
    set point (set_points.rs:108-120), so the geometric angle of attack of the freestream
    on the new geometry equals loading x set point;
  * effective set points: new angle = wrap(current + wrap(measured AoA - set point))
    (set_points.rs:122-140), with the change-rate limit (set_points.rs:43-56, 83-89);
  * measurement windows: mean / max / min over strips [start_index, n - end_offset - 1)
    (measurements.rs:50-81: the last strip is never included).

No reference run or golden vector exists for the controller; these checks pin the
restatement's conventions (signs, windows, interpolation), not its bits."""
import json
import math

import numpy as np
import pytest

from stormbird_gb300 import setups as S

SAILS, PANELS = 2, 12


def _ctrl_velocity(oracle_mod, js, velocity, direction, angles=None):
    """The oracle's wind freestream at the control points of the model's lifting line."""
    lls = json.dumps(json.loads(js)["lifting_line_simulation"])
    sim = oracle_mod.OracleSimulation(lls, nthreads=1)
    if angles is not None:
        sim.set_local_wing_angles(angles)
    cond = json.dumps({"direction_coming_from": direction,
                       "velocity_variation": {"PowerModel": {"reference_velocity": velocity}}})
    v = sim.wind_freestream(json.dumps({}), cond, 0.0, 0.0)[:SAILS * PANELS]
    return v.reshape(SAILS, PANELS, 3)


def _signed_angle(a, b, axis):
    """stormath vector_math signed angle: |angle(a, b)|, sign of a . (b x axis)."""
    cosang = np.dot(a, b) / (np.linalg.norm(a) * np.linalg.norm(b))
    ang = math.acos(max(-1.0, min(1.0, cosang)))
    return ang if np.dot(a, np.cross(b, axis)) > 0.0 else -ang


def _set_point(direction, table):
    return np.interp(direction, table["apparent_wind_directions_data"], table["angle_of_attack_data"])


@pytest.mark.parametrize("direction_deg,loading", [(60.0, 0.7), (-120.0, 1.0), (5.0, 0.5), (170.0, 0.3)])
def test_geometric_set_points(oracle_mod, direction_deg, loading):
    js = S.complete_sail_model(SAILS, PANELS)
    m = oracle_mod.OracleCompleteSailModel(js, SAILS)
    d = math.radians(direction_deg)
    m.simulate_steady_state_condition(9.0, d, 0.0, loading)
    got = m.local_wing_angles()
    v = _ctrl_velocity(oracle_mod, js, 9.0, d)
    table = S.wing_sail_set_points()
    z = np.array([0.0, 0.0, 1.0])
    for w in range(SAILS):
        dirs = [_signed_angle(np.array([1.0, 0.0, 0.0]), v[w, i], z) for i in range(PANELS)]
        awd = float(np.mean(dirs[:PANELS - 1]))  # strips 0 .. n-2
        want = awd - loading * _set_point(awd, table)
        assert abs(got[w] - want) < 1e-12, (w, got[w], want)
        # the freestream's geometric angle of attack on the new geometry is loading x set point
        # (to 1e-7: the angles come from acos, whose conditioning near 0 loses ~8 digits)
        chord = np.array([math.cos(got[w]), math.sin(got[w]), 0.0])
        aoa = float(np.mean([_signed_angle(chord, v[w, i], z) for i in range(PANELS - 1)]))
        assert abs(aoa - loading * _set_point(awd, table)) < 1e-7


def test_effective_set_points_with_rate_limit(oracle_mod):
    sp = S.wing_sail_set_points(use_effective_angle_of_attack=True, max_local_wing_angle_change_rate=0.05)
    js = S.complete_sail_model(SAILS, PANELS, set_points=[sp, sp])
    m = oracle_mod.OracleCompleteSailModel(js, SAILS)
    start = np.array([0.3, -0.2])
    m.set_local_wing_angles(start)
    d, loading = math.radians(75.0), 0.8
    m.simulate_steady_state_condition(11.0, d, 0.0, loading)
    got = m.local_wing_angles()
    v = _ctrl_velocity(oracle_mod, js, 11.0, d, angles=start)
    z = np.array([0.0, 0.0, 1.0])
    table = S.wing_sail_set_points()
    for w in range(SAILS):
        chord = np.array([math.cos(start[w]), math.sin(start[w]), 0.0])
        aoa = float(np.mean([_signed_angle(chord, v[w, i], z) for i in range(PANELS - 1)]))
        awd = float(np.mean([_signed_angle(np.array([1.0, 0.0, 0.0]), v[w, i], z) for i in range(PANELS - 1)]))
        wrap = lambda a: (a + math.pi) % (2 * math.pi) - math.pi  # noqa: E731
        raw = wrap(start[w] + wrap(aoa - loading * _set_point(awd, table)))
        want = start[w] + math.copysign(0.05, raw - start[w]) if abs(raw - start[w]) > 0.05 else raw
        assert abs(got[w] - want) < 1e-12, (w, got[w], want, raw)


@pytest.mark.parametrize("kind,start_index,end_offset", [("Max", 2, 3), ("Min", 0, 1), ("Mean", 4, 20)])
def test_measurement_windows(oracle_mod, kind, start_index, end_offset):
    settings = {"measurement_type": kind, "start_index": start_index, "end_offset": end_offset}
    js = S.complete_sail_model(SAILS, PANELS, flow_measurement={"wind_direction": settings})
    m = oracle_mod.OracleCompleteSailModel(js, SAILS)
    d, loading = math.radians(100.0), 1.0
    m.simulate_steady_state_condition(8.0, d, 0.0, loading)
    got = m.local_wing_angles()
    v = _ctrl_velocity(oracle_mod, js, 8.0, d)
    z = np.array([0.0, 0.0, 1.0])
    table = S.wing_sail_set_points()
    end = PANELS - end_offset - 1
    end = PANELS - 1 if end < 0 else min(max(end, start_index + 1), PANELS - 1)
    f = {"Max": np.max, "Min": np.min, "Mean": np.mean}[kind]
    for w in range(SAILS):
        dirs = np.array([_signed_angle(np.array([1.0, 0.0, 0.0]), v[w, i], z) for i in range(PANELS)])
        awd = float(f(dirs[start_index:end]))
        want = awd - loading * _set_point(awd, table)
        assert abs(got[w] - want) < 1e-12, (w, got[w], want)
