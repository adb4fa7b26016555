"""The oracle's restatement of the reference's wind model, pinned by the reference's own
wind tests (run here on the CPU):
  * environment.rs test_true_wind_velocity_vectors: head, tail, starboard and port winds
    point along +x, -x, -y and +y;
  * logarithmic_model.rs test_businger_dyer_unscaled_correction_at_zero_height: the stable
    correction vanishes at zero height (so the profile is zero there);
and by closed forms of the power-law profile and the gust sum."""
import json
import math

import numpy as np
import pytest

from tests import wind_cases as W


@pytest.fixture(scope="module")
def wind_at(oracle_mod):
    return oracle_mod.wind_velocity_at


def test_true_wind_directions(wind_at):
    env = json.dumps({})
    at = [[0.0, 0.0, 10.0]]
    v = {name: wind_at(env, json.dumps({"direction_coming_from": math.radians(deg),
                                        "velocity_variation": {"Constant": 8.2}}), at)[0]
         for name, deg in (("head", 0.0), ("starboard", -90.0), ("port", 90.0), ("tail", 180.0))}
    assert v["head"][0] > 0.0 and v["tail"][0] < 0.0
    assert v["starboard"][1] < 0.0 and v["port"][1] > 0.0


def test_logarithmic_profile_zero_at_zero_height(wind_at):
    cond = json.dumps({"direction_coming_from": 0.0, "velocity_variation": {"LogarithmicModel": {
        "friction_velocity": 1.0, "surface_roughness": 0.001, "obukhov_length": 10.0}}})
    assert np.max(np.abs(wind_at(json.dumps({}), cond, [[0.0, 0.0, 0.0]]))) < 1e-6


def test_power_law_and_gusts_closed_form(wind_at):
    env = json.dumps({})
    cond = json.loads(W.condition(direction_deg=0.0, profile="power", gusts=True))
    t, z, ship = 3.7, 25.0, 4.0
    u = wind_at(env, json.dumps(cond), [[1.0, 2.0, z]], time=t, ship_velocity=ship)[0]
    g = cond["parallel_gust"]
    par = 9.0 * (z / 10.0) ** (1.0 / 9.0) + sum(a * math.sin(2 * math.pi * f * t + p)
                                                 for f, a, p in zip(g["frequencies"], g["amplitudes"], g["phases"]))
    gp = cond["perpendicular_gust"]
    per = sum(a * math.sin(2 * math.pi * f * t + p) for f, a, p in zip(gp["frequencies"], gp["amplitudes"], gp["phases"]))
    gv = cond["vertical_gust"]
    ver = sum(a * math.sin(2 * math.pi * f * t + p) for f, a, p in zip(gv["frequencies"], gv["amplitudes"], gv["phases"]))
    # direction 0: parallel along +x, perpendicular = up x (+x) = +y, vertical +z; ship along +x
    assert np.allclose(u, [par + ship, per, ver], rtol=1e-13, atol=1e-13)


def test_height_uses_the_water_plane(wind_at):
    cond = W.condition(profile="power", gusts=False)
    a = wind_at(W.environment(water_plane_height=5.0), cond, [[0.0, 0.0, 15.0]])
    b = wind_at(W.environment(water_plane_height=0.0), cond, [[0.0, 0.0, 10.0]])
    assert np.allclose(a, b, rtol=1e-15)


def test_wind_json_errors(oracle_mod):
    with pytest.raises(Exception):
        oracle_mod.wind_velocity_at(json.dumps({"not_a_field": 1}), W.condition(), [[0, 0, 1]])
    with pytest.raises(Exception):
        oracle_mod.wind_velocity_at("{}", json.dumps({"velocity_variation": {"Constant": 1.0}}), [[0, 0, 1]])
