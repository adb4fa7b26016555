"""WindEnvironment / WindCondition JSON used by the wind-model tests (the reference's schema,
wind/environment.rs:21-55 and wind/wind_condition/mod.rs:19-39)."""
import json
import math


def environment(inflow_corrections=False, nr_wings=2, water_plane_height=0.0) -> str:
    d = {"water_plane_height": water_plane_height}
    if inflow_corrections:
        dirs = [math.radians(a) for a in (-180.0, -60.0, 0.0, 45.0, 120.0, 180.0)]
        corr = []
        for k, _ in enumerate(dirs):
            hs, ms, angs, ranges = [], [], [], []
            for w in range(nr_wings):
                start = len(hs)
                for h in (0.0, 12.0, 25.0, 40.0):
                    hs.append(h)
                    ms.append(0.9 + 0.02 * k + 0.001 * h + 0.03 * w)
                    angs.append(math.radians(0.5 * k - 0.05 * h + w))
                ranges.append({"start": start, "end": len(hs)})
            corr.append({"height_values": hs, "magnitude_corrections": ms, "angle_corrections": angs,
                         "wing_indices": ranges})
        d["inflow_corrections"] = {"apparent_wind_directions": dirs, "corrections": corr}
    return json.dumps(d)


def condition(direction_deg=35.0, profile="power", gusts=True) -> str:
    if profile == "power":
        vv = {"PowerModel": {"reference_velocity": 9.0}}
    elif profile == "log":
        vv = {"LogarithmicModel": {"friction_velocity": 0.35, "surface_roughness": 2e-4, "obukhov_length": -80.0}}
    elif profile == "log_stable":
        vv = {"LogarithmicModel": {"friction_velocity": 0.35, "surface_roughness": 2e-4, "obukhov_length": 150.0}}
    else:
        vv = {"Constant": 9.0}
    d = {"direction_coming_from": math.radians(direction_deg), "velocity_variation": vv}
    if gusts:
        d["parallel_gust"] = {"frequencies": [0.1, 0.27, 0.45], "amplitudes": [0.6, 0.4, 0.2], "phases": [0.3, 1.7, 4.0]}
        d["perpendicular_gust"] = {"frequencies": [0.15, 0.31], "amplitudes": [0.3, 0.2], "phases": [2.0, 0.1]}
        d["vertical_gust"] = {"frequencies": [0.2], "amplitudes": [0.1], "phases": [1.0]}
    return json.dumps(d)
