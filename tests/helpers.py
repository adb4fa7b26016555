"""Shared helpers for the parity tests: run the GPU library and the oracle side by side."""
from __future__ import annotations

import json

import numpy as np

from stormbird_gb300 import setups as S


def rel_inf(a, b) -> float:
    """max |a - b| / max |b| (relative infinity-norm error of a against b)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (den if den > 0 else 1.0))


def rel_vec(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    n = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (n if n > 0 else 1.0))


def fixed_iterations(setup_json: str, iterations: int) -> str:
    """Same setup with tolerances 0 so every step runs exactly `iterations` iterations."""
    d = json.loads(setup_json)
    settings = d["simulation_settings"]
    body = settings.get("Dynamic") or settings.get("QuasiSteady")
    si = body.setdefault("solver", {}).setdefault("SimpleIterative", {})
    si["max_iterations_per_time_step"] = iterations
    si["residual_tolerance_absolute"] = 0.0
    si["strength_difference_tolerance"] = 0.0
    return json.dumps(d)


def run_pair(gpu_sim, oracle_sim, wind, steps, dt, every=1, motion=None):
    """Steps both simulations with the same freestream; yields (step, gpu_result, oracle_result)."""
    n = gpu_sim.nr_freestream_points
    assert n == oracle_sim.nr_freestream_points
    for k in range(steps):
        t = k * dt
        if motion is not None:
            motion(gpu_sim, oracle_sim, t)
        fs = wind.freestream(t, n) if hasattr(wind, "freestream") else np.tile(wind, (n, 1))
        rg = gpu_sim.do_step(time=t, time_step=dt, freestream_velocity=fs)
        ro = oracle_sim.do_step(time=t, time_step=dt, freestream_velocity=fs)
        if k % every == 0 or k == steps - 1:
            yield k, rg, ro


def small_row(nr_sails=2, panels=8, wake_rows=20, **kw) -> str:
    return S.wing_sail_row(nr_sails=nr_sails, panels_per_sail=panels, wake_rows=wake_rows, **kw)


def panel_corners(points, nr_points_along_span, wing_ranges, nr_rows):
    """Corners [P_pan, 4, 3] of the wake panels from the wake points, in the reference's
    panel indexing (stormbird/src/lifting_line/wake/dynamic_wake/mod.rs:82-103)."""
    P = np.asarray(points).reshape(nr_rows + 1, nr_points_along_span, 3)
    cols = []
    for w, (a, b) in enumerate(wing_ranges):
        for j in range(a, b):
            cols.append((j + w, j + 1 + w))
    c0 = np.array([c[0] for c in cols])
    c1 = np.array([c[1] for c in cols])
    corners = np.stack([P[:-1][:, c0], P[:-1][:, c1], P[1:][:, c1], P[1:][:, c0]], axis=2)
    return corners.reshape(-1, 4, 3)


def row_wing_ranges(nr_sails, panels):
    return [(i * panels, (i + 1) * panels) for i in range(nr_sails)]
