"""Setup builders that emit the reference's SimulationBuilder JSON.

The reference ships pydantic builders for this JSON (interfaces/stormbird_setup, e.g.
lifting_line/simulation_builder.py:98-135); those are not available where this package
runs, so the documents for the benchmark workloads and tests are written here as plain
dicts in the same schema (stormbird/src/lifting_line/simulation_builder.rs:21-63).

Workloads (sizes as the benchmark names them):
  * `quasi_steady_single_wing` — one rectangular wing sail, span 30 m, chord 10 m, 32
    panels, horseshoe wake 100 chords long, inflow 10 m/s at 8 deg, Foil with
    Cl slope 2*pi and smooth stall at 15 deg, Cd = 0.01 + 0.05 Cl^2, core 0.05 chord,
    damped fixed point (damping 0.1, tight tolerances).
  * `wing_sail_row` — S wing sails in a row 40 m apart on a deck, span 30 m, chord 10 m,
    P panels each, free wake of W shed rows rolled up by the induced velocity, dt 0.05 s,
    core 0.1 chord, first panel dt*U/c chords long.
  * `rectangular_wing` — the reference's own test fixture RectangularWing
    (stormbird/src/lifting_line/tests/test_setup.rs:12-76).
"""
from __future__ import annotations

import json
import math

import numpy as np


def vec(x=0.0, y=0.0, z=0.0) -> dict:
    return {"x": float(x), "y": float(y), "z": float(z)}


def foil(**kw) -> dict:
    """A `{"Foil": {...}}` section model; unspecified fields take the Rust defaults."""
    return {"Foil": {k: float(v) for k, v in kw.items()}}


def wing_builder(section_points, chord_vectors, section_model, nr_sections=None) -> dict:
    d = {
        "section_points": [vec(*p) for p in section_points],
        "chord_vectors": [vec(*c) for c in chord_vectors],
        "section_model": section_model,
        "non_zero_circulation_at_ends": [False, False],
    }
    if nr_sections is not None:
        d["nr_sections"] = int(nr_sections)
    return d


def line_force_model(wings, nr_sections, density=1.225, local_wing_angles=None, rotation=(0, 0, 0),
                     translation=(0, 0, 0), output_coordinate_system="Global") -> dict:
    d = {
        "wing_builders": list(wings),
        "nr_sections": int(nr_sections),
        "density": float(density),
        "rotation": vec(*rotation),
        "translation": vec(*translation),
        "output_coordinate_system": output_coordinate_system,
    }
    if local_wing_angles is not None:
        d["local_wing_angles"] = [float(a) for a in local_wing_angles]
    return d


def simple_iterative(max_iterations=40, damping=0.05, residual_tolerance=1e-4, strength_tolerance=1e-6,
                     **extra) -> dict:
    d = {"max_iterations_per_time_step": int(max_iterations), "damping_factor": float(damping),
         "residual_tolerance_absolute": float(residual_tolerance),
         "strength_difference_tolerance": float(strength_tolerance)}
    d.update(extra)
    return {"SimpleIterative": d}


def dynamic_wake(nr_panels_per_line_element=100, viscous_core_length=None, first_panel_relative_length=0.75,
                 last_panel_relative_length=0.25, ratio_of_wake_affected_by_induced_velocities=0.0,
                 far_field_ratio=5.0, **extra) -> dict:
    d = {"nr_panels_per_line_element": int(nr_panels_per_line_element),
         "first_panel_relative_length": float(first_panel_relative_length),
         "last_panel_relative_length": float(last_panel_relative_length),
         "ratio_of_wake_affected_by_induced_velocities": float(ratio_of_wake_affected_by_induced_velocities),
         "far_field_ratio": float(far_field_ratio)}
    if viscous_core_length is not None:
        d["viscous_core_length"] = viscous_core_length
    d.update(extra)
    return d


def simulation(lfm: dict, dynamic: bool, solver: dict | None = None, wake: dict | None = None) -> str:
    body = {}
    if solver is not None:
        body["solver"] = solver
    if wake is not None:
        body["wake"] = wake
    settings = {"Dynamic": body} if dynamic else {"QuasiSteady": body}
    return json.dumps({"line_force_model": lfm, "simulation_settings": settings})


def rotate_around_z(v, angle):
    """Rodrigues rotation about +z (stormath/src/spatial_vector/transformations.rs:139-150)."""
    c, s = math.cos(angle), math.sin(angle)
    x, y, z = v
    return (x * c - y * s, y * c + x * s, z)


# --------------------------------------------------------------------------------------
# Reference test fixture
# --------------------------------------------------------------------------------------
def rectangular_wing(aspect_ratio=5.0, cl_zero_angle=0.5, angle_of_attack=0.0, nr_strips=20,
                     negative_span_orientation=False) -> dict:
    """RectangularWing (stormbird/src/lifting_line/tests/test_setup.rs:12-76), density 13.2."""
    sgn = -1.0 if negative_span_orientation else 1.0
    # (1,0,0).rotate_around_axis(-aoa, +/-z)
    a = -angle_of_attack * sgn
    chord = (math.cos(a), math.sin(a), 0.0)
    last_z = sgn * aspect_ratio
    w = wing_builder([(0, 0, 0), (0, 0, last_z)], [chord, chord],
                     foil(cl_zero_angle=cl_zero_angle, mean_positive_stall_angle=math.radians(45.0),
                          mean_negative_stall_angle=math.radians(45.0)))
    return line_force_model([w], nr_strips, density=13.2)


# --------------------------------------------------------------------------------------
# Benchmark workloads
# --------------------------------------------------------------------------------------
SPAN = 30.0
CHORD = 10.0


def quasi_steady_single_wing(nr_panels=32) -> tuple[str, np.ndarray]:
    """Quasi-steady static case; returns (setup JSON, freestream vector)."""
    f = foil(cl_initial_slope=2 * math.pi, mean_positive_stall_angle=math.radians(15.0),
             mean_negative_stall_angle=math.radians(15.0), cd_min=0.01, cdi_correction_factor=0.05)
    w = wing_builder([(0, 0, 0), (0, 0, SPAN)], [(CHORD, 0, 0), (CHORD, 0, 0)], f)
    lfm = line_force_model([w], nr_panels)
    solver = {"SimpleIterative": {"max_iterations_per_time_step": 1000, "damping_factor": 0.1,
                                  "residual_tolerance_absolute": 1e-8, "strength_difference_tolerance": 1e-7}}
    wake = {"wake_length_factor": 100.0, "viscous_core_length": {"Absolute": 0.05 * CHORD}}
    aoa = math.radians(8.0)
    u = 10.0 * np.array([math.cos(aoa), math.sin(aoa), 0.0])
    return simulation(lfm, dynamic=False, solver=solver, wake=wake), u


def wing_sail_row(nr_sails=4, panels_per_sail=64, wake_rows=300, time_step=0.05, wind_speed=12.0,
                  apparent_wind_angle_deg=45.0, angle_of_attack_deg=8.0, far_field_ratio=5.0,
                  spacing=40.0, max_iterations=40, damping=0.05, residual_tolerance=1e-4,
                  strength_tolerance=1e-6, ratio_of_wake_affected=1.0) -> str:
    """Dynamic free-wake case: sails in a row on the deck, local angle = AWA - AoA."""
    f = foil(cl_initial_slope=2 * math.pi, mean_positive_stall_angle=math.radians(15.0),
             mean_negative_stall_angle=math.radians(15.0), cd_min=0.01, cdi_correction_factor=0.05)
    wings = [wing_builder([(spacing * i, 0, 0), (spacing * i, 0, SPAN)], [(CHORD, 0, 0), (CHORD, 0, 0)], f)
             for i in range(nr_sails)]
    local = [math.radians(apparent_wind_angle_deg - angle_of_attack_deg)] * nr_sails
    lfm = line_force_model(wings, panels_per_sail, local_wing_angles=local)
    wake = dynamic_wake(nr_panels_per_line_element=wake_rows, viscous_core_length={"Absolute": 0.1 * CHORD},
                        first_panel_relative_length=time_step * wind_speed / CHORD,
                        ratio_of_wake_affected_by_induced_velocities=ratio_of_wake_affected,
                        far_field_ratio=far_field_ratio)
    solver = simple_iterative(max_iterations, damping, residual_tolerance, strength_tolerance)
    return simulation(lfm, dynamic=True, solver=solver, wake=wake)


class GustyWind:
    """Uniform apparent wind with a parallel gust: U(t) = (U0 + sum_k a_k sin(2 pi f_k t + phi_k)) e.

    The gust is the reference's DiscretizedSpectrum form
    (stormbird/src/wind/wind_condition/discretized_spectrum.rs:38-46) with K seeded
    frequencies in [0.1, 0.5] Hz, phases in [0, 2 pi) and amplitudes normalised to a total
    of `gust_amplitude`.
    """

    def __init__(self, wind_speed=12.0, apparent_wind_angle_deg=45.0, gust_amplitude=1.5, nr_frequencies=8, seed=0):
        rng = np.random.default_rng(seed)
        self.frequencies = rng.uniform(0.1, 0.5, nr_frequencies)
        self.phases = rng.uniform(0.0, 2 * math.pi, nr_frequencies)
        a = rng.uniform(0.5, 1.0, nr_frequencies)
        self.amplitudes = a / a.sum() * gust_amplitude
        self.speed = wind_speed
        th = math.radians(apparent_wind_angle_deg)
        self.direction = np.array([math.cos(th), math.sin(th), 0.0])

    def velocity(self, t: float) -> np.ndarray:
        g = float(np.sum(self.amplitudes * np.sin(2 * math.pi * self.frequencies * t + self.phases)))
        return (self.speed + g) * self.direction

    def freestream(self, t: float, nr_points: int) -> np.ndarray:
        return np.tile(self.velocity(t), (nr_points, 1))

    def condition_json(self) -> str:
        """The same wind as a reference WindCondition (constant profile, parallel gust):
        the zero direction (1, 0, 0) turned by the angle about +z gives `direction`."""
        return json.dumps({"direction_coming_from": math.atan2(self.direction[1], self.direction[0]),
                           "velocity_variation": {"Constant": self.speed},
                           "parallel_gust": {"frequencies": self.frequencies.tolist(),
                                             "amplitudes": self.amplitudes.tolist(),
                                             "phases": self.phases.tolist()}})


def synthetic_sail_row_wake(nr_sails=4, panels_per_sail=64, wake_rows=300, time_step=0.05, wind_speed=12.0,
                            apparent_wind_angle_deg=45.0, angle_of_attack_deg=8.0, spacing=40.0, seed=0):
    """A shed-wake-shaped panel set without running the solver: for sail row geometry of
    `wing_sail_row`, rows of wake points leave the trailing edge along the wind with a
    growing sinusoidal roll-up displacement, and every panel carries an elliptic-like
    circulation with seeded +-10 % variation. Returns (corners [P, 4, 3], strengths [P],
    core lengths [P], wake points [(W+1) * Np, 3]) in the reference's panel indexing
    (stormbird/src/lifting_line/wake/dynamic_wake/mod.rs:82-103)."""
    rng = np.random.default_rng(seed)
    npts = panels_per_sail + 1
    th = math.radians(apparent_wind_angle_deg)
    wind = np.array([math.cos(th), math.sin(th), 0.0])
    ch = math.radians(apparent_wind_angle_deg - angle_of_attack_deg)
    chord_dir = np.array([math.cos(ch), math.sin(ch), 0.0])
    z = np.linspace(0.0, SPAN, npts)
    rows = []
    for s in range(wake_rows + 1):
        row = []
        for i in range(nr_sails):
            base = np.stack([np.full(npts, spacing * i), np.zeros(npts), z], axis=1)
            if s == 0:
                p = base
            else:
                p = base + chord_dir * (time_step * wind_speed) + wind * (time_step * wind_speed * (s - 1))
                roll = 0.02 * s * np.sin(np.pi * z / SPAN + 0.1 * s)
                p = p + np.outer(roll, [0.0, 0.0, 1.0]) + np.outer(0.01 * s * np.cos(np.pi * z / SPAN), [-wind[1], wind[0], 0])
            row.append(p)
        rows.append(np.concatenate(row))
    pts = np.stack(rows)  # [W+1, Np, 3]
    zc = 0.5 * (z[:-1] + z[1:])
    g_span = -30.0 * np.sqrt(np.clip(1.0 - (2 * zc / SPAN - 1.0) ** 2, 0.0, 1.0)) - 1.0
    # panel (row s, sail i, line j) has corners a, a+1 on row s and a+1, a on row s+1, a = i*npts + j
    a = np.array([i * npts + j for i in range(nr_sails) for j in range(panels_per_sail)])
    corners = np.stack([pts[:-1][:, a], pts[:-1][:, a + 1], pts[1:][:, a + 1], pts[1:][:, a]], axis=2).reshape(-1, 4, 3)
    strengths = np.tile(g_span, wake_rows * nr_sails) * rng.uniform(0.9, 1.1, wake_rows * nr_sails * panels_per_sail)
    cores = np.full(len(strengths), 0.1 * CHORD)
    return corners, strengths, cores, pts.reshape(-1, 3)


def uneven_cases(n_cases, seed=0, sails=(1, 6), panels=(16, 96), wake_rows=(50, 400), awa_deg=(20.0, 180.0),
                 wind_speed=(5.0, 20.0), time_step=0.05, gust_amplitude=1.5, **kw):
    """Independent dynamic cases drawn uniformly (seeded): apparent wind angle, wind speed,
    sail count, panels per sail and wake length, each sail row otherwise as wing_sail_row.

    Returns [(setup_json, GustyWind)], one per case; integer ranges are inclusive.
    """
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_cases):
        awa = float(rng.uniform(*awa_deg))
        u = float(rng.uniform(*wind_speed))
        s = int(rng.integers(sails[0], sails[1] + 1))
        p = int(rng.integers(panels[0], panels[1] + 1))
        w = int(rng.integers(wake_rows[0], wake_rows[1] + 1))
        js = wing_sail_row(nr_sails=s, panels_per_sail=p, wake_rows=w, time_step=time_step, wind_speed=u,
                           apparent_wind_angle_deg=awa, **kw)
        out.append((js, GustyWind(wind_speed=u, apparent_wind_angle_deg=awa, gust_amplitude=gust_amplitude,
                                  seed=int(rng.integers(0, 2**31)))))
    return out


def quasi_steady_cases(n_cases, seed=0, sails=(1, 6), panels=(16, 96), awa_deg=(20.0, 180.0),
                       wind_speed=(5.0, 20.0), angle_of_attack_deg=8.0, spacing=40.0):
    """Independent quasi-steady sail rows drawn uniformly (seeded), the shape of a
    CompleteSailModel wind-angle sweep: sail count, panels per sail, apparent wind angle and
    speed per case; local wing angle = AWA - AoA; the quasi-steady defaults (Linearized
    solver, horseshoe wake). Returns [(setup_json, freestream vector)]."""
    rng = np.random.default_rng(seed)
    f = foil(cl_initial_slope=2 * math.pi, mean_positive_stall_angle=math.radians(15.0),
             mean_negative_stall_angle=math.radians(15.0), cd_min=0.01, cdi_correction_factor=0.05)
    out = []
    for _ in range(n_cases):
        awa = float(rng.uniform(*awa_deg))
        u = float(rng.uniform(*wind_speed))
        s = int(rng.integers(sails[0], sails[1] + 1))
        p = int(rng.integers(panels[0], panels[1] + 1))
        wings = [wing_builder([(spacing * i, 0, 0), (spacing * i, 0, SPAN)], [(CHORD, 0, 0), (CHORD, 0, 0)], f)
                 for i in range(s)]
        lfm = line_force_model(wings, p, local_wing_angles=[math.radians(awa - angle_of_attack_deg)] * s)
        th = math.radians(awa)
        out.append((simulation(lfm, dynamic=False), u * np.array([math.cos(th), math.sin(th), 0.0])))
    return out


def wing_sail_set_points(max_angle_deg: float = 15.0, **extra) -> dict:
    """Set points of a single-element wing sail: angle-of-attack set point 0 for apparent wind
    within 10 deg of the bow, ramping to +/- max_angle at 15 deg and held to 180 deg (the
    reference's default, stormbird_setup/controller.py new_default_wing_sail_single_element)."""
    d = {"apparent_wind_directions_data": [math.radians(a) for a in (-180, -15, -10, 10, 15, 180)],
         "angle_of_attack_data": [math.radians(a) for a in
                                  (-max_angle_deg, -max_angle_deg, 0.0, 0.0, max_angle_deg, max_angle_deg)]}
    d.update(extra)
    return d


def complete_sail_model(nr_sails=2, panels_per_sail=24, spacing=40.0, set_points=None, flow_measurement=None,
                        wind_environment=None, solver=None, **controller_extra) -> str:
    """CompleteSailModelBuilder JSON (complete_sail_model/builder.rs:19-24): a quasi-steady row
    of wing sails (span 30 m, chord 10 m), the default wind environment, a controller with
    one set point table per sail."""
    f = foil(cl_initial_slope=2 * math.pi, mean_positive_stall_angle=math.radians(15.0),
             mean_negative_stall_angle=math.radians(15.0), cd_min=0.01, cdi_correction_factor=0.05)
    wings = [wing_builder([(spacing * i, 0, 0), (spacing * i, 0, SPAN)], [(CHORD, 0, 0), (CHORD, 0, 0)], f)
             for i in range(nr_sails)]
    lls = json.loads(simulation(line_force_model(wings, panels_per_sail), dynamic=False, solver=solver))
    controller = {"set_points": set_points if set_points is not None else [wing_sail_set_points()] * nr_sails}
    if flow_measurement is not None:
        controller["flow_measurement_settings"] = flow_measurement
    controller.update(controller_extra)
    return json.dumps({"lifting_line_simulation": lls,
                       "wind_environment": wind_environment if wind_environment is not None else {},
                       "controller": controller})


def setup_rollup_pairs(setup_json: str) -> int:
    """Panel-target pairs of a dynamic setup's roll-up sweep once its wake is full: every wake
    point (rows + 1 per span point) against every panel (rows per span line)."""
    d = json.loads(setup_json)
    wings = d["line_force_model"]["wing_builders"]
    nsec = d["line_force_model"]["nr_sections"]
    lines = sum(int(w.get("nr_sections") or nsec) for w in wings)  # straight wings: one segment each
    rows = d["simulation_settings"]["Dynamic"]["wake"]["nr_panels_per_line_element"]
    return (rows + 1) * (lines + len(wings)) * rows * lines


def batch_freestream(batch, winds, t: float) -> np.ndarray:
    """Freestream of every case of a Batch at time t, case after case."""
    return np.concatenate([w.freestream(t, c["freestream_points"]) for w, c in zip(winds, batch.cases)])
