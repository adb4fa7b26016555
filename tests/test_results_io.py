"""Result output in the reference's formats (common_utils/results/simulation.rs):

  * the JSON history file (a JSON array of SimulationResult, the shape serde writes:
    simulation.rs:20-34, forces_and_moments.rs:22-72, rigid_body_motion.rs:22-28) holds, per
    step, exactly the values do_step returned (shortest round-trip numbers parse back to
    the same doubles), with the reference's field names;
  * sb_sim_result_json of the last step equals the history's last entry;
  * the CSV file holds the reduced header once and one row per step
    (as_reduced_flatten_csv_string, simulation.rs:168-205: "time, " then each wing's total
    force and moment), and a second writer on the same file appends rows without a header
    (io_utils/csv_data.rs:11-33).
"""
import json

import numpy as np
import pytest

from stormbird_gb300 import setups as S

pytestmark = pytest.mark.gpu

KEYS = {"time", "ctrl_points", "solver_input_ctrl_points_velocity", "force_input", "sectional_forces",
        "integrated_forces", "integrated_moments", "input_power", "iterations", "residual", "wing_indices",
        "rigid_body_motion"}
COMPONENTS = ["circulatory", "viscous_lift", "sectional_drag", "added_mass", "gyroscopic", "total"]


def _v(lst):
    return np.array([[p["x"], p["y"], p["z"]] for p in lst])


def _run(path, fmt, steps=5):
    from stormbird_gb300 import Simulation

    sim = Simulation(S.wing_sail_row(2, 8, 20, time_step=0.05))
    wind = S.GustyWind(seed=4)
    sim.write_results_to(str(path), fmt)
    results = []
    for k in range(steps):
        r = sim.do_step(time=0.05 * k, time_step=0.05, freestream_velocity=wind.freestream(0.05 * k, sim.nr_freestream_points))
        results.append((r.circulation_strength.copy(), r.integrated_forces_sum().copy(), r))
    sim.flush_results()
    return sim, results


def test_json_history(gpu_lib, tmp_path):
    path = tmp_path / "history.json"
    sim, results = _run(path, "json")
    last_json = json.loads(sim.result_json())
    sim.write_results_to(None)  # closes the array
    hist = json.loads(path.read_text())
    assert len(hist) == len(results)
    for k, (gamma, fsum, r) in enumerate(results):
        h = hist[k]
        assert set(h) == KEYS
        assert h["time"] == 0.05 * k
        assert np.array_equal(np.array(h["force_input"]["circulation_strength"]), gamma)
        assert set(h["force_input"]) == {"circulation_strength", "velocity", "angles_of_attack", "acceleration",
                                         "rotation_velocity", "coordinate_system"}
        assert h["force_input"]["coordinate_system"] == "Global"
        assert set(h["sectional_forces"]) == set(COMPONENTS) | {"coordinate_system"}
        tot = sum(_v([w["total"]])[0] for w in h["integrated_forces"])
        assert np.allclose(tot, fsum, rtol=1e-12, atol=0)
        assert [w["start"] for w in h["wing_indices"]] == [0, 8] and [w["end"] for w in h["wing_indices"]] == [8, 16]
        assert h["input_power"] == [0.0, 0.0]
        assert h["rigid_body_motion"]["rotation_type"] == "XYZ"
        assert isinstance(h["iterations"], int) and h["iterations"] == r.iterations
    assert hist[-1] == last_json
    last = results[-1][2]
    assert np.array_equal(_v(hist[-1]["ctrl_points"]), last.ctrl_points)
    assert np.array_equal(np.array(hist[-1]["force_input"]["angles_of_attack"]), last.force_input.angles_of_attack)


def test_csv_rows_and_append(gpu_lib, tmp_path):
    path = tmp_path / "forces.csv"
    sim, results = _run(path, "csv", steps=4)
    sim.write_results_to(None)
    lines = path.read_text().splitlines()
    want_header = ["time"]
    for w in range(2):
        want_header += [f"force_{w}.{a}" for a in "xyz"] + [f"moment_{w}.{a}" for a in "xyz"]
    assert lines[0] == ",".join(want_header)
    assert len(lines) == 1 + len(results)
    for k, line in enumerate(lines[1:]):
        t, rest = line.split(", ", 1)
        assert float(t) == 0.05 * k
        vals = np.array([float(x) for x in rest.split(",")]).reshape(2, 6)
        assert np.allclose(vals[:, :3].sum(axis=0), results[k][1], rtol=1e-12, atol=0)
    h, d = sim.as_reduced_flatten_csv_string()
    assert h == lines[0] and d == lines[-1]
    # a second writer on the existing file appends rows only
    sim2, results2 = _run(path, "csv", steps=2)
    sim2.write_results_to(None)
    lines2 = path.read_text().splitlines()
    assert len(lines2) == len(lines) + 2 and lines2[:len(lines)] == lines


def test_wake_vtk_files(gpu_lib, tmp_path):
    """A dynamic setup with write_wake_data_to_file writes, per step, the VTK PolyData file of
    lifting_line/wake/dynamic_wake/export.rs:75-163 to {folder}/wake_{time / dt as integer}.vtp:
    the wake's points and strengths as sb_sim_get_wake_state gives them (exact: shortest
    round-trip numbers), the panels' corner indices (dynamic_wake/mod.rs:82-91), offsets and
    the viscous core length of every panel."""
    import xml.etree.ElementTree as ET

    from stormbird_gb300 import Simulation

    sails, panels, rows, dt = 2, 6, 12, 0.05
    d = json.loads(S.wing_sail_row(sails, panels, rows, time_step=dt))
    wake = d["simulation_settings"]["Dynamic"]["wake"]
    wake["write_wake_data_to_file"] = True
    wake["wake_files_folder_path"] = str(tmp_path)
    sim = Simulation(json.dumps(d))
    wind = S.GustyWind(seed=9)
    N, Np = sails * panels, sails * (panels + 1)
    for k in range(4):
        t = dt * k
        sim.do_step(time=t, time_step=dt, freestream_velocity=wind.freestream(t, sim.nr_freestream_points))
        sim.flush_results()
        path = tmp_path / f"wake_{int(t / dt)}.vtp"
        root = ET.parse(path).getroot()
        piece = root.find("PolyData/Piece")
        assert piece.get("NumberOfPoints") == str(Np * (rows + 1)) and piece.get("NumberOfPolys") == str(N * rows)
        arrays = {a.get("Name"): a for a in root.iter("DataArray")}
        pts_file = np.array(piece.find("Points/DataArray").text.split(), dtype=float).reshape(-1, 3)
        pts, strengths, _ = sim.wake_state()
        assert np.array_equal(pts_file, pts)
        assert np.array_equal(np.array(arrays["strength"].text.split(), dtype=float), strengths)
        assert np.all(np.array(arrays["viscous_core_length"].text.split(), dtype=float) == 0.1 * S.CHORD)
        conn = np.array(arrays["connectivity"].text.split(), dtype=int).reshape(-1, 4)
        want = []
        for s_ in range(rows):
            for j in range(N):
                c = j + j // panels  # span index + wing index
                want.append([s_ * Np + c, s_ * Np + c + 1, (s_ + 1) * Np + c + 1, (s_ + 1) * Np + c])
        assert np.array_equal(conn, np.array(want))
        offs = np.array(arrays["offsets"].text.split(), dtype=int)
        assert np.array_equal(offs, 4 * np.arange(1, N * rows + 1))
