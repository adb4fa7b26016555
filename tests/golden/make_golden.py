"""Generates the committed golden fixtures in this folder. Run here, where the reference
tree is available (not on the GPU machines, which read only the committed outputs):

    python tests/golden/make_golden.py /path/to/stormbird

1. setup_stormbird_setup_*.json — setup documents emitted by the reference's own Python
   builders (interfaces/stormbird_setup, pydantic; lifting_line/simulation_builder.py:98-135),
   so the tests prove that the library reads exactly what the reference's users write.
2. golden_*.npz — per-step circulation, control-point velocity and integrated forces of
   the f64 oracle for those setups under a fixed seeded freestream, so the GPU tests can
   check against committed numbers and the oracle is pinned against regressions.
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def reference_setups(reference_root: str) -> dict:
    sys.path.insert(0, os.path.join(reference_root, "interfaces", "stormbird_setup", "src"))
    from stormbird_setup.lifting_line.simulation_builder import DynamicSettings, QuasiSteadySettings, SimulationBuilder
    from stormbird_setup.lifting_line.solver import SimpleIterative
    from stormbird_setup.lifting_line.wake import DynamicWakeBuilder, ViscousCoreLength
    from stormbird_setup.line_force_model import LineForceModelBuilder, WingBuilder
    from stormbird_setup.section_models import Foil, SectionModel
    from stormbird_setup.spatial_vector import SpatialVector as V

    def lfm():
        f = Foil(cl_initial_slope=2 * math.pi, mean_positive_stall_angle=math.radians(15.0),
                 mean_negative_stall_angle=math.radians(15.0), cd_min=0.01, cdi_correction_factor=0.05)
        b = LineForceModelBuilder(nr_sections=16)
        for i in range(2):
            b.add_wing_builder(WingBuilder(section_points=[V(x=40.0 * i), V(x=40.0 * i, z=30.0)],
                                           chord_vectors=[V(x=10.0), V(x=10.0)],
                                           section_model=SectionModel(model=f)))
        b.local_wing_angles = [math.radians(37.0), math.radians(37.0)]
        return b

    dyn = SimulationBuilder(
        line_force_model=lfm(),
        simulation_settings=DynamicSettings(
            solver=SimpleIterative(max_iterations_per_time_step=30, damping_factor=0.1),
            wake=DynamicWakeBuilder(nr_panels_per_line_element=30,
                                    viscous_core_length=ViscousCoreLength.new_absolute(1.0),
                                    first_panel_relative_length=0.06,
                                    ratio_of_wake_affected_by_induced_velocities=1.0)))
    qs = SimulationBuilder(line_force_model=lfm(), simulation_settings=QuasiSteadySettings())
    return {"dynamic": dyn.to_json_string(), "quasi_steady": qs.to_json_string()}


def run_oracle(setup: str, steps: int, dt: float, seed: int) -> dict:
    from oracle.binding import OracleSimulation
    from stormbird_gb300.setups import GustyWind

    sim = OracleSimulation(setup)
    wind = GustyWind(seed=seed)
    n = sim.nr_freestream_points
    out = {"gamma": [], "velocity": [], "force": [], "moment": [], "iterations": [], "residual": []}
    for k in range(steps):
        t = k * dt
        r = sim.do_step(time=t, time_step=dt, freestream_velocity=wind.freestream(t, n))
        out["gamma"].append(r.circulation_strength)
        out["velocity"].append(r.output_ctrl_points_velocity)
        out["force"].append(r.integrated_forces_sum())
        out["moment"].append(r.integrated_moments_sum())
        out["iterations"].append(r.iterations)
        out["residual"].append(r.residual)
    res = {k: np.array(v) for k, v in out.items()}
    res.update(dt=np.array(dt), seed=np.array(seed), steps=np.array(steps))
    return res


def main(reference_root: str):
    docs = reference_setups(reference_root)
    for name, js in docs.items():
        with open(os.path.join(HERE, f"setup_stormbird_setup_{name}.json"), "w") as f:
            f.write(js)
    np.savez(os.path.join(HERE, "golden_stormbird_setup_dynamic.npz"),
             **run_oracle(docs["dynamic"], steps=12, dt=0.05, seed=11))
    np.savez(os.path.join(HERE, "golden_stormbird_setup_quasi_steady.npz"),
             **run_oracle(docs["quasi_steady"], steps=3, dt=0.05, seed=12))
    print("written:", sorted(f for f in os.listdir(HERE) if f.startswith(("setup_", "golden_"))))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the reference checkout (NTNU-IMT/stormbird)>")
    main(sys.argv[1])
