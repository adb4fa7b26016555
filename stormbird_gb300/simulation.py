"""Python host interface mirroring the reference's pystormbird `Simulation`.

Reference: interfaces/pystormbird/src/lifting_line/simulation.rs:24-165 — same class
name, constructor argument (the SimulationBuilder JSON string), method names, keyword-only
`do_step(*, time, time_step, freestream_velocity)` and setter names. Every call goes
through the C ABI of include/stormbird_gb300.h into the CUDA library; errors raise
`SbError` carrying the SB_ERR_* code (the reference panics or unwraps in these cases).
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._abi import SB_ERR_BAD_JSON, OutputBuffers, SbError, as_ptr, vec3_array
from .native import lib


def _check(rc: int):
    if rc != 0:
        raise SbError(rc, lib().sb_last_error().decode())


def _d(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


class Simulation:
    """A lifting-line simulation on one GPU (quasi-steady or dynamic, per the setup)."""

    def __init__(self, setup_string: str, device: int = 0):
        L = lib()
        h = L.sb_sim_new(setup_string.encode(), int(device))
        if not h:
            raise SbError(L.sb_last_status() or SB_ERR_BAD_JSON, L.sb_last_error().decode())
        self._h = ctypes.c_void_p(h)
        n, s, nfs = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_size_t()
        _check(L.sb_sim_sizes(self._h, ctypes.byref(n), ctypes.byref(s), ctypes.byref(nfs)))
        self.nr_span_lines, self.nr_wings, self.nr_freestream_points = n.value, s.value, nfs.value
        self._out = OutputBuffers(self.nr_span_lines, self.nr_wings)

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None:
            lib().sb_sim_free(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- reference API -----------------------------------------------------------------
    def get_freestream_velocity_points(self) -> np.ndarray:
        out = np.zeros((self.nr_freestream_points, 3))
        _check(lib().sb_sim_get_freestream_points(self._h, as_ptr(out), self.nr_freestream_points))
        return out

    def do_step(self, *, time: float, time_step: float, freestream_velocity):
        fs = vec3_array(freestream_velocity, self.nr_freestream_points, "freestream_velocity")
        _check(lib().sb_sim_do_step(self._h, float(time), float(time_step), as_ptr(fs), fs.shape[0],
                                    ctypes.byref(self._out.struct)))
        return self._out.to_result(time)

    def induced_velocities(self, points) -> np.ndarray:
        p = vec3_array(points)
        out = np.zeros_like(p)
        _check(lib().sb_sim_induced_velocities(self._h, as_ptr(p), p.shape[0], as_ptr(out)))
        return out

    def set_translation_and_rotation_with_finite_difference_for_the_velocity(self, time_step, translation, rotation):
        _check(lib().sb_sim_set_translation_and_rotation_with_finite_difference(
            self._h, float(time_step), as_ptr(_d(translation)), as_ptr(_d(rotation))))

    def set_translation_only(self, translation):
        _check(lib().sb_sim_set_translation_only(self._h, as_ptr(_d(translation))))

    def set_rotation_only(self, rotation):
        _check(lib().sb_sim_set_rotation_only(self._h, as_ptr(_d(rotation))))

    def set_velocity_linear(self, linear_velocity):
        _check(lib().sb_sim_set_velocity_linear(self._h, as_ptr(_d(linear_velocity))))

    def set_velocity_angular(self, angular_velocity):
        _check(lib().sb_sim_set_velocity_angular(self._h, as_ptr(_d(angular_velocity))))

    def set_local_wing_angles(self, local_wing_angles):
        a = _d(local_wing_angles)
        _check(lib().sb_sim_set_local_wing_angles(self._h, as_ptr(a), a.size))

    def local_wing_angles(self) -> np.ndarray:
        out = np.zeros(self.nr_wings)
        _check(lib().sb_sim_get_local_wing_angles(self._h, as_ptr(out), self.nr_wings))
        return out

    def reset_previous_circulation_strength(self):
        _check(lib().sb_sim_reset_previous_circulation(self._h))

    # -- additions of this library -------------------------------------------------------
    @property
    def previous_circulation_strength(self) -> np.ndarray:
        out = np.zeros(self.nr_span_lines)
        _check(lib().sb_sim_get_previous_circulation(self._h, as_ptr(out), out.size))
        return out

    @previous_circulation_strength.setter
    def previous_circulation_strength(self, g):
        a = _d(g)
        _check(lib().sb_sim_set_previous_circulation(self._h, as_ptr(a), a.size))

    def do_step_device(self, *, time: float, time_step: float, freestream_device_ptr: int):
        """do_step with the freestream already on the GPU (a device pointer to n*3 f64)."""
        _check(lib().sb_sim_do_step_device(self._h, float(time), float(time_step),
                                           ctypes.c_void_p(int(freestream_device_ptr)), self.nr_freestream_points))

    def read_output(self, time: float = 0.0):
        _check(lib().sb_sim_read_output(self._h, ctypes.byref(self._out.struct)))
        return self._out.to_result(time)

    def wake_state(self):
        """(points [P_pts, 3], strengths [P_pan], velocity at points [P_pts, 3])."""
        npts, npan, nspan, W = (ctypes.c_size_t() for _ in range(4))
        _check(lib().sb_sim_wake_sizes(self._h, ctypes.byref(npts), ctypes.byref(npan), ctypes.byref(nspan),
                                       ctypes.byref(W)))
        p = np.zeros((npts.value, 3))
        s = np.zeros(npan.value)
        v = np.zeros((npts.value, 3))
        _check(lib().sb_sim_get_wake_state(self._h, as_ptr(p), as_ptr(s), as_ptr(v)))
        return p, s, v

    def state(self) -> np.ndarray:
        """The state the next step reads (sb_sim_get_state layout): step counters, wake points,
        velocity at the points, strengths, previous circulation and flow-derivative history."""
        n = ctypes.c_size_t()
        _check(lib().sb_sim_state_size(self._h, ctypes.byref(n)))
        out = np.zeros(n.value)
        _check(lib().sb_sim_get_state(self._h, as_ptr(out), out.size))
        return out

    def set_state(self, state):
        a = np.ascontiguousarray(np.asarray(state, dtype=np.float64).reshape(-1))
        _check(lib().sb_sim_set_state(self._h, as_ptr(a), a.size))

    def wake_sizes(self) -> dict:
        npts, npan, nspan, W = (ctypes.c_size_t() for _ in range(4))
        _check(lib().sb_sim_wake_sizes(self._h, ctypes.byref(npts), ctypes.byref(npan), ctypes.byref(nspan),
                                       ctypes.byref(W)))
        return {"points": npts.value, "panels": npan.value, "points_along_span": nspan.value,
                "panels_per_line_element": W.value}

    def set_precision(self, mode: str | int):
        """Biot-Savart arithmetic: 'kahan' (FP32 compensated, default), 'fp32', 'fp64'."""
        m = {"kahan": 0, "fp32": 1, "fp64": 2}.get(mode, mode)
        _check(lib().sb_sim_set_precision(self._h, int(m)))

    def enable_timing(self, on: bool = True):
        _check(lib().sb_sim_enable_timing(self._h, 1 if on else 0))

    def last_step_timing(self) -> dict:
        ms = np.zeros(12)
        _check(lib().sb_sim_last_step_timing(self._h, as_ptr(ms), 12))
        keys = ("step", "wake_update", "free_wake_sweep", "unit_matrix", "solve", "rollup_sweep", "forces",
                "rollup_sweep_kernel", "free_wake_sweep_kernel", "wake_advect_kernel", "wake_panels_kernel",
                "chain_records_kernel")
        return dict(zip(keys, ms.tolist()))

    def last_step_counters(self) -> dict:
        c = np.zeros(7)
        _check(lib().sb_sim_last_step_counters(self._h, as_ptr(c), 7))
        keys = ("rollup_targets", "rollup_panels", "ctrl_targets", "free_wake_panels", "steps_completed",
                "kernel_launches", "rollup_segments")
        return dict(zip(keys, c.tolist()))

    # -- freestream from a wind model (CompleteSailModel::freestream_velocity on the GPU) --
    def set_wind(self, environment_json: str, condition_json: str):
        """WindEnvironment and WindCondition JSON of the reference (wind/environment.rs,
        wind/wind_condition/mod.rs)."""
        _check(lib().sb_sim_set_wind(self._h, environment_json.encode(), condition_json.encode()))

    def wind_freestream(self, *, time: float, ship_velocity: float) -> np.ndarray:
        out = np.zeros((self.nr_freestream_points, 3))
        _check(lib().sb_sim_wind_freestream(self._h, float(time), float(ship_velocity), as_ptr(out), out.shape[0]))
        return out

    def do_step_wind(self, *, time: float, time_step: float, ship_velocity: float):
        """do_step with the freestream generated on the GPU from the wind model."""
        _check(lib().sb_sim_do_step_wind(self._h, float(time), float(time_step), float(ship_velocity),
                                         ctypes.byref(self._out.struct)))
        return self._out.to_result(time)

    # -- result output (common_utils/results/simulation.rs) ------------------------------
    def result_json(self) -> str:
        """The last step's SimulationResult as the reference serialises it (write_to_file)."""
        n = ctypes.c_size_t()
        lib().sb_sim_result_json(self._h, None, 0, ctypes.byref(n))
        buf = ctypes.create_string_buffer(n.value)
        _check(lib().sb_sim_result_json(self._h, buf, n.value, ctypes.byref(n)))
        return buf.value.decode()

    def as_reduced_flatten_csv_string(self) -> tuple[str, str]:
        """(header, data) of the last step: time and each wing's total force and moment."""
        cap = 64 * (self.nr_wings + 1) * 8
        h, d = ctypes.create_string_buffer(cap), ctypes.create_string_buffer(cap * 4)
        _check(lib().sb_sim_result_csv(self._h, h, cap, d, cap * 4))
        return h.value.decode(), d.value.decode()

    def write_results_to(self, path: str | None, fmt: str = "json"):
        """Every following do_step / do_step_wind result is written to `path` on a background
        thread: "json" a JSON array of SimulationResult, "csv" reduced rows (None stops)."""
        code = {"json": 1, "csv": 2}[fmt] if path else 0
        _check(lib().sb_sim_set_result_file(self._h, path.encode() if path else None, code))

    def flush_results(self):
        _check(lib().sb_sim_flush_results(self._h))

    def set_segment_sharing(self, on: bool = True):
        """Shared-segment roll-up sweep (default on; used when every pair is near-field and all
        panels share one core length): each wake segment evaluated once with the strength
        difference of its two panels."""
        _check(lib().sb_sim_set_segment_sharing(self._h, 1 if on else 0))

    @property
    def segment_sharing_active(self) -> bool:
        v = ctypes.c_int()
        _check(lib().sb_sim_segment_sharing_active(self._h, ctypes.byref(v)))
        return bool(v.value)


def measure_fp32_peak(device: int = 0, reps: int = 5) -> float:
    """Measured FP32 FMA throughput (TFLOP/s) of a device, from the library's probe kernel."""
    v = ctypes.c_double()
    _check(lib().sb_measure_fp32_peak(int(device), int(reps), ctypes.byref(v)))
    return v.value


def measure_fp64_peak(device: int = 0, reps: int = 3) -> float:
    """Measured FP64 FMA throughput (TFLOP/s) of a device."""
    v = ctypes.c_double()
    _check(lib().sb_measure_fp64_peak(int(device), int(reps), ctypes.byref(v)))
    return v.value


def panel_sweep(corners, strengths, core_lengths, targets, far_field_ratio: float = 5.0, symmetry: int = 0,
                precision: str | int = "kahan", device: int = 0) -> np.ndarray:
    """Standalone Biot-Savart sweep over caller-given vortex-ring panels (sb_panel_sweep)."""
    c = _d(corners).reshape(-1, 12)
    s = _d(strengths).reshape(-1)
    r = _d(core_lengths).reshape(-1)
    t = vec3_array(targets)
    out = np.zeros_like(t)
    m = {"kahan": 0, "fp32": 1, "fp64": 2}.get(precision, precision)
    _check(lib().sb_panel_sweep(int(device), as_ptr(c), as_ptr(s), as_ptr(r), c.shape[0], float(far_field_ratio),
                                int(symmetry), as_ptr(t), t.shape[0], int(m), as_ptr(out)))
    return out
