"""ORACLE — TEST INFRASTRUCTURE ONLY.

ctypes binding of the f64 C++ restatement (oracle/sb_oracle.hpp). Imported by tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg only; the product package never
imports it. `OracleSimulation` mirrors the reference's pystormbird `Simulation`
(interfaces/pystormbird/src/lifting_line/simulation.rs:24-165).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from stormbird_gb300._abi import OutputBuffers, SbError, StepOutput, as_ptr, vec3_array

from . import build as _build

_LIB = None


def lib() -> ctypes.CDLL:
    global _LIB
    if _LIB is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        c_void_p, c_int, c_size_t, c_double = ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t, ctypes.c_double
        dp = ctypes.POINTER(ctypes.c_double)
        szp = ctypes.POINTER(ctypes.c_size_t)
        L.sbo_last_error.restype = ctypes.c_char_p
        L.sbo_sim_new.restype = c_void_p
        L.sbo_sim_new.argtypes = [ctypes.c_char_p, c_int]
        L.sbo_sim_free.argtypes = [c_void_p]
        L.sbo_sim_set_threads.argtypes = [c_void_p, c_int]
        L.sbo_sim_sizes.argtypes = [c_void_p, szp, szp, szp]
        L.sbo_sim_get_freestream_points.argtypes = [c_void_p, dp, c_size_t]
        L.sbo_sim_do_step.argtypes = [c_void_p, c_double, c_double, dp, c_size_t, ctypes.POINTER(StepOutput)]
        L.sbo_sim_induced_velocities.argtypes = [c_void_p, dp, c_size_t, dp]
        L.sbo_sim_set_translation_and_rotation_with_finite_difference.argtypes = [c_void_p, c_double, dp, dp]
        L.sbo_sim_set_translation_only.argtypes = [c_void_p, dp]
        L.sbo_sim_set_rotation_only.argtypes = [c_void_p, dp]
        L.sbo_sim_set_velocity_linear.argtypes = [c_void_p, dp]
        L.sbo_sim_set_velocity_angular.argtypes = [c_void_p, dp]
        L.sbo_sim_set_local_wing_angles.argtypes = [c_void_p, dp, c_size_t]
        L.sbo_sim_reset_previous_circulation.argtypes = [c_void_p]
        L.sbo_sim_set_previous_circulation.argtypes = [c_void_p, dp, c_size_t]
        L.sbo_sim_wake_sizes.argtypes = [c_void_p, szp, szp, szp, szp]
        L.sbo_sim_get_wake_state.argtypes = [c_void_p, dp, dp, dp]
        L.sbo_panel_unit_velocity.argtypes = [dp, c_double, c_double, dp, c_int, dp]
        L.sbo_line_unit_velocity.argtypes = [dp, dp, dp, c_double, dp]
        L.sbo_quad_area.restype = c_double
        L.sbo_quad_area.argtypes = [dp]
        L.sbo_rotate.argtypes = [dp, dp, c_int, dp]
        L.sbo_sigmoid.restype = c_double
        L.sbo_sigmoid.argtypes = [c_double, c_double, c_double]
        L.sbo_foil_eval.argtypes = [ctypes.c_char_p, c_double, dp]
        L.sbo_bs_sweep.argtypes = [dp, dp, dp, c_size_t, c_double, dp, c_size_t, dp, c_int]
        L.sbo_sim_state_size.argtypes = [c_void_p, ctypes.POINTER(c_size_t)]
        L.sbo_sim_get_state.argtypes = [c_void_p, dp, c_size_t]
        L.sbo_sim_set_state.argtypes = [c_void_p, dp, c_size_t]
        L.sbo_sim_skip_next_rollup.argtypes = [c_void_p]
        L.sbo_bs_sweep_sym.argtypes = [dp, dp, dp, c_size_t, c_double, c_int, dp, c_size_t, dp, c_int]
        L.sbo_sim_wind_freestream.argtypes = [c_void_p, ctypes.c_char_p, ctypes.c_char_p, c_double, c_double, dp,
                                              c_size_t]
        L.sbo_wind_velocity_at.argtypes = [ctypes.c_char_p, ctypes.c_char_p, dp, c_size_t, c_double, c_double, dp]
        L.sbo_csm_new.restype = c_void_p
        L.sbo_csm_new.argtypes = [ctypes.c_char_p]
        L.sbo_csm_free.argtypes = [c_void_p]
        L.sbo_csm_steady_state.argtypes = [c_void_p, c_double, c_double, c_double, c_double, dp, c_size_t]
        L.sbo_csm_local_wing_angles.argtypes = [c_void_p, dp, c_size_t]
        L.sbo_csm_set_local_wing_angles.argtypes = [c_void_p, dp, c_size_t]
        _LIB = L
    return _LIB


def _check(rc: int):
    if rc != 0:
        raise SbError(rc, lib().sbo_last_error().decode())


def _d(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


class OracleSimulation:
    """f64 reference-algorithm simulation with pystormbird's method names."""

    def __init__(self, setup_string: str, nthreads: int | None = None):
        L = lib()
        t = nthreads if nthreads is not None else (os.cpu_count() or 1)
        h = L.sbo_sim_new(setup_string.encode(), int(t))
        if not h:
            raise SbError(-3, L.sbo_last_error().decode())
        self._h = ctypes.c_void_p(h)
        n, s, nfs = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_size_t()
        _check(L.sbo_sim_sizes(self._h, ctypes.byref(n), ctypes.byref(s), ctypes.byref(nfs)))
        self.nr_span_lines, self.nr_wings = n.value, s.value
        self._out = OutputBuffers(self.nr_span_lines, self.nr_wings)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _LIB is not None:
            _LIB.sbo_sim_free(h)
            self._h = None

    def set_threads(self, n: int):
        _check(lib().sbo_sim_set_threads(self._h, int(n)))

    @property
    def nr_freestream_points(self) -> int:
        n, s, nfs = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_size_t()
        _check(lib().sbo_sim_sizes(self._h, ctypes.byref(n), ctypes.byref(s), ctypes.byref(nfs)))
        return nfs.value

    def get_freestream_velocity_points(self) -> np.ndarray:
        n = self.nr_freestream_points
        out = np.zeros((n, 3))
        _check(lib().sbo_sim_get_freestream_points(self._h, as_ptr(out), n))
        return out

    def do_step(self, *, time: float, time_step: float, freestream_velocity):
        fs = vec3_array(freestream_velocity)
        _check(lib().sbo_sim_do_step(self._h, float(time), float(time_step), as_ptr(fs), fs.shape[0],
                                     ctypes.byref(self._out.struct)))
        return self._out.to_result(time)

    def induced_velocities(self, points) -> np.ndarray:
        p = vec3_array(points)
        out = np.zeros_like(p)
        _check(lib().sbo_sim_induced_velocities(self._h, as_ptr(p), p.shape[0], as_ptr(out)))
        return out

    def set_translation_and_rotation_with_finite_difference_for_the_velocity(self, time_step, translation, rotation):
        _check(lib().sbo_sim_set_translation_and_rotation_with_finite_difference(
            self._h, float(time_step), as_ptr(_d(translation)), as_ptr(_d(rotation))))

    def set_translation_only(self, translation):
        _check(lib().sbo_sim_set_translation_only(self._h, as_ptr(_d(translation))))

    def set_rotation_only(self, rotation):
        _check(lib().sbo_sim_set_rotation_only(self._h, as_ptr(_d(rotation))))

    def set_velocity_linear(self, v):
        _check(lib().sbo_sim_set_velocity_linear(self._h, as_ptr(_d(v))))

    def set_velocity_angular(self, v):
        _check(lib().sbo_sim_set_velocity_angular(self._h, as_ptr(_d(v))))

    def set_local_wing_angles(self, angles):
        a = _d(angles)
        _check(lib().sbo_sim_set_local_wing_angles(self._h, as_ptr(a), a.size))

    def reset_previous_circulation_strength(self):
        _check(lib().sbo_sim_reset_previous_circulation(self._h))

    def set_previous_circulation_strength(self, g):
        a = _d(g)
        _check(lib().sbo_sim_set_previous_circulation(self._h, as_ptr(a), a.size))

    def wind_freestream(self, environment_json: str, condition_json: str, time: float, ship_velocity: float):
        """CompleteSailModel::freestream_velocity at this simulation's freestream points."""
        out = np.zeros((self.nr_freestream_points, 3))
        _check(lib().sbo_sim_wind_freestream(self._h, environment_json.encode(), condition_json.encode(), float(time),
                                             float(ship_velocity), as_ptr(out), out.shape[0]))
        return out

    def state(self) -> np.ndarray:
        """State between steps, in the GPU library's sb_sim_get_state layout."""
        n = ctypes.c_size_t()
        _check(lib().sbo_sim_state_size(self._h, ctypes.byref(n)))
        out = np.zeros(n.value)
        _check(lib().sbo_sim_get_state(self._h, as_ptr(out), out.size))
        return out

    def set_state(self, state):
        a = _d(state).reshape(-1)
        _check(lib().sbo_sim_set_state(self._h, as_ptr(a), a.size))

    def skip_next_rollup(self):
        """The next step leaves the wake's induced velocity out of the velocity at the wake
        points (harness option: that step's circulation and forces do not depend on it)."""
        _check(lib().sbo_sim_skip_next_rollup(self._h))

    def wake_state(self):
        npts, npan, nspan, W = (ctypes.c_size_t() for _ in range(4))
        _check(lib().sbo_sim_wake_sizes(self._h, ctypes.byref(npts), ctypes.byref(npan), ctypes.byref(nspan),
                                        ctypes.byref(W)))
        p = np.zeros((npts.value, 3))
        s = np.zeros(npan.value)
        v = np.zeros((npts.value, 3))
        _check(lib().sbo_sim_get_wake_state(self._h, as_ptr(p), as_ptr(s), as_ptr(v)))
        return p, s, v


def panel_unit_velocity(corners, far_field_ratio, core, x, mode=0) -> np.ndarray:
    out = np.zeros(3)
    _check(lib().sbo_panel_unit_velocity(as_ptr(_d(corners).reshape(-1)), float(far_field_ratio), float(core),
                                         as_ptr(_d(x)), int(mode), as_ptr(out)))
    return out


def line_unit_velocity(a, b, x, core) -> np.ndarray:
    out = np.zeros(3)
    _check(lib().sbo_line_unit_velocity(as_ptr(_d(a)), as_ptr(_d(b)), as_ptr(_d(x)), float(core), as_ptr(out)))
    return out


def quad_area(corners) -> float:
    return lib().sbo_quad_area(as_ptr(_d(corners).reshape(-1)))


def rotate(v, r, rotation_type=0) -> np.ndarray:
    out = np.zeros(3)
    _check(lib().sbo_rotate(as_ptr(_d(v)), as_ptr(_d(r)), int(rotation_type), as_ptr(out)))
    return out


def sigmoid(x, x0, r) -> float:
    return lib().sbo_sigmoid(float(x), float(x0), float(r))


def foil_eval(foil_json: str, alpha: float) -> dict:
    out = np.zeros(6)
    _check(lib().sbo_foil_eval(foil_json.encode(), float(alpha), as_ptr(out)))
    return dict(zip(("cl", "cl_pre_stall", "cl_post_stall", "cd", "stall", "cl_linear"), out.tolist()))


def wind_velocity_at(environment_json: str, condition_json: str, points, time: float = 0.0,
                     ship_velocity: float = 0.0) -> np.ndarray:
    """Unsteady apparent wind of the reference's wind model at arbitrary points."""
    p = vec3_array(points)
    out = np.zeros_like(p)
    _check(lib().sbo_wind_velocity_at(environment_json.encode(), condition_json.encode(), as_ptr(p), p.shape[0],
                                      float(time), float(ship_velocity), as_ptr(out)))
    return out


def bs_sweep(corners, cores, strengths, far_field_ratio, targets, nthreads=1, symmetry=0) -> np.ndarray:
    c = _d(corners).reshape(-1, 12)
    t = vec3_array(targets)
    out = np.zeros_like(t)
    if symmetry:
        _check(lib().sbo_bs_sweep_sym(as_ptr(c), as_ptr(_d(cores)), as_ptr(_d(strengths)), c.shape[0],
                                      float(far_field_ratio), int(symmetry), as_ptr(t), t.shape[0], as_ptr(out),
                                      int(nthreads)))
        return out
    _check(lib().sbo_bs_sweep(as_ptr(c), as_ptr(_d(cores)), as_ptr(_d(strengths)), c.shape[0], float(far_field_ratio),
                              as_ptr(t), t.shape[0], as_ptr(out), int(nthreads)))
    return out


class OracleCompleteSailModel:
    """f64 restatement of CompleteSailModel's steady-state conditions (controller + wind + step)."""

    def __init__(self, setup_string: str, nr_sails: int):
        h = lib().sbo_csm_new(setup_string.encode())
        if not h:
            raise SbError(-3, lib().sbo_last_error().decode())
        self._h = ctypes.c_void_p(h)
        self.nr_sails = nr_sails

    def close(self):
        if self._h:
            lib().sbo_csm_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def simulate_steady_state_condition(self, velocity: float, direction: float, ship_velocity: float,
                                        loading: float) -> np.ndarray:
        """Per sail [force (3), moment (3), input power]."""
        out = np.zeros((self.nr_sails, 7))
        _check(lib().sbo_csm_steady_state(self._h, float(velocity), float(direction), float(ship_velocity),
                                          float(loading), as_ptr(out), self.nr_sails))
        return out

    def local_wing_angles(self) -> np.ndarray:
        out = np.zeros(self.nr_sails)
        _check(lib().sbo_csm_local_wing_angles(self._h, as_ptr(out), self.nr_sails))
        return out

    def set_local_wing_angles(self, angles):
        a = _d(angles)
        _check(lib().sbo_csm_set_local_wing_angles(self._h, as_ptr(a), a.size))
