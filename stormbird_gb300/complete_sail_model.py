"""CompleteSailModel: a lifting-line simulation with a wind environment and a sail controller.

Mirrors pystormbird's `CompleteSailModel` (interfaces/pystormbird/src/lifting_line/
complete_sail_model.rs: constructor from the CompleteSailModelBuilder JSON, keyword-only
`apply_controller_based_on_wind_condition`, `do_step`, `local_wing_angles`,
`set_local_wing_angles`) and cstormbird's `complete_sail_model_*` calls
(interfaces/cstormbird/src/lifting_line/complete_sail_model.rs: steady-state conditions from
a (velocity, direction) wind condition with per-sail force / moment / input power), over
the sb_csm_* functions of the C ABI. Sweeps of conditions run as one batch of replicas on
the GPU (`sweep_steady_state`, `simulate_condition_optimal_controller_loading`).

A wind condition is either a WindCondition JSON string (wind_condition/mod.rs:19-39) or a
`(velocity, direction_coming_from)` pair, which stands for cstormbird's WindCondition: a
power-law profile with that velocity at 10 m and factor 1/9 (interfaces/cstormbird/src/
wind.rs:15-33).
"""
from __future__ import annotations

import ctypes
import json

import numpy as np

from ._abi import SB_ERR_BAD_JSON, OutputBuffers, SbError, SingleSailResultC, WindConditionC, as_ptr
from .native import lib


def _check(rc: int):
    if rc < 0:
        raise SbError(rc, lib().sb_last_error().decode())


def power_model_condition(velocity: float, direction_coming_from: float) -> str:
    """cstormbird's WindCondition as a WindCondition JSON document."""
    return json.dumps({"direction_coming_from": float(direction_coming_from),
                       "velocity_variation": {"PowerModel": {"reference_velocity": float(velocity)}}})


def _condition_json(c) -> str:
    if isinstance(c, str):
        return c
    v, d = c
    return power_model_condition(v, d)


def _results(arr, n_sails: int, n: int = 1) -> np.ndarray:
    """[n][sails][7]: force (3), moment (3), input power."""
    out = np.zeros((n, n_sails, 7))
    for i in range(n):
        for w in range(n_sails):
            r = arr[i * n_sails + w]
            out[i, w, :3] = r.force[:]
            out[i, w, 3:6] = r.moment[:]
            out[i, w, 6] = r.input_power
    return out


class CompleteSailModel:
    """Sails (lifting line) + wind environment + controller on one GPU."""

    def __init__(self, setup_string: str, device: int = 0):
        L = lib()
        h = L.sb_csm_new(setup_string.encode(), int(device))
        if not h:
            raise SbError(L.sb_last_status() or SB_ERR_BAD_JSON, L.sb_last_error().decode())
        self._h = ctypes.c_void_p(h)
        self.nr_sails = L.sb_csm_get_number_of_sails(self._h)
        sim = ctypes.c_void_p()
        _check(L.sb_csm_sim(self._h, ctypes.byref(sim)))
        self._sim = sim
        n, s, nfs = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_size_t()
        _check(L.sb_sim_sizes(self._sim, ctypes.byref(n), ctypes.byref(s), ctypes.byref(nfs)))
        self.nr_span_lines = n.value
        self._out = OutputBuffers(n.value, s.value)

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None:
            lib().sb_csm_free(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- pystormbird API -----------------------------------------------------------------
    def apply_controller_based_on_wind_condition(self, *, time: float, time_step: float, wind_condition,
                                                 ship_velocity: float, controller_loading: float):
        _check(lib().sb_csm_apply_controller(self._h, float(time), float(time_step),
                                             _condition_json(wind_condition).encode(), float(ship_velocity),
                                             float(controller_loading)))

    def do_step(self, *, time: float, time_step: float, wind_condition, ship_velocity: float):
        _check(lib().sb_csm_do_step(self._h, float(time), float(time_step), _condition_json(wind_condition).encode(),
                                    float(ship_velocity), ctypes.byref(self._out.struct)))
        return self._out.to_result(time)

    def local_wing_angles(self) -> np.ndarray:
        out = np.zeros(self.nr_sails)
        _check(lib().sb_sim_get_local_wing_angles(self._sim, as_ptr(out), self.nr_sails))
        return out

    def set_local_wing_angles(self, local_wing_angles):
        a = np.ascontiguousarray(np.asarray(local_wing_angles, dtype=np.float64))
        _check(lib().sb_sim_set_local_wing_angles(self._sim, as_ptr(a), a.size))

    # -- cstormbird API ------------------------------------------------------------------
    def simulate_steady_state_condition(self, *, wind_velocity: float, wind_direction: float, ship_velocity: float,
                                        controller_loading: float) -> np.ndarray:
        """Per sail [force (3), moment (3), input power] of one steady-state condition."""
        res = (SingleSailResultC * self.nr_sails)()
        rc = lib().sb_csm_simulate_steady_state_condition(self._h, WindConditionC(wind_velocity, wind_direction),
                                                          float(ship_velocity), float(controller_loading), res,
                                                          self.nr_sails)
        _check(rc)
        return _results(res, self.nr_sails)[0]

    # -- batched -------------------------------------------------------------------------
    def sweep_steady_state(self, wind_velocities, wind_directions, ship_velocities, controller_loadings) -> np.ndarray:
        """[n][sails][7] for n conditions solved together, each on a replica of the model that
        starts from the model's current wing angles and motion."""
        v = np.atleast_1d(np.asarray(wind_velocities, dtype=np.float64))
        n = v.size
        d = np.broadcast_to(np.asarray(wind_directions, dtype=np.float64), (n,))
        s = np.ascontiguousarray(np.broadcast_to(np.asarray(ship_velocities, dtype=np.float64), (n,)))
        lo = np.ascontiguousarray(np.broadcast_to(np.asarray(controller_loadings, dtype=np.float64), (n,)))
        conds = (WindConditionC * n)(*[WindConditionC(float(v[i]), float(d[i])) for i in range(n)])
        res = (SingleSailResultC * (n * self.nr_sails))()
        _check(lib().sb_csm_sweep_steady_state(self._h, conds, as_ptr(s), as_ptr(lo), n, res, n * self.nr_sails))
        return _results(res, self.nr_sails, n)

    def simulate_condition_optimal_controller_loading(self, *, wind_velocity: float, wind_direction: float,
                                                      ship_velocity: float, nr_loadings_to_test: int):
        """(per-sail results [sails][7], best loading) over loadings linspace(0.1, 1, n)."""
        res = (SingleSailResultC * self.nr_sails)()
        best = ctypes.c_double()
        _check(lib().sb_csm_simulate_condition_optimal_controller_loading(
            self._h, WindConditionC(wind_velocity, wind_direction), float(ship_velocity), int(nr_loadings_to_test),
            res, self.nr_sails, ctypes.byref(best)))
        return _results(res, self.nr_sails)[0], best.value
