"""Batched lifting-line cases on one GPU (the C ABI's sb_batch_* functions).

The reference runs independent cases as separate `Simulation`s, one `do_step` each
(stormbird/src/lifting_line/simulation.rs:107-203). `Batch` takes one setup JSON per case
and steps all of them together: every case computes what its own Simulation would, while
the Biot-Savart sweeps of all cases run as one persistent launch per sweep kind and the
steady step is replayed as a CUDA graph.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._abi import SB_ERR_BAD_JSON, OutputBuffers, SbError, as_ptr, vec3_array
from .native import lib

SUMMARY = 11  # SB_BATCH_SUMMARY
INFO_KEYS = ("last_step_ms", "pairs", "waves", "blocks_per_sm", "rollup_grid", "rollup_items", "tuned",
             "tune_candidates", "tune_best_ms", "graph", "steps", "tile", "schedule")


def _check(rc: int):
    if rc != 0:
        raise SbError(rc, lib().sb_last_error().decode())


class Batch:
    """Independent lifting-line cases stepped together on one GPU."""

    def __init__(self, setup_strings, device: int = 0):
        L = lib()
        enc = [s.encode() for s in setup_strings]
        arr = (ctypes.c_char_p * len(enc))(*enc)
        h = L.sb_batch_new(arr, len(enc), int(device))
        if not h:
            raise SbError(L.sb_last_status() or SB_ERR_BAD_JSON, L.sb_last_error().decode())
        self._h = ctypes.c_void_p(h)
        nc, nl, nf = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_size_t()
        _check(L.sb_batch_sizes(self._h, ctypes.byref(nc), ctypes.byref(nl), ctypes.byref(nf)))
        self.n_cases, self.total_lines, self.total_freestream = nc.value, nl.value, nf.value
        self.cases = []
        for i in range(self.n_cases):
            v = [ctypes.c_size_t() for _ in range(5)]
            _check(L.sb_batch_case_sizes(self._h, i, *(ctypes.byref(x) for x in v)))
            n, s, nfs, lo, fo = (x.value for x in v)
            self.cases.append({"lines": n, "wings": s, "freestream_points": nfs, "line_offset": lo,
                               "freestream_offset": fo})

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None:
            lib().sb_batch_free(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_freestream_velocity_points(self) -> np.ndarray:
        out = np.zeros((self.total_freestream, 3))
        _check(lib().sb_batch_get_freestream_points(self._h, as_ptr(out), self.total_freestream))
        return out

    def case_slice(self, i: int, what: str = "lines") -> slice:
        c = self.cases[i]
        if what == "lines":
            return slice(c["line_offset"], c["line_offset"] + c["lines"])
        return slice(c["freestream_offset"], c["freestream_offset"] + c["freestream_points"])

    def do_step(self, *, time: float, time_step: float, freestream_velocity):
        fs = vec3_array(freestream_velocity, self.total_freestream, "freestream_velocity")
        _check(lib().sb_batch_do_step(self._h, float(time), float(time_step), as_ptr(fs), fs.shape[0]))

    def do_step_device(self, *, time: float, time_step: float, freestream_device_ptr: int):
        _check(lib().sb_batch_do_step_device(self._h, float(time), float(time_step),
                                             ctypes.c_void_p(int(freestream_device_ptr)), self.total_freestream))

    def set_wind(self, environment_json: str, condition_jsons):
        """One WindEnvironment for all cases and one WindCondition per case (reference JSON)."""
        enc = [c.encode() for c in condition_jsons]
        if len(enc) != self.n_cases:
            raise SbError(-2, "one wind condition per case is needed")
        arr = (ctypes.c_char_p * len(enc))(*enc)
        _check(lib().sb_batch_set_wind(self._h, environment_json.encode(), arr))

    def do_step_wind(self, *, time: float, time_step: float, ship_velocities):
        """A step of every case with its freestream generated on the GPU from its wind model."""
        v = np.ascontiguousarray(np.broadcast_to(np.asarray(ship_velocities, dtype=np.float64), (self.n_cases,)))
        _check(lib().sb_batch_do_step_wind(self._h, float(time), float(time_step), as_ptr(v)))

    def circulation(self) -> np.ndarray:
        out = np.zeros(self.total_lines)
        _check(lib().sb_batch_get_circulation(self._h, as_ptr(out), out.size))
        return out

    def summary(self) -> np.ndarray:
        """[n_cases, 11]: force sum (3), moment sum (3), residual, iterations, converged, status,
        warm start taken (1 candidate, 0 plain start, -1 no candidate)."""
        out = np.zeros((self.n_cases, SUMMARY))
        _check(lib().sb_batch_get_summary(self._h, as_ptr(out), out.size))
        return out

    def read_case_output(self, i: int, time: float = 0.0):
        c = self.cases[i]
        buf = OutputBuffers(c["lines"], c["wings"])
        _check(lib().sb_batch_read_case_output(self._h, int(i), ctypes.byref(buf.struct)))
        return buf.to_result(time)

    def case_state(self, i: int) -> np.ndarray:
        """State of case i after the last step (the layout of Simulation.state())."""
        n = ctypes.c_size_t()
        _check(lib().sb_batch_case_state_size(self._h, int(i), ctypes.byref(n)))
        out = np.zeros(n.value)
        _check(lib().sb_batch_get_case_state(self._h, int(i), as_ptr(out), out.size))
        return out

    def set_warm_start(self, network_handle, mode: int = 1):
        """Warm start of every case's solve (sb_batch_set_warm_start): mode 1 with a network
        handle, 2 to record features and targets only, 0 off."""
        _check(lib().sb_batch_set_warm_start(self._h, network_handle, int(mode)))

    def set_warm_start_guard(self, margin: float):
        """Factor the network's start must beat the best other start by, on the mean and the
        largest per-line residual (sb_batch_set_warm_start_guard; default 0.5)."""
        _check(lib().sb_batch_set_warm_start_guard(self._h, float(margin)))

    def set_case_state(self, i: int, state):
        a = np.ascontiguousarray(np.asarray(state, dtype=np.float64).reshape(-1))
        _check(lib().sb_batch_set_case_state(self._h, int(i), as_ptr(a), a.size))

    def set_initial_circulation(self, circulation):
        a = np.ascontiguousarray(np.asarray(circulation, dtype=np.float64).reshape(-1))
        _check(lib().sb_batch_set_initial_circulation(self._h, as_ptr(a), a.size))

    def previous_circulation_device_ptr(self) -> int:
        p = ctypes.c_void_p()
        _check(lib().sb_batch_previous_circulation_device(self._h, ctypes.byref(p)))
        return int(p.value or 0)

    def set_precision(self, mode: str | int):
        m = {"kahan": 0, "fp32": 1, "fp64": 2}.get(mode, mode)
        _check(lib().sb_batch_set_precision(self._h, int(m)))

    def use_graph(self, on: bool = True):
        _check(lib().sb_batch_use_graph(self._h, 1 if on else 0))

    def autotune(self, budget_seconds: float = 5.0):
        _check(lib().sb_batch_autotune(self._h, float(budget_seconds)))

    def info(self) -> dict:
        v = np.zeros(len(INFO_KEYS))
        _check(lib().sb_batch_info(self._h, as_ptr(v), v.size))
        return dict(zip(INFO_KEYS, v.tolist()))
