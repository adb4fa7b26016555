"""ctypes mirror of include/stormbird_gb300.h and the Python-side result objects.

`SimulationResult` mirrors the reference's result structure
(stormbird/src/common_utils/results/simulation.rs:27-40, exposed to Python by
pystormbird's result_structs) with the fields and helpers the lifting-line callers use:
`integrated_forces_sum()`, `integrated_moments_sum()`, `force_input`, `sectional_forces`,
`iterations`, `residual`.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

SB_OK = 0
SB_ERR_NULL_ARG = -1
SB_ERR_SIZE = -2
SB_ERR_BAD_JSON = -3
SB_ERR_CUDA = -4
SB_ERR_NONFINITE = -5
SB_ERR_TIMEOUT = -6
SB_ERR_UNSUPPORTED = -7
SB_ERR_STATE = -8

ERROR_NAMES = {
    SB_ERR_NULL_ARG: "SB_ERR_NULL_ARG",
    SB_ERR_SIZE: "SB_ERR_SIZE",
    SB_ERR_BAD_JSON: "SB_ERR_BAD_JSON",
    SB_ERR_CUDA: "SB_ERR_CUDA",
    SB_ERR_NONFINITE: "SB_ERR_NONFINITE",
    SB_ERR_TIMEOUT: "SB_ERR_TIMEOUT",
    SB_ERR_UNSUPPORTED: "SB_ERR_UNSUPPORTED",
    SB_ERR_STATE: "SB_ERR_STATE",
}

COMPONENTS = ("circulatory", "viscous_lift", "sectional_drag", "added_mass", "gyroscopic", "total")

_dp = ctypes.POINTER(ctypes.c_double)


class StepOutput(ctypes.Structure):
    _fields_ = [
        ("circulation_strength", _dp),
        ("ctrl_points_velocity", _dp),
        ("solver_input_velocity", _dp),
        ("angles_of_attack", _dp),
        ("force_input_velocity", _dp),
        ("acceleration", _dp),
        ("ctrl_points", _dp),
        ("sectional_forces", _dp),
        ("integrated_forces", _dp),
        ("integrated_moments", _dp),
        ("force_sum", ctypes.c_double * 3),
        ("moment_sum", ctypes.c_double * 3),
        ("residual", ctypes.c_double),
        ("iterations", ctypes.c_int64),
        ("converged", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]


class WindConditionC(ctypes.Structure):
    """sb_wind_condition (cstormbird WindCondition)."""
    _fields_ = [("velocity", ctypes.c_double), ("direction_coming_from", ctypes.c_double)]


class SingleSailResultC(ctypes.Structure):
    """sb_single_sail_result (cstormbird SingleSailResult)."""
    _fields_ = [("force", ctypes.c_double * 3), ("moment", ctypes.c_double * 3), ("input_power", ctypes.c_double)]


class SbError(RuntimeError):
    """An SB_ERR_* status from the C ABI."""

    def __init__(self, code: int, message: str):
        self.code = code
        super().__init__(f"{ERROR_NAMES.get(code, code)}: {message}")


def as_ptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


@dataclass
class IntegratedValues:
    circulatory: np.ndarray
    viscous_lift: np.ndarray
    sectional_drag: np.ndarray
    added_mass: np.ndarray
    gyroscopic: np.ndarray
    total: np.ndarray


@dataclass
class SectionalForcesInput:
    circulation_strength: np.ndarray
    velocity: np.ndarray
    angles_of_attack: np.ndarray
    acceleration: np.ndarray


@dataclass
class SectionalForces:
    circulatory: np.ndarray
    viscous_lift: np.ndarray
    sectional_drag: np.ndarray
    added_mass: np.ndarray
    gyroscopic: np.ndarray
    total: np.ndarray


@dataclass
class SimulationResult:
    time: float
    ctrl_points: np.ndarray
    solver_input_ctrl_points_velocity: np.ndarray
    output_ctrl_points_velocity: np.ndarray
    force_input: SectionalForcesInput
    sectional_forces: SectionalForces
    integrated_forces: list = field(default_factory=list)
    integrated_moments: list = field(default_factory=list)
    iterations: int = 0
    residual: float = 0.0
    converged: bool = False
    force_sum: np.ndarray = None
    moment_sum: np.ndarray = None

    def integrated_forces_sum(self) -> np.ndarray:
        """Sum of the wings' total integrated force (results/simulation.rs:61-69)."""
        return self.force_sum.copy()

    def integrated_moments_sum(self) -> np.ndarray:
        """Sum of the wings' total integrated moment (results/simulation.rs:71-79)."""
        return self.moment_sum.copy()

    @property
    def circulation_strength(self) -> np.ndarray:
        return self.force_input.circulation_strength


class OutputBuffers:
    """Host arrays bound to an sb_step_output struct for one model size."""

    def __init__(self, n: int, s: int):
        self.n, self.s = n, s
        self.circulation = np.zeros(n)
        self.ctrl_velocity = np.zeros((n, 3))
        self.solver_input = np.zeros((n, 3))
        self.aoa = np.zeros(n)
        self.force_velocity = np.zeros((n, 3))
        self.acceleration = np.zeros((n, 3))
        self.ctrl_points = np.zeros((n, 3))
        self.sectional = np.zeros((6, n, 3))
        self.int_forces = np.zeros((s, 6, 3))
        self.int_moments = np.zeros((s, 6, 3))
        self.struct = StepOutput()
        st = self.struct
        st.circulation_strength = as_ptr(self.circulation)
        st.ctrl_points_velocity = as_ptr(self.ctrl_velocity)
        st.solver_input_velocity = as_ptr(self.solver_input)
        st.angles_of_attack = as_ptr(self.aoa)
        st.force_input_velocity = as_ptr(self.force_velocity)
        st.acceleration = as_ptr(self.acceleration)
        st.ctrl_points = as_ptr(self.ctrl_points)
        st.sectional_forces = as_ptr(self.sectional)
        st.integrated_forces = as_ptr(self.int_forces)
        st.integrated_moments = as_ptr(self.int_moments)

    def to_result(self, time: float) -> SimulationResult:
        st = self.struct
        sec = SectionalForces(*[self.sectional[c].copy() for c in range(6)])
        fi = SectionalForcesInput(self.circulation.copy(), self.force_velocity.copy(), self.aoa.copy(),
                                  self.acceleration.copy())
        ints = [IntegratedValues(*[self.int_forces[w, c].copy() for c in range(6)]) for w in range(self.s)]
        intm = [IntegratedValues(*[self.int_moments[w, c].copy() for c in range(6)]) for w in range(self.s)]
        return SimulationResult(
            time=time,
            ctrl_points=self.ctrl_points.copy(),
            solver_input_ctrl_points_velocity=self.solver_input.copy(),
            output_ctrl_points_velocity=self.ctrl_velocity.copy(),
            force_input=fi,
            sectional_forces=sec,
            integrated_forces=ints,
            integrated_moments=intm,
            iterations=int(st.iterations),
            residual=float(st.residual),
            converged=bool(st.converged),
            force_sum=np.array(st.force_sum[:]),
            moment_sum=np.array(st.moment_sum[:]),
        )


def vec3_array(a, n: int | None = None, name: str = "array") -> np.ndarray:
    """Converts a list of [x, y, z] (or an (n, 3) array) to a C-contiguous float64 (n, 3) array."""
    arr = np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1, 3))
    if n is not None and arr.shape[0] != n:
        raise SbError(SB_ERR_SIZE, f"{name} has {arr.shape[0]} points, expected {n}")
    return arr
