"""Loader for the CUDA C-ABI library (stormbird_gb300/_build/libstormbird_gb300.so).

There is no CPU fallback: when the library is missing or cannot be loaded, `lib()`
raises, naming the build step (`python -m stormbird_gb300.build` or
`__graft_entry__.build()`).
"""
from __future__ import annotations

import ctypes
import os

from ._abi import SingleSailResultC, StepOutput, WindConditionC

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libstormbird_gb300.so")

# Every entry point of include/stormbird_gb300.h: (name, restype, argtypes)
_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_szp = ctypes.POINTER(ctypes.c_size_t)
_vp = ctypes.c_void_p
SIGNATURES = [
    ("sb_last_error", ctypes.c_char_p, []),
    ("sb_last_status", ctypes.c_int, []),
    ("sb_version", ctypes.c_char_p, []),
    ("sb_sim_new", _vp, [ctypes.c_char_p, ctypes.c_int]),
    ("sb_sim_free", None, [_vp]),
    ("sb_sim_sizes", ctypes.c_int, [_vp, _szp, _szp, _szp]),
    ("sb_sim_get_freestream_points", ctypes.c_int, [_vp, _dp, ctypes.c_size_t]),
    ("sb_sim_do_step", ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_double, _dp, ctypes.c_size_t,
                                      ctypes.POINTER(StepOutput)]),
    ("sb_sim_do_step_device", ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_double, _vp, ctypes.c_size_t]),
    ("sb_sim_read_output", ctypes.c_int, [_vp, ctypes.POINTER(StepOutput)]),
    ("sb_sim_induced_velocities", ctypes.c_int, [_vp, _dp, ctypes.c_size_t, _dp]),
    ("sb_sim_set_translation_and_rotation_with_finite_difference", ctypes.c_int, [_vp, ctypes.c_double, _dp, _dp]),
    ("sb_sim_set_translation_only", ctypes.c_int, [_vp, _dp]),
    ("sb_sim_set_rotation_only", ctypes.c_int, [_vp, _dp]),
    ("sb_sim_set_velocity_linear", ctypes.c_int, [_vp, _dp]),
    ("sb_sim_set_velocity_angular", ctypes.c_int, [_vp, _dp]),
    ("sb_sim_set_local_wing_angles", ctypes.c_int, [_vp, _dp, ctypes.c_size_t]),
    ("sb_sim_get_local_wing_angles", ctypes.c_int, [_vp, _dp, ctypes.c_size_t]),
    ("sb_sim_reset_previous_circulation", ctypes.c_int, [_vp]),
    ("sb_sim_set_previous_circulation", ctypes.c_int, [_vp, _dp, ctypes.c_size_t]),
    ("sb_sim_get_previous_circulation", ctypes.c_int, [_vp, _dp, ctypes.c_size_t]),
    ("sb_sim_wake_sizes", ctypes.c_int, [_vp, _szp, _szp, _szp, _szp]),
    ("sb_sim_get_wake_state", ctypes.c_int, [_vp, _dp, _dp, _dp]),
    ("sb_sim_state_size", ctypes.c_int, [_vp, _szp]),
    ("sb_sim_get_state", ctypes.c_int, [_vp, _dp, ctypes.c_size_t]),
    ("sb_sim_set_state", ctypes.c_int, [_vp, _dp, ctypes.c_size_t]),
    ("sb_sim_set_precision", ctypes.c_int, [_vp, ctypes.c_int]),
    ("sb_sim_enable_timing", ctypes.c_int, [_vp, ctypes.c_int]),
    ("sb_sim_last_step_timing", ctypes.c_int, [_vp, _dp, ctypes.c_size_t]),
    ("sb_sim_last_step_counters", ctypes.c_int, [_vp, _dp, ctypes.c_size_t]),
    ("sb_sim_set_segment_sharing", ctypes.c_int, [_vp, ctypes.c_int]),
    ("sb_sim_set_wind", ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_char_p]),
    ("sb_sim_wind_freestream", ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_double, _dp, ctypes.c_size_t]),
    ("sb_sim_do_step_wind", ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                           ctypes.POINTER(StepOutput)]),
    ("sb_sim_segment_sharing_active", ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int)]),
    ("sb_panel_sweep", ctypes.c_int, [ctypes.c_int, _dp, _dp, _dp, ctypes.c_size_t, ctypes.c_double, ctypes.c_int,
                                      _dp, ctypes.c_size_t, ctypes.c_int, _dp]),
    ("sb_panel_sweep_no_alloc", ctypes.c_int, [ctypes.c_int, _vp, _vp, _vp, ctypes.c_size_t, ctypes.c_double,
                                               ctypes.c_int, _vp, ctypes.c_size_t, _vp, _vp]),
    ("sb_measure_fp32_peak", ctypes.c_int, [ctypes.c_int, ctypes.c_int, _dp]),
    ("sb_measure_fp64_peak", ctypes.c_int, [ctypes.c_int, ctypes.c_int, _dp]),
    ("sb_set_sweep_wait_polls", ctypes.c_int, [ctypes.c_int]),
    ("sb_wait_timeout_self_test", ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
    ("sb_batch_new", _vp, [ctypes.POINTER(ctypes.c_char_p), ctypes.c_size_t, ctypes.c_int]),
    ("sb_batch_free", None, [_vp]),
    ("sb_batch_sizes", ctypes.c_int, [_vp, _szp, _szp, _szp]),
    ("sb_batch_case_sizes", ctypes.c_int, [_vp, ctypes.c_size_t, _szp, _szp, _szp, _szp, _szp]),
    ("sb_batch_get_freestream_points", ctypes.c_int, [_vp, _dp, ctypes.c_size_t]),
    ("sb_batch_do_step", ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_double, _dp, ctypes.c_size_t]),
    ("sb_batch_do_step_device", ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_double, _vp, ctypes.c_size_t]),
    ("sb_batch_set_wind", ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.POINTER(ctypes.c_char_p)]),
    ("sb_batch_do_step_wind", ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_double, _dp]),
    ("sb_batch_get_circulation", ctypes.c_int, [_vp, _dp, ctypes.c_size_t]),
    ("sb_batch_get_summary", ctypes.c_int, [_vp, _dp, ctypes.c_size_t]),
    ("sb_batch_read_case_output", ctypes.c_int, [_vp, ctypes.c_size_t, ctypes.POINTER(StepOutput)]),
    ("sb_batch_case_state_size", ctypes.c_int, [_vp, ctypes.c_size_t, _szp]),
    ("sb_batch_get_case_state", ctypes.c_int, [_vp, ctypes.c_size_t, _dp, ctypes.c_size_t]),
    ("sb_batch_set_case_state", ctypes.c_int, [_vp, ctypes.c_size_t, _dp, ctypes.c_size_t]),
    ("sb_batch_set_initial_circulation", ctypes.c_int, [_vp, _dp, ctypes.c_size_t]),
    ("sb_batch_set_initial_circulation_device", ctypes.c_int, [_vp, _vp, ctypes.c_size_t]),
    ("sb_batch_previous_circulation_device", ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_void_p)]),
    ("sb_batch_set_precision", ctypes.c_int, [_vp, ctypes.c_int]),
    ("sb_batch_use_graph", ctypes.c_int, [_vp, ctypes.c_int]),
    ("sb_batch_autotune", ctypes.c_int, [_vp, ctypes.c_double]),
    ("sb_batch_info", ctypes.c_int, [_vp, _dp, ctypes.c_size_t]),
    ("sb_mlp_new", _vp, [ctypes.c_int, ctypes.c_int, ctypes.c_ulonglong]),
    ("sb_mlp_free", None, [_vp]),
    ("sb_mlp_num_params", ctypes.c_int, [_vp, _szp]),
    ("sb_mlp_get_params", ctypes.c_int, [_vp, _fp, ctypes.c_size_t]),
    ("sb_mlp_set_params", ctypes.c_int, [_vp, _fp, ctypes.c_size_t]),
    ("sb_mlp_forward", ctypes.c_int, [_vp, _vp, ctypes.c_size_t, _vp]),
    ("sb_mlp_gradients", ctypes.c_int, [_vp, _vp, _vp, ctypes.c_size_t, _fp, _dp]),
    ("sb_mlp_train_step", ctypes.c_int, [_vp, _vp, _vp, ctypes.c_size_t, ctypes.c_float, _dp]),
    ("sb_batch_set_warm_start", ctypes.c_int, [_vp, _vp, ctypes.c_int]),
    ("sb_batch_set_warm_start_guard", ctypes.c_int, [_vp, ctypes.c_double]),
    ("sb_batch_copy_warm_start_data", ctypes.c_int, [_vp, _vp, _vp, ctypes.c_size_t]),
    ("sb_sim_result_json", ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_size_t, _szp]),
    ("sb_sim_result_csv", ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_size_t]),
    ("sb_sim_set_result_file", ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_int]),
    ("sb_sim_flush_results", ctypes.c_int, [_vp]),
    ("sb_csm_new", _vp, [ctypes.c_char_p, ctypes.c_int]),
    ("sb_csm_free", None, [_vp]),
    ("sb_csm_get_number_of_sails", ctypes.c_int, [_vp]),
    ("sb_csm_simulate_steady_state_condition", ctypes.c_int, [_vp, WindConditionC, ctypes.c_double, ctypes.c_double,
                                                              ctypes.POINTER(SingleSailResultC), ctypes.c_size_t]),
    ("sb_csm_apply_controller", ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_double, ctypes.c_char_p,
                                               ctypes.c_double, ctypes.c_double]),
    ("sb_csm_do_step", ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_double, ctypes.c_char_p, ctypes.c_double,
                                      ctypes.POINTER(StepOutput)]),
    ("sb_csm_sim", ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_void_p)]),
    ("sb_csm_sweep_steady_state", ctypes.c_int, [_vp, ctypes.POINTER(WindConditionC), _dp, _dp, ctypes.c_size_t,
                                                 ctypes.POINTER(SingleSailResultC), ctypes.c_size_t]),
    ("sb_csm_simulate_condition_optimal_controller_loading", ctypes.c_int,
     [_vp, WindConditionC, ctypes.c_double, ctypes.c_size_t, ctypes.POINTER(SingleSailResultC), ctypes.c_size_t,
      _dp]),
]

_LIB = None


def lib() -> ctypes.CDLL:
    """The loaded CUDA library; raises if it was not built."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"CUDA library {LIB_PATH} is missing: build it with `python -m stormbird_gb300.build` "
                "(there is no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB
