"""CompleteSailModel on the GPU (sb_csm_*) against the oracle's restatement.

  * steady-state conditions (controller + GPU wind freestream + one Linearized step) match
    the oracle per sail (force and moment, relative 1e-9: the Linearized test's tolerance)
    and leave the same wing angles (1e-12);
  * a sweep of conditions (one batch of replicas: one measurement pass, one batched solve)
    gives what the same conditions give one call at a time on fresh models (bit-identical:
    the same kernels and host controller) and what the oracle gives;
  * the optimal-loading search picks the loading of the best effective power of its sweep;
  * effective-angle set points with a rate limit, over consecutive calls (the controller
    reads the current wing angles), match the oracle call by call;
  * errors: malformed setup, more set points than sails, zero-length output.
"""
import math

import numpy as np
import pytest

from stormbird_gb300 import setups as S

pytestmark = pytest.mark.gpu

SAILS, PANELS = 3, 16
CONDS = [(9.0, 60.0, 0.0, 0.7), (12.0, -120.0, 6.0, 1.0), (7.0, 100.0, 3.0, 0.4), (15.0, 35.0, 8.0, 0.9)]


def _rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def test_steady_state_matches_oracle(gpu_lib, oracle_mod):
    from stormbird_gb300 import CompleteSailModel

    js = S.complete_sail_model(SAILS, PANELS)
    for v, d_deg, ship, loading in CONDS:
        g = CompleteSailModel(js)
        o = oracle_mod.OracleCompleteSailModel(js, SAILS)
        d = math.radians(d_deg)
        rg = g.simulate_steady_state_condition(wind_velocity=v, wind_direction=d, ship_velocity=ship,
                                               controller_loading=loading)
        ro = o.simulate_steady_state_condition(v, d, ship, loading)
        assert rg.shape == (SAILS, 7)
        assert _rel(rg[:, :3], ro[:, :3]) <= 1e-9 and _rel(rg[:, 3:6], ro[:, 3:6]) <= 1e-9, (v, d_deg)
        assert np.all(rg[:, 6] == 0.0)
        assert np.max(np.abs(g.local_wing_angles() - o.local_wing_angles())) <= 1e-12
        g.close()


def test_sweep_equals_single_calls_and_oracle(gpu_lib, oracle_mod):
    from stormbird_gb300 import CompleteSailModel

    js = S.complete_sail_model(SAILS, PANELS)
    v = [c[0] for c in CONDS]
    d = [math.radians(c[1]) for c in CONDS]
    ship = [c[2] for c in CONDS]
    loading = [c[3] for c in CONDS]
    m = CompleteSailModel(js)
    for _ in range(2):  # the second sweep reuses the replicas
        sw = m.sweep_steady_state(v, d, ship, loading)
        assert sw.shape == (len(CONDS), SAILS, 7)
        for i in range(len(CONDS)):
            single = CompleteSailModel(js)
            r = single.simulate_steady_state_condition(wind_velocity=v[i], wind_direction=d[i], ship_velocity=ship[i],
                                                       controller_loading=loading[i])
            single.close()
            assert np.array_equal(sw[i], r), i
            ro = oracle_mod.OracleCompleteSailModel(js, SAILS).simulate_steady_state_condition(v[i], d[i], ship[i],
                                                                                                loading[i])
            assert _rel(sw[i, :, :6], ro[:, :6]) <= 1e-9, i
    # the model itself is untouched by sweeps
    assert np.all(m.local_wing_angles() == 0.0)


def test_optimal_controller_loading(gpu_lib):
    from stormbird_gb300 import CompleteSailModel

    js = S.complete_sail_model(SAILS, PANELS)
    m = CompleteSailModel(js)
    n, v, d, ship = 7, 10.0, math.radians(95.0), 5.0
    best, loading = m.simulate_condition_optimal_controller_loading(wind_velocity=v, wind_direction=d,
                                                                    ship_velocity=ship, nr_loadings_to_test=n)
    loadings, x = [], 0.1  # linspace by accumulated steps (stormath/src/array_generation.rs:16-30)
    for _ in range(n):
        loadings.append(x)
        x += (1.0 - 0.1) / (n - 1)
    sw = m.sweep_steady_state([v] * n, [d] * n, [ship] * n, loadings)
    eff = [-sw[k, :, 0].sum() * ship - sw[k, :, 6].sum() for k in range(n)]
    k = int(np.argmax(eff))
    assert abs(loading - loadings[k]) < 1e-12
    assert np.array_equal(best, sw[k])


def test_effective_set_points_over_consecutive_calls(gpu_lib, oracle_mod):
    from stormbird_gb300 import CompleteSailModel

    sp = S.wing_sail_set_points(use_effective_angle_of_attack=True, max_local_wing_angle_change_rate=0.08)
    js = S.complete_sail_model(SAILS, PANELS, set_points=[sp] * SAILS,
                               flow_measurement={"angle_of_attack": {"measurement_type": "Max", "start_index": 1}})
    g = CompleteSailModel(js)
    o = oracle_mod.OracleCompleteSailModel(js, SAILS)
    start = np.array([0.4, -0.1, 0.2])
    g.set_local_wing_angles(start)
    o.set_local_wing_angles(start)
    for k in range(4):
        d = math.radians(70.0 + 10.0 * k)
        rg = g.simulate_steady_state_condition(wind_velocity=10.0, wind_direction=d, ship_velocity=4.0,
                                               controller_loading=0.8)
        ro = o.simulate_steady_state_condition(10.0, d, 4.0, 0.8)
        assert np.max(np.abs(g.local_wing_angles() - o.local_wing_angles())) <= 1e-12, k
        assert _rel(rg[:, :6], ro[:, :6]) <= 1e-9, k


def test_errors(gpu_lib):
    from stormbird_gb300 import CompleteSailModel, SbError

    with pytest.raises(SbError) as e:
        CompleteSailModel("{not json")
    assert e.value.code == -3
    with pytest.raises(SbError) as e:
        CompleteSailModel(S.complete_sail_model(2, 8, set_points=[S.wing_sail_set_points()] * 3))
    assert e.value.code == -2 and "set points" in str(e.value)
    from stormbird_gb300._abi import SingleSailResultC, WindConditionC

    m = CompleteSailModel(S.complete_sail_model(2, 8))
    res = (SingleSailResultC * 2)()
    assert gpu_lib.sb_csm_simulate_steady_state_condition(m._h, WindConditionC(8.0, 1.0), 0.0, 1.0, res, 0) == -2
    assert gpu_lib.sb_csm_simulate_steady_state_condition(m._h, WindConditionC(8.0, 1.0), 0.0, 1.0, res, 1) == 1
    assert gpu_lib.sb_csm_get_number_of_sails(None) == -1
