"""Freestream generated on the GPU from the reference's wind model (sb_sim_set_wind,
sb_sim_wind_freestream, sb_sim_do_step_wind) against the oracle's restatement of
CompleteSailModel::freestream_velocity (complete_sail_model/mod.rs:213-257):
  * at every freestream point of a fresh simulation, with power-law / logarithmic / constant
    profiles, three gust spectra, ship velocity and inflow corrections: relative 1e-12;
  * after wind-driven steps, at the GPU's own (moved) wake points: relative 1e-12;
  * do_step_wind equals do_step with the same freestream (bit-identical), and a wind-driven
    dynamic run matches the oracle run at a fixed iteration count (1e-5);
  * error codes for bad JSON, too few correction ranges and a missing wind model.
"""
import numpy as np
import pytest

from stormbird_gb300 import setups as S
from tests import wind_cases as W
from tests.helpers import fixed_iterations, rel_inf, rel_vec

pytestmark = pytest.mark.gpu

DT = 0.05


def _setup():
    return fixed_iterations(S.wing_sail_row(2, 6, 10, far_field_ratio=5.0), 15)


@pytest.mark.parametrize("profile", ["power", "log", "log_stable", "constant"])
@pytest.mark.parametrize("corrections", [False, True])
def test_wind_freestream_matches_oracle(gpu_lib, oracle_mod, profile, corrections):
    from stormbird_gb300 import Simulation

    js = _setup()
    env, cond = W.environment(inflow_corrections=corrections, water_plane_height=-2.0), W.condition(70.0, profile)
    g = Simulation(js)
    g.set_wind(env, cond)
    o = oracle_mod.OracleSimulation(js)
    for t, ship in ((0.0, 0.0), (1.3, 3.0), (7.9, -2.5)):
        ug = g.wind_freestream(time=t, ship_velocity=ship)
        uo = o.wind_freestream(env, cond, t, ship)
        assert rel_inf(ug, uo) <= 1e-12, (t, ship)


def test_wind_freestream_at_moved_wake_points(gpu_lib, oracle_mod):
    from stormbird_gb300 import Simulation

    env, cond = W.environment(), W.condition(120.0, "log")
    g = Simulation(_setup())
    g.set_wind(env, cond)
    for k in range(6):
        g.do_step_wind(time=k * DT, time_step=DT, ship_velocity=2.0)
    t = 6 * DT
    ug = g.wind_freestream(time=t, ship_velocity=2.0)
    pts = g.get_freestream_velocity_points()
    uo = oracle_mod.wind_velocity_at(env, cond, pts, time=t, ship_velocity=2.0)
    assert rel_inf(ug, uo) <= 1e-12


def test_do_step_wind_equals_do_step(gpu_lib):
    from stormbird_gb300 import Simulation

    env, cond = W.environment(inflow_corrections=True), W.condition(40.0, "power")
    a, b = Simulation(_setup()), Simulation(_setup())
    a.set_wind(env, cond)
    b.set_wind(env, cond)
    for k in range(8):
        ra = a.do_step_wind(time=k * DT, time_step=DT, ship_velocity=1.5)
        fs = b.wind_freestream(time=k * DT, ship_velocity=1.5)
        rb = b.do_step(time=k * DT, time_step=DT, freestream_velocity=fs)
        assert np.array_equal(ra.circulation_strength, rb.circulation_strength), k
        assert np.array_equal(ra.integrated_forces_sum(), rb.integrated_forces_sum()), k


def test_wind_driven_run_matches_oracle(gpu_lib, oracle_mod):
    from stormbird_gb300 import Simulation

    js = _setup()
    env, cond = W.environment(inflow_corrections=True), W.condition(55.0, "power")
    g = Simulation(js)
    g.set_wind(env, cond)
    o = oracle_mod.OracleSimulation(js)
    for k in range(9):
        rg = g.do_step_wind(time=k * DT, time_step=DT, ship_velocity=3.0)
        ro = o.do_step(time=k * DT, time_step=DT, freestream_velocity=o.wind_freestream(env, cond, k * DT, 3.0))
        assert rel_inf(rg.circulation_strength, ro.circulation_strength) <= 1e-5, k
        assert rel_vec(rg.integrated_forces_sum(), ro.integrated_forces_sum()) <= 1e-5, k


def test_wind_errors(gpu_lib):
    from stormbird_gb300 import SbError, Simulation

    g = Simulation(_setup())
    with pytest.raises(SbError) as e:
        g.do_step_wind(time=0.0, time_step=DT, ship_velocity=0.0)
    assert e.value.code == -8
    with pytest.raises(SbError) as e:
        g.set_wind('{"bad_field": 1}', W.condition())
    assert e.value.code == -3
    with pytest.raises(SbError) as e:
        g.set_wind(W.environment(inflow_corrections=True, nr_wings=1), W.condition())
    assert e.value.code == -2


def test_batched_wind_sweep_matches_single_cases(gpu_lib):
    """A wind-direction sweep as one batch (CompleteSailModel over conditions) equals the
    same cases stepped one by one with do_step_wind; graphs are replayed after step 3."""
    from stormbird_gb300 import Batch, Simulation

    js = _setup()
    env = W.environment(inflow_corrections=True)
    conds = [W.condition(d, p) for d, p in ((20.0, "power"), (75.0, "log"), (140.0, "constant"), (-60.0, "power"))]
    ships = [0.0, 2.0, 4.0, 6.0]
    b = Batch([js] * len(conds))
    b.set_wind(env, conds)
    sims = [Simulation(js) for _ in conds]
    for s, c in zip(sims, conds):
        s.set_wind(env, c)
    for k in range(10):
        b.do_step_wind(time=k * DT, time_step=DT, ship_velocities=ships)
        g = b.circulation()
        for i, s in enumerate(sims):
            r = s.do_step_wind(time=k * DT, time_step=DT, ship_velocity=ships[i])
            assert rel_inf(g[b.case_slice(i)], r.circulation_strength) <= 2e-6, (k, i)
    assert b.info()["graph"] == 1.0
