"""The oracle's state between steps (CPU): a state copied into a second oracle simulation of
the same setup continues bit-identically, and leaving one step's roll-up out (the harness
option the full-size parity tests use) changes none of that step's outputs."""
import numpy as np

from stormbird_gb300 import setups as S

DT = 0.05


def _run(sim, wind, k0, k1):
    n = sim.nr_freestream_points
    out = []
    for k in range(k0, k1):
        r = sim.do_step(time=k * DT, time_step=DT, freestream_velocity=wind.freestream(k * DT, n))
        out.append((r.circulation_strength.copy(), r.integrated_forces_sum().copy(), r.iterations))
    return out


def test_oracle_state_round_trip(oracle_mod):
    setup = S.wing_sail_row(2, 6, 12, time_step=DT)
    wind = S.GustyWind(seed=2)
    a = oracle_mod.OracleSimulation(setup, nthreads=2)
    _run(a, wind, 0, 8)
    st = a.state()
    assert st[0] == 8 and st[1] == 1 and st[2] == 8
    b = oracle_mod.OracleSimulation(setup, nthreads=2)
    b.set_state(st)
    assert np.array_equal(b.state(), st)
    for (ga, fa, ia), (gb, fb, ib) in zip(_run(a, wind, 8, 12), _run(b, wind, 8, 12)):
        assert np.array_equal(ga, gb) and np.array_equal(fa, fb) and ia == ib


def test_skipping_the_rollup_leaves_the_step_outputs_unchanged(oracle_mod):
    setup = S.wing_sail_row(2, 6, 12, time_step=DT)
    wind = S.GustyWind(seed=3)
    a = oracle_mod.OracleSimulation(setup, nthreads=2)
    _run(a, wind, 0, 7)
    b = oracle_mod.OracleSimulation(setup, nthreads=2)
    b.set_state(a.state())
    b.skip_next_rollup()
    (ga, fa, _), = _run(a, wind, 7, 8)
    (gb, fb, _), = _run(b, wind, 7, 8)
    assert np.array_equal(ga, gb) and np.array_equal(fa, fb)
    # the velocity at the wake points is the freestream alone after the skipped roll-up
    _, _, va = a.wake_state()
    _, _, vb = b.wake_state()
    fs = wind.freestream(7 * DT, 1)[0]
    assert np.allclose(vb, fs, rtol=0, atol=0) and not np.allclose(va, fs)
