"""Batched cases (sb_batch_*): every case of a batch computes what its own Simulation would.

Checked through the C ABI on seeded uneven cases (sail count, panels per sail, wake length,
apparent wind angle and speed drawn per case):
  * against the same cases run one by one with sb_sim (the plain path), step by step, at a
    fixed iteration count: circulation and force sums within the FP32 sweep tolerance
    (the two paths cut the sweeps into different chunks, so sums differ in rounding);
  * against the f64 oracle for a subset of cases (relative circulation and force <= 1e-5);
  * CUDA-graph replay against eager launches of the same batch: bit-identical (the same
    kernels, work lists and chunk-ordered reductions);
  * after autotuning, every step within 1e-5 of the oracle's step from the same state, and
    within the FP32 tolerance of the single-case path;
  * the warm-start hook, size checks and the error that names a bad case;
  * quasi-steady cases in a batch (bit-identical to their own Simulations).
"""
import json

import numpy as np
import pytest

from stormbird_gb300 import setups as S
from tests.helpers import fixed_iterations, rel_inf, rel_vec

pytestmark = pytest.mark.gpu

DT = 0.05
TOL_GPU = 2e-6   # batch vs single-case GPU path (FP32 sweeps, different chunking)
TOL_ORACLE = 1e-5


def _small_cases(n, seed, iterations=12):
    cases = S.uneven_cases(n, seed, sails=(1, 3), panels=(3, 10), wake_rows=(5, 16), wind_speed=(6.0, 14.0))
    return [(fixed_iterations(js, iterations), w) for js, w in cases]


def _single_runs(cases, steps):
    from stormbird_gb300 import Simulation

    res = []
    for js, w in cases:
        sim = Simulation(js)
        g, f = [], []
        for k in range(steps):
            r = sim.do_step(time=k * DT, time_step=DT, freestream_velocity=w.freestream(k * DT, sim.nr_freestream_points))
            g.append(r.force_input.circulation_strength.copy())
            f.append(r.integrated_forces_sum().copy())
        sim.close()
        res.append((g, f))
    return res


def _batch_run(batch, winds, steps):
    g, s = [], []
    for k in range(steps):
        batch.do_step(time=k * DT, time_step=DT, freestream_velocity=S.batch_freestream(batch, winds, k * DT))
        g.append(batch.circulation())
        s.append(batch.summary())
    return g, s


def test_batch_matches_single_case_path(gpu_lib):
    from stormbird_gb300 import Batch

    cases = _small_cases(6, seed=11)
    steps = 12  # graphs are captured at steps 4 and 5 and replayed after
    single = _single_runs(cases, steps)
    b = Batch([js for js, _ in cases])
    g, s = _batch_run(b, [w for _, w in cases], steps)
    assert b.info()["graph"] == 1.0
    for i in range(len(cases)):
        sl = b.case_slice(i)
        for k in range(steps):
            eg = rel_inf(g[k][sl], single[i][0][k])
            ef = rel_vec(s[k][i, :3], single[i][1][k])
            assert eg <= TOL_GPU and ef <= TOL_GPU, f"case {i} step {k}: circulation {eg:.3e} force {ef:.3e}"
        assert s[-1][i, 9] == 0.0 and s[-1][i, 7] == 12.0


def test_batch_matches_oracle(gpu_lib, oracle_mod):
    from stormbird_gb300 import Batch

    cases = _small_cases(3, seed=5, iterations=15)
    steps = 9
    b = Batch([js for js, _ in cases])
    g, s = _batch_run(b, [w for _, w in cases], steps)
    for i, (js, w) in enumerate(cases):
        o = oracle_mod.OracleSimulation(js)
        for k in range(steps):
            r = o.do_step(time=k * DT, time_step=DT, freestream_velocity=w.freestream(k * DT, o.nr_freestream_points))
            eg = rel_inf(g[k][b.case_slice(i)], r.force_input.circulation_strength)
            ef = rel_vec(s[k][i, :3], r.integrated_forces_sum())
            assert eg <= TOL_ORACLE and ef <= TOL_ORACLE, f"case {i} step {k}: {eg:.3e} {ef:.3e}"


def test_graph_replay_is_bit_identical_to_eager(gpu_lib):
    from stormbird_gb300 import Batch

    cases = _small_cases(5, seed=3)
    winds = [w for _, w in cases]
    a = Batch([js for js, _ in cases])
    b = Batch([js for js, _ in cases])
    b.use_graph(False)
    ga, sa = _batch_run(a, winds, 10)
    gb, sb = _batch_run(b, winds, 10)
    assert a.info()["graph"] == 1.0 and b.info()["graph"] == 0.0
    for k in range(10):
        assert np.array_equal(ga[k], gb[k]), f"step {k}"
        assert np.array_equal(sa[k], sb[k]), f"step {k}"


def test_autotuned_batch_stays_within_tolerance(gpu_lib, oracle_mod):
    """Autotuning changes the tile shape (panels summed in FP32 before the compensated fold)
    and the chunking. Every step of the tuned batch against the oracle's step from the batch's
    own state before it (a per-step error; from a cold start two trajectories of unconverged
    fixed-iteration solves drift apart over steps whatever the arithmetic), and the first
    tuned step against the untuned single-case path from the same state."""
    from stormbird_gb300 import Batch, Simulation

    cases = _small_cases(6, seed=17)
    winds = [w for _, w in cases]
    b = Batch([js for js, _ in cases])
    _batch_run(b, winds, 5)
    b.autotune(budget_seconds=2.0)
    info = b.info()
    assert info["tuned"] == 1.0 and info["tune_candidates"] >= 1
    for k in range(5, 10):
        states = [b.case_state(i) for i in range(len(cases))]
        b.do_step(time=k * DT, time_step=DT, freestream_velocity=S.batch_freestream(b, winds, k * DT))
        g = b.circulation()
        for i, (js, w) in enumerate(cases):
            o = oracle_mod.OracleSimulation(js)
            o.set_state(states[i])
            r = o.do_step(time=k * DT, time_step=DT, freestream_velocity=w.freestream(k * DT, o.nr_freestream_points))
            e = rel_inf(g[b.case_slice(i)], r.force_input.circulation_strength)
            assert e <= TOL_ORACLE, f"case {i} step {k}: {e:.2e}"
            if k == 5:
                sim = Simulation(js)
                sim.set_state(states[i])
                rs = sim.do_step(time=k * DT, time_step=DT, freestream_velocity=w.freestream(k * DT, sim.nr_freestream_points))
                es = rel_inf(g[b.case_slice(i)], rs.force_input.circulation_strength)
                assert es <= TOL_GPU, f"case {i}: tuned batch vs single-case path {es:.2e}"
                sim.close()


def test_warm_start_hook_cuts_iterations(gpu_lib):
    from stormbird_gb300 import Batch

    js, w = S.uneven_cases(1, 2, sails=(2, 2), panels=(8, 8), wake_rows=(10, 10), wind_speed=(10.0, 10.0))[0]
    d = json.loads(js)
    si = d["simulation_settings"]["Dynamic"]["solver"]["SimpleIterative"]
    si["max_iterations_per_time_step"] = 400
    si["residual_tolerance_absolute"] = 1e-7
    js = json.dumps(d)
    a, b = Batch([js]), Batch([js])
    # the first step zeroes the previous circulation (Simulation::initialize,
    # simulation.rs:65-94), so the hook acts from the second step on
    for x in (a, b):
        x.do_step(time=0.0, time_step=DT, freestream_velocity=S.batch_freestream(x, [w], 0.0))
    fs = S.batch_freestream(a, [w], DT)
    a.do_step(time=DT, time_step=DT, freestream_velocity=fs)
    plain = a.summary()[0, 7]
    b.set_initial_circulation(a.circulation())
    b.do_step(time=DT, time_step=DT, freestream_velocity=fs)
    warm = b.summary()[0, 7]
    assert warm < plain
    assert rel_inf(b.circulation(), a.circulation()) <= 1e-5


def test_batch_errors(gpu_lib):
    from stormbird_gb300 import Batch, SbError

    cases = _small_cases(2, seed=1)
    with pytest.raises(SbError) as e:
        Batch([cases[0][0], "{not json"])
    assert e.value.code == -3 and "case 1" in str(e.value)
    b = Batch([js for js, _ in cases])
    long_fs = np.zeros((b.total_freestream + 1, 3))
    rc = gpu_lib.sb_batch_do_step(b._h, 0.0, DT, long_fs.ctypes.data_as(gpu_lib.sb_batch_do_step.argtypes[3]),
                                  b.total_freestream + 1)
    assert rc == -2 and "expected" in gpu_lib.sb_last_error().decode()
    bad = S.batch_freestream(b, [w for _, w in cases], 0.0)
    bad[3, 1] = np.nan
    with pytest.raises(SbError) as e:
        b.do_step(time=0.0, time_step=DT, freestream_velocity=bad)
    assert e.value.code == -5


def test_quasi_steady_cases_in_a_batch(gpu_lib):
    """Quasi-steady cases (Linearized, the quasi-steady default, and SimpleIterative) in one
    batch give what their own Simulations give: the same kernels on the same inputs."""
    from stormbird_gb300 import Batch, Simulation

    js_si, u = S.quasi_steady_single_wing(24)
    d = json.loads(js_si)
    del d["simulation_settings"]["QuasiSteady"]["solver"]  # Linearized default
    js_lin = json.dumps(d)
    cases = [js_si, js_lin, js_lin]
    speeds = [1.0, 0.8, 1.3]
    b = Batch(cases)
    sims = [Simulation(js) for js in cases]
    for k in range(6):
        fs = np.concatenate([np.tile(u * sp, (c["freestream_points"], 1)) for sp, c in zip(speeds, b.cases)])
        b.do_step(time=k * DT, time_step=DT, freestream_velocity=fs)
        g, s = b.circulation(), b.summary()
        for i, (sim, sp) in enumerate(zip(sims, speeds)):
            r = sim.do_step(time=k * DT, time_step=DT, freestream_velocity=np.tile(u * sp, (sim.nr_freestream_points, 1)))
            assert np.array_equal(g[b.case_slice(i)], r.circulation_strength), (k, i)
            assert np.array_equal(s[i, :3], r.integrated_forces_sum()), (k, i)


def test_batched_linearized_quasi_steady_sweep(gpu_lib, oracle_mod):
    """An angle sweep of quasi-steady cases with the Linearized solver: the batch solves them
    in one launch (a CTA per case) and every case gives what its own Simulation gives
    (bit-identical: the same device function) and what the oracle gives (1e-9, the tolerance
    of the single-case Linearized test). Sizes 8 to 600 span lines: up to 164 the matrix sits
    in one CTA's shared memory; 180, 400 and 600 are spread over clusters of 2, 8 and 16 CTAs
    (one launch per cluster size)."""
    import math

    from stormbird_gb300 import Batch, Simulation

    sizes = [8, 24, 64, 180, 31, 100, 400, 600]
    cases, winds = [], []
    for k, n in enumerate(sizes):
        cases.append(S.simulation(S.rectangular_wing(5.0, 1.2, math.radians(2.0 + k), n), dynamic=False))
        a = math.radians(1.5 * k)
        winds.append(np.array([1.2 * math.cos(a), 1.2 * math.sin(a), 0.0]))
    b = Batch(cases)
    sims = [Simulation(js) for js in cases]
    oracles = [oracle_mod.OracleSimulation(js) for js in cases]
    for step in range(3):
        scale = 1.0 + 0.1 * step
        fs = np.concatenate([np.tile(w * scale, (c["freestream_points"], 1)) for w, c in zip(winds, b.cases)])
        b.do_step(time=0.2 * step, time_step=0.2, freestream_velocity=fs)
        g, s = b.circulation(), b.summary()
        for i, (sim, o, w) in enumerate(zip(sims, oracles, winds)):
            fi = np.tile(w * scale, (sim.nr_freestream_points, 1))
            r = sim.do_step(time=0.2 * step, time_step=0.2, freestream_velocity=fi)
            assert np.array_equal(g[b.case_slice(i)], r.circulation_strength), (step, i)
            assert np.array_equal(s[i, :3], r.integrated_forces_sum()), (step, i)
            ro = o.do_step(time=0.2 * step, time_step=0.2, freestream_velocity=fi)
            assert rel_inf(g[b.case_slice(i)], ro.circulation_strength) <= 1e-9, (step, i)
            assert rel_vec(s[i, :3], ro.integrated_forces_sum()) <= 1e-9, (step, i)
