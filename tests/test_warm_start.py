"""Warm-start network on the GPU (sb_mlp_*, tcgen05 BF16 GEMMs) and its use in a batch.

  * forward pass and mean-squared-error gradients through the C ABI against the f64
    restatement tests/mlp_ref.py with the GPU's BF16 roundings emulated (tolerances below:
    FP32 tensor-core accumulation against f64, plus rare BF16 rounding flips);
  * training with the library's Adam lowers the loss of a smooth regression;
  * a network trained on data the batch itself records warm-starts held-out cases: the
    results agree with the plain solves to within 1e-5 (solver tolerance 1e-7 residual), and
    the iteration counts of the plain start, the extrapolation alone and extrapolation plus
    network are reported (the gain the network brings over the method without it).
"""
import numpy as np
import pytest

from tests import mlp_ref as R

pytestmark = pytest.mark.gpu

TOL_Y = 5e-3      # relative infinity norm of the outputs
TOL_GRAD = 1e-2   # relative L2 norm per parameter block


def _net(seed=3):
    from stormbird_gb300.warm_start import WarmStartNet

    return WarmStartNet(16, seed=seed)


def test_forward_matches_reference(gpu_lib):
    torch = pytest.importorskip("torch")
    net = _net()
    p = net.get_params()
    rng = np.random.default_rng(1)
    x = rng.normal(size=(300, 16)).astype(np.float32)
    y = net.forward(torch.from_numpy(x).cuda()).cpu().numpy()
    yr, _, _ = R.forward(p.astype(np.float64), x.astype(np.float64), emulate=True)
    err = np.max(np.abs(y - yr)) / np.max(np.abs(yr))
    assert err <= TOL_Y, err


def test_gradients_match_reference(gpu_lib):
    torch = pytest.importorskip("torch")
    net = _net(seed=5)
    p = net.get_params().astype(np.float64)
    rng = np.random.default_rng(2)
    x = rng.normal(size=(1000, 16)).astype(np.float32)
    t = rng.normal(size=1000).astype(np.float32)
    g, loss = net.gradients(torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda())
    loss_r, g_r = R.loss_and_grad(p, x.astype(np.float64), t.astype(np.float64), emulate=True)
    assert abs(loss - loss_r) <= 1e-3 * loss_r
    for name, sl in R.blocks():
        a, b = g[sl].astype(np.float64), g_r[sl]
        err = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        assert err <= TOL_GRAD, (name, err)


def test_training_lowers_the_loss(gpu_lib):
    torch = pytest.importorskip("torch")
    net = _net(seed=7)
    rng = np.random.default_rng(3)
    x = rng.uniform(-1, 1, size=(16384, 16)).astype(np.float32)
    t = (np.sin(2 * x[:, 0]) + x[:, 1] * x[:, 2] - 0.5 * x[:, 3] ** 2).astype(np.float32)
    X, T = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    first = None
    for epoch in range(40):
        perm = torch.randperm(X.shape[0], device=X.device)
        for s0 in range(0, X.shape[0], 4096):
            idx = perm[s0:s0 + 4096]
            loss = net.train_step(X[idx].contiguous(), T[idx].contiguous(), 2e-3)
            if first is None:
                first = loss
    _, final = net.gradients(X, T)
    assert final < 0.05 * first, (first, final)


def test_training_reads_rows_after_the_callers_stream(gpu_lib):
    """A training step reads rows PyTorch has just gathered on its default stream: the call
    orders its own stream after that work, so stepping straight after the gather gives the
    same losses and parameters as synchronising first."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(9)
    X = torch.from_numpy(rng.normal(size=(262144, 16)).astype(np.float32)).cuda()
    T = torch.from_numpy(rng.normal(size=262144).astype(np.float32)).cuda()
    g = torch.Generator(device=X.device)
    runs = []
    for sync in (False, True):
        net = _net(seed=13)
        g.manual_seed(4)
        losses = []
        for _ in range(3):
            perm = torch.randperm(X.shape[0], device=X.device, generator=g)
            Xs, Ts = X[perm].contiguous(), T[perm].contiguous()  # gathered on PyTorch's stream
            if sync:
                torch.cuda.synchronize()
            losses.append(net.train_step(Xs[:8192], Ts[:8192], 1e-3))
            del Xs, Ts
        runs.append((losses, net.get_params()))
    assert runs[0][0] == runs[1][0]
    assert np.array_equal(runs[0][1], runs[1][1])


def test_warm_start_on_held_out_cases(gpu_lib):
    """The three starts on held-out cases: every arm ends within 1e-5 of the plain solves, the
    extrapolation in time saves iterations over the plain start, and the network arm is no
    worse than the extrapolation alone (the guard takes the network's start only when its
    residuals are half the extrapolation's). What the network gains over the extrapolation,
    as measured at full scale (config-4 network trained on 204,800 converged solves of the
    512 uneven cases, evaluated on those cases with every wake full): nothing. Its start was
    taken in 0 %, 0.23 % and 1.5 % of solves at guard factors 0.5, 0.8 and 1.0, and the
    iterations per solve were 88.21, 88.21 and 88.24 against 88.21 for the extrapolation
    alone and 97.03 for the plain start."""
    pytest.importorskip("torch")
    from stormbird_gb300 import setups as S
    from stormbird_gb300 import warm_start as WS

    def cases(n, seed):
        cs = S.uneven_cases(n, seed, sails=(1, 3), panels=(6, 16), wake_rows=(8, 24), wind_speed=(6.0, 14.0))
        return [(WS.tight_solver(js), w) for js, w in cs]

    X, T = WS.collect(cases(24, seed=100), steps=24)
    net = _net(seed=11)
    losses = WS.train(net, X, T, epochs=30, batch_rows=2048)
    assert losses[-1] < losses[0]
    rep = WS.evaluate(net, cases(6, seed=200), steps=16)
    print("warm start on held-out cases:", rep)
    for arm in ("extrapolation", "warm"):
        assert rep[f"max_rel_circulation_diff_{arm}"] <= 1e-5
        assert 0.0 <= rep[f"fallback_rate_{arm}"] <= 1.0
    assert rep["iterations_extrapolation"] < rep["iterations_plain"]
    assert rep["iterations_warm"] <= 1.02 * rep["iterations_extrapolation"]


def test_loaded_state_restarts_the_warm_start_history(gpu_lib):
    """A state loaded into a batch (sb_batch_set_case_state) carries no warm-start history:
    the first step after it has no trend and no freestream change in its features (both
    need the batch's own earlier steps; the freestream change compares |U| with itself, two
    f64 evaluations that may differ in the last bit), the second a freestream change but no
    trend, the third both, although the loaded case's step count is past two from the start.
    Stale history (the batch's own step 3) would give changes of the gust's size, ~1e-2."""
    torch = pytest.importorskip("torch")
    import ctypes

    from stormbird_gb300 import Batch
    from stormbird_gb300 import setups as S
    from stormbird_gb300.native import lib

    dt = 0.05
    cs = S.uneven_cases(2, 31, sails=(1, 2), panels=(6, 10), wake_rows=(12, 20), wind_speed=(8.0, 12.0))
    setups, winds = [js for js, _ in cs], [w for _, w in cs]
    src, dst = Batch(setups), Batch(setups)
    for k in range(16):
        src.do_step(time=k * dt, time_step=dt, freestream_velocity=S.batch_freestream(src, winds, k * dt))
    # dst records features from its own early steps, then takes src's later state
    dst.set_warm_start(None, 2)
    for k in range(4):
        dst.do_step(time=k * dt, time_step=dt, freestream_velocity=S.batch_freestream(dst, winds, k * dt))
    for i in range(len(setups)):
        dst.set_case_state(i, src.case_state(i))
    x = torch.empty((dst.total_lines, 16), dtype=torch.float32, device="cuda:0")
    for j, k in enumerate(range(16, 19)):
        dst.do_step(time=k * dt, time_step=dt, freestream_velocity=S.batch_freestream(dst, winds, k * dt))
        assert lib().sb_batch_copy_warm_start_data(dst._h, ctypes.c_void_p(x.data_ptr()), None, dst.total_lines) == 0
        f = x.cpu().numpy()
        trend, du = np.abs(f[:, 4]).max(), np.abs(f[:, 5]).max()
        assert (trend == 0.0) == (j < 2), f"step {j} after the load: trend feature {trend}"
        assert (du < 1e-12) == (j < 1) and (j < 1 or du > 1e-6), f"step {j} after the load: freestream change {du}"
    src.close()
    dst.close()
