"""Learned warm start for batched dynamic lifting-line solves (sb_mlp_* and the batch's
warm-start mode).

The reference starts every SimpleIterative solve from the previous step's circulation
(stormbird/src/lifting_line/simulation.rs:165,189; solvers/simple_iterative.rs:86-101). Here
the candidate start is the solution extrapolated linearly in time (2 G[t-1] - G[t-2], in f64)
plus a correction a network predicts per panel from features the batch builds on the GPU
(previous solution and its neighbours, its last change, freestream change, geometric angle of
attack, span position, sail index and counts, wake fill). The solve evaluates the residual of
the plain start, of the extrapolation and of extrapolation plus correction and starts from
the lowest, so the fallback is decided per case and step and the solver alone decides
the result.
A network whose output layer is zero gives the extrapolation alone (`extrapolation_only`),
the ablation that separates what the trained network adds.

Training runs on the GPU through the library's own kernels (tcgen05 BF16 GEMMs with FP32
accumulation, Adam); torch only holds the device tensors and shuffles the rows.
"""
from __future__ import annotations

import ctypes
import json

import numpy as np

from ._abi import SbError
from .batch import Batch
from .native import lib
from . import setups as S

FEATURES = 16  # SB_WARM_START_FEATURES


def _check(rc: int):
    if rc != 0:
        raise SbError(rc, lib().sb_last_error().decode())


def _torch():
    import torch

    return torch


class WarmStartNet:
    """The network: n_inputs -> 4 x 256 (GELU) -> 1, BF16 weights, FP32 accumulation."""

    def __init__(self, n_inputs: int = FEATURES, seed: int = 0, device: int = 0):
        h = lib().sb_mlp_new(int(device), int(n_inputs), ctypes.c_ulonglong(int(seed)))
        if not h:
            raise SbError(lib().sb_last_status(), lib().sb_last_error().decode())
        self._h = ctypes.c_void_p(h)
        self.n_inputs = n_inputs
        self.device = device
        n = ctypes.c_size_t()
        _check(lib().sb_mlp_num_params(self._h, ctypes.byref(n)))
        self.n_params = n.value

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None:
            lib().sb_mlp_free(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.n_params, dtype=np.float32)
        _check(lib().sb_mlp_get_params(self._h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), p.size))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(np.asarray(p, dtype=np.float32).reshape(-1))
        _check(lib().sb_mlp_set_params(self._h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), p.size))

    def forward(self, x):
        """x: CUDA float32 tensor [rows, n_inputs] -> CUDA float32 tensor [rows]."""
        torch = _torch()
        x = x.contiguous()
        y = torch.empty(x.shape[0], dtype=torch.float32, device=x.device)
        _check(lib().sb_mlp_forward(self._h, ctypes.c_void_p(x.data_ptr()), x.shape[0], ctypes.c_void_p(y.data_ptr())))
        return y

    def gradients(self, x, t):
        """(gradient [n_params] float32 numpy, mean-squared error) on CUDA tensors x, t."""
        g = np.zeros(self.n_params, dtype=np.float32)
        loss = ctypes.c_double()
        x, t = x.contiguous(), t.contiguous()
        _check(lib().sb_mlp_gradients(self._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(t.data_ptr()), x.shape[0],
                                      g.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), ctypes.byref(loss)))
        return g, loss.value

    def zero_output(self):
        """Output layer set to zero: the network predicts no correction (extrapolation only)."""
        p = self.get_params()
        p[-257:] = 0.0
        self.set_params(p)

    def train_step(self, x, t, lr: float, want_loss: bool = True):
        loss = ctypes.c_double()
        _check(lib().sb_mlp_train_step(self._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(t.data_ptr()), x.shape[0],
                                       ctypes.c_float(lr), ctypes.byref(loss) if want_loss else None))
        return loss.value if want_loss else None


def tight_solver(setup_json: str, max_iterations: int = 1000, residual_tolerance: float = 1e-7) -> str:
    """The setup with a SimpleIterative solve run to a tight residual (no strength-change exit)."""
    d = json.loads(setup_json)
    si = d["simulation_settings"]["Dynamic"].setdefault("solver", {}).setdefault("SimpleIterative", {})
    si["max_iterations_per_time_step"] = int(max_iterations)
    si["residual_tolerance_absolute"] = float(residual_tolerance)
    si["strength_difference_tolerance"] = 0.0
    return json.dumps(d)


def collect(cases, steps: int, dt: float = 0.05, skip: int = 2, device: int = 0, clip: float = 0.25):
    """Runs the cases as one batch with features and targets recorded; returns CUDA tensors
    X [rows, 16], T [rows] of steps skip..steps-1 (every case and panel), targets clipped to
    [-clip, clip] (the start-up steps hold a few large changes the guard rejects anyway)."""
    torch = _torch()
    b = Batch([js for js, _ in cases], device=device)
    winds = [w for _, w in cases]
    b.set_warm_start(None, 2)
    xs, ts = [], []
    for k in range(steps):
        b.do_step(time=k * dt, time_step=dt, freestream_velocity=S.batch_freestream(b, winds, k * dt))
        if k >= skip:
            x = torch.empty((b.total_lines, FEATURES), dtype=torch.float32, device=f"cuda:{device}")
            t = torch.empty(b.total_lines, dtype=torch.float32, device=f"cuda:{device}")
            _check(lib().sb_batch_copy_warm_start_data(b._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(t.data_ptr()),
                                                      b.total_lines))
            xs.append(x)
            ts.append(t)
    b.close()
    X, T = torch.cat(xs), torch.cat(ts).clamp_(-clip, clip)
    del xs, ts
    return X, T


def train(net: WarmStartNet, X, T, epochs: int = 4, batch_rows: int = 8192, lr: float = 5e-4, seed: int = 0,
          loss_every: int = 1):
    """Mini-batch Adam over shuffled rows; returns the mean loss of each epoch (over every
    `loss_every`-th step). An epoch whose loss is not finite is undone (parameters of the last
    good epoch) and the learning rate halved."""
    torch = _torch()
    g = torch.Generator(device=X.device)
    g.manual_seed(seed)
    out = []
    n = X.shape[0]
    batch_rows = min(batch_rows, n)
    good = net.get_params()
    for _ in range(epochs):
        perm = torch.randperm(n, device=X.device, generator=g)
        Xs, Ts = X[perm].contiguous(), T[perm].contiguous()
        tot, cnt = 0.0, 0
        for k, s0 in enumerate(range(0, n - batch_rows + 1, batch_rows)):
            want = k % loss_every == 0
            loss = net.train_step(Xs[s0:s0 + batch_rows], Ts[s0:s0 + batch_rows], lr, want_loss=want)
            if want:
                tot += loss
                cnt += 1
        m = tot / max(cnt, 1)
        if not np.isfinite(m):
            net.set_params(good)
            lr *= 0.5
            continue
        good = net.get_params()
        out.append(m)
    return out


def extrapolation_only(device: int = 0) -> WarmStartNet:
    """A network with a zero output layer: candidates are the linear extrapolation alone."""
    net = WarmStartNet(FEATURES, seed=0, device=device)
    net.zero_output()
    return net


def run_batch(cases, steps: int, net: WarmStartNet | None = None, dt: float = 0.05, device: int = 0,
              timed_from: int = 1, tune_seconds: float = 0.0, state_before_last: bool = False) -> dict:
    """Steps the cases as one batch (warm-started when `net` is given) on their freestream.

    Returns per step the circulation, iterations and start taken of every case, the host
    time of steps timed_from.. (one solve = one case advanced by one step) and, with
    tune_seconds > 0, the time the autotuner took before step timed_from (untimed; it
    needs 4 steps of wake, so timed_from >= 4). With state_before_last, also every case's
    state before the last step (sb_batch_get_case_state, outside the timed calls).
    """
    import time

    winds = [w for _, w in cases]
    b = Batch([js for js, _ in cases], device=device)
    if net is not None:
        b.set_warm_start(net.handle)
    its, taken, gam, t_run, t_tune, states = [], [], [], 0.0, 0.0, None
    for k in range(steps):
        if state_before_last and k == steps - 1:
            states = [b.case_state(i) for i in range(b.n_cases)]
        if tune_seconds > 0.0 and k == timed_from and k >= 4:
            t0 = time.perf_counter()
            b.autotune(tune_seconds)
            t_tune = time.perf_counter() - t0
        fs = S.batch_freestream(b, winds, k * dt)
        t0 = time.perf_counter()
        b.do_step(time=k * dt, time_step=dt, freestream_velocity=fs)
        if k >= timed_from:
            t_run += time.perf_counter() - t0
        s = b.summary()
        its.append(s[:, 7].copy())
        taken.append(s[:, 10].copy())
        g = b.circulation()
        gam.append([g[b.case_slice(i)] for i in range(b.n_cases)])
    info = b.info()
    b.close()
    return {"iterations": np.array(its), "start": np.array(taken), "gamma": gam, "seconds": t_run,
            "tune_seconds": t_tune, "tuning": {k: info[k] for k in ("waves", "blocks_per_sm", "tile", "schedule", "tuned")},
            "states_before_last": states}


def max_rel_diff(a, ref) -> float:
    """Largest relative (infinity-norm) difference per case and step between two runs."""
    worst = 0.0
    for ga, gr in zip(a["gamma"], ref["gamma"]):
        for x, y in zip(ga, gr):
            den = np.max(np.abs(y))
            if den > 0:
                worst = max(worst, float(np.max(np.abs(x - y)) / den))
    return worst


def evaluate(net: WarmStartNet, cases, steps: int, dt: float = 0.05, device: int = 0) -> dict:
    """Plain, extrapolation-only and network warm starts on the same cases and freestream.

    Iterations per solve and the fallback rate (solves that took the plain start) count
    steps 2.. (the extrapolation needs two previous solutions); the circulation differences
    are against the plain run over all steps.
    """
    plain = run_batch(cases, steps, None, dt, device, timed_from=2)
    ex_net = extrapolation_only(device)
    extra = run_batch(cases, steps, ex_net, dt, device, timed_from=2)
    ex_net.close()
    warm = run_batch(cases, steps, net, dt, device, timed_from=2)
    ip = plain["iterations"][2:]
    out = {"iterations_plain": float(ip.mean())}
    for name, r in (("extrapolation", extra), ("warm", warm)):
        it = r["iterations"][2:]
        out[f"iterations_{name}"] = float(it.mean())
        out[f"iterations_saved_fraction_{name}"] = float(1.0 - it.sum() / max(ip.sum(), 1.0))
        out[f"fallback_rate_{name}"] = float(np.mean(r["start"][2:] == 0.0))
        out[f"network_start_rate_{name}"] = float(np.mean(r["start"][2:] == 2.0))
        out[f"max_rel_circulation_diff_{name}"] = max_rel_diff(r, plain)
        out[f"seconds_{name}"] = r["seconds"]
    out["seconds_plain"] = plain["seconds"]
    return out
