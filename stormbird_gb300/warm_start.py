"""Learned warm start for batched dynamic lifting-line solves (sb_mlp_* and the batch's
warm-start mode).

The reference starts every SimpleIterative solve from the previous step's circulation
(stormbird/src/lifting_line/simulation.rs:165,189; solvers/simple_iterative.rs:86-101). Here a
network predicts, per panel, how the solution changes in this step, from features the batch
builds on the GPU (previous solution and its neighbours, freestream change, geometric angle
of attack, span position, sail index and counts, wake fill). The solve evaluates the residual
of the plain start and of the prediction and starts from the lower one, so the fallback to
the plain start is decided per case and step and the solver remains the judge of the result.

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

    def train_step(self, x, t, lr: float, want_loss: bool = True):
        loss = ctypes.c_double()
        _check(lib().sb_mlp_train_step(self._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(t.data_ptr()), x.shape[0],
                                       ctypes.c_float(lr), ctypes.byref(loss) if want_loss else None))
        return loss.value if want_loss else None


def tight_solver(setup_json: str, max_iterations: int = 600, residual_tolerance: float = 1e-6) -> str:
    """The setup with a SimpleIterative solve run to a tight residual (no strength-change exit)."""
    d = json.loads(setup_json)
    si = d["simulation_settings"]["Dynamic"].setdefault("solver", {}).setdefault("SimpleIterative", {})
    si["max_iterations_per_time_step"] = int(max_iterations)
    si["residual_tolerance_absolute"] = float(residual_tolerance)
    si["strength_difference_tolerance"] = 0.0
    return json.dumps(d)


def collect(cases, steps: int, dt: float = 0.05, skip: int = 1, device: int = 0):
    """Runs the cases as one batch with features and targets recorded; returns CUDA tensors
    X [rows, 16], T [rows] of steps skip..steps-1 (every case and panel)."""
    torch = _torch()
    b = Batch([js for js, _ in cases], device=device)
    winds = [w for _, w in cases]
    _check(lib().sb_batch_set_warm_start(b._h, None, 2))
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
    return torch.cat(xs), torch.cat(ts)


def train(net: WarmStartNet, X, T, epochs: int = 4, batch_rows: int = 8192, lr: float = 1e-3, seed: int = 0):
    """Mini-batch Adam over shuffled rows; returns the mean loss of each epoch."""
    torch = _torch()
    g = torch.Generator(device=X.device)
    g.manual_seed(seed)
    out = []
    n = X.shape[0]
    for _ in range(epochs):
        perm = torch.randperm(n, device=X.device, generator=g)
        Xs, Ts = X[perm].contiguous(), T[perm].contiguous()
        tot, cnt = 0.0, 0
        for s0 in range(0, n - batch_rows + 1, batch_rows):
            loss = net.train_step(Xs[s0:s0 + batch_rows], Ts[s0:s0 + batch_rows], lr)
            tot += loss
            cnt += 1
        out.append(tot / max(cnt, 1))
    return out


def evaluate(net: WarmStartNet, cases, steps: int, dt: float = 0.05, device: int = 0) -> dict:
    """Runs the cases twice as batches, plain and warm-started, on the same freestream.

    Returns iterations per solve (plain, warm), the fraction of solves that took the plain
    start (fallback), the largest relative circulation difference between the two runs,
    and the wall time of each run's steps.
    """
    import time

    winds = [w for _, w in cases]
    res = {}
    gam = {}
    for mode in ("plain", "warm"):
        b = Batch([js for js, _ in cases], device=device)
        if mode == "warm":
            _check(lib().sb_batch_set_warm_start(b._h, net.handle, 1))
        its, taken, t_run = [], [], 0.0
        g_steps = []
        for k in range(steps):
            fs = S.batch_freestream(b, winds, k * dt)
            t0 = time.perf_counter()
            b.do_step(time=k * dt, time_step=dt, freestream_velocity=fs)
            t_run += time.perf_counter() - t0
            s = b.summary()
            its.append(s[:, 7].copy())
            taken.append(s[:, 10].copy())
            g_steps.append(b.circulation())
        res[mode] = {"iterations": np.array(its), "start": np.array(taken), "seconds": t_run}
        gam[mode] = (g_steps, [b.case_slice(i) for i in range(b.n_cases)])
        b.close()
    worst = 0.0
    for (gp, sl), (gw, _) in [(gam["plain"], gam["warm"])]:
        for k in range(steps):
            for s in sl:
                den = np.max(np.abs(gp[k][s]))
                if den > 0:
                    worst = max(worst, float(np.max(np.abs(gw[k][s] - gp[k][s])) / den))
    # the first step has no previous solution: the warm start is not offered there
    ip = res["plain"]["iterations"][1:]
    iw = res["warm"]["iterations"][1:]
    st = res["warm"]["start"][1:]
    return {
        "iterations_plain": float(ip.mean()),
        "iterations_warm": float(iw.mean()),
        "iterations_saved_fraction": float(1.0 - iw.sum() / max(ip.sum(), 1.0)),
        "fallback_rate": float(np.mean(st == 0.0)),
        "max_rel_circulation_diff": worst,
        "seconds_plain": res["plain"]["seconds"],
        "seconds_warm": res["warm"]["seconds"],
    }
