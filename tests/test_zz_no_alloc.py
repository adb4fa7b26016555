"""sb_panel_sweep_no_alloc: the Biot-Savart sweep for callers that may not allocate device
memory while they run (a real-time co-simulation master stepping the lifting line, or a
framework whose memory pool owns the GPU). The caller owns every input and output buffer;
the sweep's scratch is a fixed device array inside the library.

Checked through the C ABI against the allocating entry point sb_panel_sweep on the same
panels and targets, on two calls in a row (the second reuses the scratch the first left
behind), within the FP32 sweep's tolerance. Collected last on purpose (file name) so that a
run stopping at the first failure has run every other test before it.
"""
import ctypes

import numpy as np
import pytest

from tests.helpers import rel_inf

pytestmark = pytest.mark.gpu

TOL = 1e-6  # relative infinity-norm error, as for the other FP32 sweep comparisons


def _device_inputs(torch, dev, corners, strengths, cores, targets):
    f = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64).reshape(-1)).to(dev)
    return f(corners), f(strengths), f(cores), f(targets)


def test_no_alloc_sweep_matches_allocating_sweep(gpu_lib):
    torch = pytest.importorskip("torch")
    from stormbird_gb300 import setups as S
    from stormbird_gb300.simulation import panel_sweep

    corners, strengths, cores, pts = S.synthetic_sail_row_wake(2, 16, 40, seed=5)
    rng = np.random.default_rng(7)
    targets = np.concatenate([pts, rng.uniform([-10, -10, 1], [90, 60, 29], (300, 3))])
    P, M = len(strengths), len(targets)
    expected = panel_sweep(corners, strengths, cores, targets, far_field_ratio=5.0)

    dev = torch.device("cuda", 0)
    dc, ds, dr, dt = _device_inputs(torch, dev, corners, strengths, cores, targets)
    out = torch.empty((M, 3), dtype=torch.float64, device=dev)
    for call in range(2):
        out.fill_(float("nan"))
        torch.cuda.synchronize()
        rc = gpu_lib.sb_panel_sweep_no_alloc(0, dc.data_ptr(), ds.data_ptr(), dr.data_ptr(), P, 5.0, 0,
                                             dt.data_ptr(), M, out.data_ptr(), None)
        assert rc == 0, gpu_lib.sb_last_error().decode()
        got = out.cpu().numpy()
        assert np.all(np.isfinite(got)), f"call {call}: output not fully written"
        assert rel_inf(got, expected) <= TOL, f"call {call}"


def test_no_alloc_sweep_rejects_sizes_beyond_its_maximum(gpu_lib):
    from stormbird_gb300 import setups as S

    torch = pytest.importorskip("torch")
    corners, strengths, cores, pts = S.synthetic_sail_row_wake(1, 4, 3, seed=1)
    dev = torch.device("cuda", 0)
    dc, ds, dr, dt = _device_inputs(torch, dev, corners, strengths, cores, pts)
    out = torch.empty((len(pts), 3), dtype=torch.float64, device=dev)
    rc = gpu_lib.sb_panel_sweep_no_alloc(0, dc.data_ptr(), ds.data_ptr(), dr.data_ptr(), 16384 + 1, 5.0, 0,
                                         dt.data_ptr(), len(pts), out.data_ptr(), None)
    assert rc == -2 and "at most 16384 panels" in gpu_lib.sb_last_error().decode()
    rc = gpu_lib.sb_panel_sweep_no_alloc(0, dc.data_ptr(), ds.data_ptr(), dr.data_ptr(), len(strengths), 5.0, 0,
                                         dt.data_ptr(), 65536 + 1, out.data_ptr(), None)
    assert rc == -2
