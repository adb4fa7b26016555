"""sb_panel_sweep_no_alloc: the Biot-Savart sweep for callers that may not allocate device
memory while they run (a real-time co-simulation master stepping the lifting line, or a
framework whose memory pool owns the GPU). The caller owns every input and output buffer;
the sweep's scratch is a fixed device array inside the library.

Checked through the C ABI against the allocating entry point sb_panel_sweep on the same
panels and targets, on two calls in a row (the second reuses the scratch the first left
behind), within the FP32 sweep's tolerance, and against the f64 oracle's sweep, for every
symmetry condition. Also: no panels, a caller-created stream, the largest target count.
Collected last on purpose (file name) so that a run stopping at the first failure has run
every other test before it.
"""
import numpy as np
import pytest

from tests.helpers import rel_inf

pytestmark = pytest.mark.gpu

TOL = 1e-6         # relative infinity-norm error against sb_panel_sweep (same FP32 arithmetic, other chunking)
TOL_ORACLE = 1e-5  # relative infinity-norm error against the f64 oracle


def _device_inputs(torch, dev, corners, strengths, cores, targets):
    f = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64).reshape(-1)).to(dev)
    return f(corners), f(strengths), f(cores), f(targets)


def _case(seed=5, extra=300):
    from stormbird_gb300 import setups as S

    corners, strengths, cores, pts = S.synthetic_sail_row_wake(2, 16, 40, seed=seed)
    rng = np.random.default_rng(7)
    targets = np.concatenate([pts, rng.uniform([-10, -10, 1], [90, 60, 29], (extra, 3))])
    return corners, strengths, cores, targets


def _call(gpu_lib, torch, d, P, M, sym, out, stream=None):
    dc, ds, dr, dt = d
    torch.cuda.synchronize()
    rc = gpu_lib.sb_panel_sweep_no_alloc(0, dc.data_ptr(), ds.data_ptr(), dr.data_ptr(), P, 5.0, sym,
                                         dt.data_ptr(), M, out.data_ptr(), stream)
    assert rc == 0, gpu_lib.sb_last_error().decode()
    assert gpu_lib.sb_last_status() == 0
    return out.cpu().numpy()


@pytest.mark.parametrize("symmetry", [0, 1, 2, 3])
def test_no_alloc_sweep_matches_allocating_sweep_and_oracle(gpu_lib, oracle_mod, symmetry):
    torch = pytest.importorskip("torch")
    from stormbird_gb300.simulation import panel_sweep

    corners, strengths, cores, targets = _case()
    P, M = len(strengths), len(targets)
    expected = panel_sweep(corners, strengths, cores, targets, far_field_ratio=5.0, symmetry=symmetry)
    ref = oracle_mod.bs_sweep(corners, cores, strengths, 5.0, targets, nthreads=8, symmetry=symmetry)
    dev = torch.device("cuda", 0)
    d = _device_inputs(torch, dev, corners, strengths, cores, targets)
    out = torch.empty((M, 3), dtype=torch.float64, device=dev)
    for call in range(2):
        out.fill_(float("nan"))
        got = _call(gpu_lib, torch, d, P, M, symmetry, out)
        assert np.all(np.isfinite(got)), f"call {call}: output not fully written"
        assert rel_inf(got, expected) <= TOL, f"call {call}"
        assert rel_inf(got, ref) <= TOL_ORACLE, f"call {call}"


def test_no_alloc_sweep_without_panels_writes_zeros(gpu_lib):
    torch = pytest.importorskip("torch")
    corners, strengths, cores, targets = _case()
    dev = torch.device("cuda", 0)
    d = _device_inputs(torch, dev, corners, strengths, cores, targets)
    out = torch.full((len(targets), 3), float("nan"), dtype=torch.float64, device=dev)
    got = _call(gpu_lib, torch, d, 0, len(targets), 0, out)
    assert np.array_equal(got, np.zeros_like(got))


def test_no_alloc_sweep_on_a_caller_stream(gpu_lib):
    """Work is ordered on the stream the caller passes (a non-default torch stream here)."""
    torch = pytest.importorskip("torch")
    from stormbird_gb300.simulation import panel_sweep

    corners, strengths, cores, targets = _case(seed=9)
    expected = panel_sweep(corners, strengths, cores, targets, far_field_ratio=5.0)
    dev = torch.device("cuda", 0)
    d = _device_inputs(torch, dev, corners, strengths, cores, targets)
    s = torch.cuda.Stream(device=dev)
    out = torch.empty((len(targets), 3), dtype=torch.float64, device=dev)
    with torch.cuda.stream(s):
        out.fill_(float("nan"))
    got = _call(gpu_lib, torch, d, len(strengths), len(targets), 0, out, stream=s.cuda_stream)
    assert rel_inf(got, expected) <= TOL


def test_no_alloc_sweep_at_its_largest_target_count(gpu_lib):
    """65,536 targets: the partial-sum space then holds few source chunks."""
    torch = pytest.importorskip("torch")
    from stormbird_gb300.simulation import panel_sweep

    corners, strengths, cores, _ = _case()
    rng = np.random.default_rng(3)
    targets = rng.uniform([-20, -20, -5], [100, 80, 35], (65536, 3))
    expected = panel_sweep(corners, strengths, cores, targets, far_field_ratio=5.0)
    dev = torch.device("cuda", 0)
    d = _device_inputs(torch, dev, corners, strengths, cores, targets)
    out = torch.empty((len(targets), 3), dtype=torch.float64, device=dev)
    got = _call(gpu_lib, torch, d, len(strengths), len(targets), 0, out)
    assert rel_inf(got, expected) <= TOL


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
