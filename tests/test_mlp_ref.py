"""The network's f64 restatement (tests/mlp_ref.py) against central finite differences:
the gradient formulas the GPU kernels are checked against are themselves right."""
import numpy as np

from tests import mlp_ref as R


def test_reference_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    n_in = 16
    p = R.init_params(n_in, seed=1)
    x = rng.normal(size=(24, n_in))
    t = rng.normal(size=24)
    _, g = R.loss_and_grad(p, x, t, emulate=False)
    h = 1e-6
    for name, sl in R.blocks():
        idx = np.arange(sl.start, sl.stop)
        if name == "W1":  # only the columns of real inputs carry a gradient
            idx = idx[(idx - sl.start) % R.INPAD < n_in]
        for i in rng.choice(idx, size=min(4, idx.size), replace=False):
            pp, pm = p.copy(), p.copy()
            pp[i] += h
            pm[i] -= h
            fd = (R.loss_and_grad(pp, x, t, emulate=False)[0] - R.loss_and_grad(pm, x, t, emulate=False)[0]) / (2 * h)
            assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)) + 1e-8, (name, i, fd, g[i])


def test_bf16_rounding_is_nearest_even():
    assert R.bf16(np.float32(1.0))[()] == 1.0
    # 1 + 2^-8 lies halfway between 1 and 1 + 2^-7: ties to even gives 1
    assert R.bf16(np.float32(1.0 + 2.0 ** -8))[()] == 1.0
    assert R.bf16(np.float32(1.0 + 3 * 2.0 ** -8))[()] == 1.0 + 2.0 ** -6
    assert R.bf16(np.float32(-2.5))[()] == -2.5
