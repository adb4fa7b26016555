"""The far-field fast path's box test, restated on the host in the kernel's FP32 arithmetic
(k_bs_sweep in csrc/k_biot_savart.cu: per quarter tile, the box of the warp's 64 target hi
parts against the box of the quarter's panel-centre hi parts and its largest far-field
radius squared, each gap shrunk by 2^-23 of the largest coordinate magnitude, then
gap^2 > 1.001 max ff2). Property: whenever the test says "all far", every pair is far by the
reference's f64 rule (panel.rs:53-57: the doublet when |x - c| > far-field length), for
boxes placed anywhere in space with gaps just above and below the radius."""
import numpy as np

F = np.float32


def box_test(targets, centres, ff2):
    th = targets.astype(F)
    ch = centres.astype(F)
    fh = ff2.astype(F)
    wb = np.concatenate([th.min(0), th.max(0)])
    c7 = np.concatenate([ch.min(0), ch.max(0), [fh.max()]]).astype(F)
    g2 = F(0)
    for q in range(3):
        m = max(abs(c7[q]), abs(c7[q + 3]), abs(wb[q]), abs(wb[q + 3]))
        d = max(F(c7[q] - wb[q + 3]), F(wb[q] - c7[q + 3]))
        g = max(F(0), F(d - F(2.0 ** -23) * m))
        g2 = F(g2 + F(g * g))
    return bool(c7[6] < np.inf and g2 > F(1.001) * c7[6])


def test_box_test_never_calls_a_near_pair_far():
    rng = np.random.default_rng(7)
    said_far = 0
    for trial in range(4000):
        origin = rng.uniform(-1, 1, 3) * 10.0 ** rng.uniform(0, 5)
        radius = 10.0 ** rng.uniform(-2, 1)
        # the quarter's 16 panel centres along a short segment, radii up to `radius`
        centres = origin + np.outer(rng.uniform(0, 1, 16), rng.normal(size=3)) * radius
        ff2 = (radius * rng.uniform(0.5, 1.0, 16)) ** 2
        # the warp's 64 targets along a segment whose box sits at about the radius from the
        # centres' box, just inside or just outside
        direction = rng.normal(size=3)
        direction /= np.linalg.norm(direction)
        dist = np.sqrt(ff2.max()) * (1.0 + rng.uniform(-3e-3, 3e-3)) + radius * rng.uniform(0, 2)
        start = centres.max(0) + direction * dist * (1.0 + radius)
        targets = start + np.outer(rng.uniform(0, 1, 64), rng.normal(size=3)) * radius * 0.3
        if box_test(targets, centres, ff2):
            said_far += 1
            d2 = ((targets[:, None, :] - centres[None, :, :]) ** 2).sum(-1)
            assert np.all(d2 > ff2[None, :]), f"trial {trial}: a near pair in a box called far"
    assert said_far > 100  # the test is exercised on both sides


def test_box_test_near_threshold_at_large_coordinates():
    # boxes 1e5 m from the origin, gap a few FP32 ulps of the coordinates beyond the radius:
    # the slack must keep the test from calling them far when the f64 gap is not beyond it
    rng = np.random.default_rng(11)
    for _ in range(2000):
        base = np.array([1e5, -3e4, 2e3]) * rng.uniform(0.5, 1.5)
        r = rng.uniform(0.5, 3.0)
        centres = base + rng.uniform(-0.1, 0.1, (16, 3))
        ff2 = np.full(16, r * r)
        gap = r * (1.0 + rng.uniform(-1e-6, 1e-6))
        targets = centres.max(0) + np.array([gap, 0.0, 0.0]) + rng.uniform(0, 0.05, (64, 3))
        if box_test(targets, centres, ff2):
            d2 = ((targets[:, None, :] - centres[None, :, :]) ** 2).sum(-1)
            assert np.all(d2 > ff2[None, :])
