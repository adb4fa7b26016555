"""Target order of the FP32 far-field panel sweeps over wake points (BsJob::slots,
bs_slot_target in csrc/sb_kernels.h), checked on the host: the slots are a permutation of
every point of the rows that hold the M targets, they run wing by wing and within a wing
row by row, so that 64 consecutive slots (a warp's targets) belong to one wing except
where one wing's points end and the next wing's begin."""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "stormbird_gb300", "csrc")
INCLUDE = os.path.join(HERE, "..", "include")

# (M, points per wing): the sail row of the benchmark (4 x 65 points, 300 rows, the last
# point left out as the reference's ratio 1.0 does), uneven wings, a partial last row
CASES = [
    (300 * 260 + 259, [65, 65, 65, 65]),
    (7 * 305 - 1, [17, 49, 97, 65, 77]),
    (3 * 8 + 5, [3, 5]),
    (1, [92, 92, 92]),
    (51 * 546, [91] * 6),
]


@pytest.fixture(scope="module")
def mappings():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "slot_order_check")
        subprocess.run([nvcc, "-std=c++17", "-x", "cu", "-I", CSRC, "-I", INCLUDE,
                        os.path.join(HERE, "slot_order_check.cu"), "-o", exe], check=True, capture_output=True)
        inp = "".join(f"{m} {len(p)} {' '.join(map(str, p))}\n" for m, p in CASES)
        out = subprocess.run([exe], input=inp, text=True, check=True, capture_output=True).stdout
    return [np.array(line.split(), dtype=np.int64) for line in out.strip().splitlines()]


@pytest.mark.parametrize("k", range(len(CASES)))
def test_slot_order_is_wing_by_wing_permutation(mappings, k):
    M, pts = CASES[k]
    Np = sum(pts)
    rows = -(-M // Np)
    idx = mappings[k]
    assert idx.size == rows * Np
    assert np.array_equal(np.sort(idx), np.arange(rows * Np))  # every point of the rows once
    off = np.concatenate([[0], np.cumsum(pts)])
    wing = np.searchsorted(off, idx % Np, side="right") - 1
    row = idx // Np
    assert np.all(np.diff(wing) >= 0)  # wing by wing
    for w in range(len(pts)):
        sel = wing == w
        assert sel.sum() == rows * pts[w]
        r, j = row[sel], idx[sel] % Np - off[w]
        assert np.all(np.diff(r) >= 0)  # rows in order within a wing
        assert np.array_equal(r * pts[w] + j, np.arange(rows * pts[w]))  # points in order within a row
    # a warp's 64 slots span at most two wings, and one wing unless a wing ends among them
    for s0 in range(0, idx.size, 64):
        ws = np.unique(wing[s0:s0 + 64])
        assert ws.size <= 2
