"""CPU tests of bench.py's whole-workload accuracy check.

After its timed region the benchmark compares one clean gridding call with
the FP64-accumulation oracle (host-threaded, bit-identical to the serial
yardstick) and reports the max-rel grid error against the 1e-5 bound, the
skip counts and the norm, beside the reference FP32 gridder's own error.
Here the "GPU" grid is the oracle's FP32 restatement itself, and one with a
planted error, so the check is exercised without a GPU.
"""
from __future__ import annotations

import os
import sys

import numpy as np

from conftest import load_golden

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_accuracy_check_passes_the_reference_gridder():
    wl, _ = load_golden("small_f")
    cpu = bench.cpu_run(wl, 2, keep=True)
    _, grid, ns, nm = cpu
    acc = bench.accuracy_vs_fp64(wl, grid, ns, nm, 2, cpu)
    assert acc["ok"]
    assert acc["num_skipped"] == acc["num_skipped_fp64"] == ns
    assert 0 < acc["grid_max_rel_err"] <= bench.GRID_TOL
    assert acc["reference_f_max_rel_err"] == acc["grid_max_rel_err"]
    assert acc["norm_rel_err"] == 0.0


def test_accuracy_check_flags_a_planted_error():
    wl, _ = load_golden("small_f")
    _, grid, ns, nm = bench.cpu_run(wl, 2, keep=True)
    bad = grid.copy()
    i = np.unravel_index(np.abs(bad).argmax(), bad.shape)
    bad[i] *= np.float32(1.001)
    acc = bench.accuracy_vs_fp64(wl, bad, ns, nm, 2)
    assert not acc["ok"]
    assert acc["grid_max_rel_err"] > bench.GRID_TOL
    acc = bench.accuracy_vs_fp64(wl, grid, ns + 1, nm, 2)
    assert not acc["ok"]


def test_max_rel_err():
    ref = np.array([1.0, -4.0, 2.0])
    assert bench.max_rel_err(ref, ref) == 0.0
    assert abs(bench.max_rel_err(ref + [0.0, 0.0, 0.4], ref) - 0.1) < 1e-15
    assert bench.max_rel_err(np.ones(2), np.zeros(2)) == 1.0
