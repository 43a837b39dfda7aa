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
    # The reference gridder against itself: zero error, within the stated
    # tolerance against _f.
    vf = acc["vs_reference_f"]
    assert vf["max_rel"] == 0.0 and vf["rms_rel"] == 0.0
    assert vf["tolerance"] >= bench.GRID_TOL and vf["num_skipped_equal"]
    assert 0 < acc["vs_fp64"]["rms_rel"] <= acc["vs_fp64"]["max_rel"]
    # Against the reference's FP64 gridder on the promoted inputs: the
    # placement disagreements are counted, and the error is that of the
    # FP32 sums plus the displaced visibilities.
    vd = acc["vs_reference_d"]
    assert vd["placement_disagreements"] >= \
        vd["placement_disagreements_gridded"] >= 0
    assert vd["num_skipped_d"] >= 0 and vd["rms_rel"] <= vd["max_rel"]
    assert vd["reference_f_vs_d"]["max_rel"] == vd["max_rel"]


def test_error_vs_is_max_and_rms():
    ref = np.zeros((4, 4, 2))
    ref[1, 2] = (3.0, 4.0)
    a = ref.copy()
    a[0, 0, 0] = 0.5
    e = bench.error_vs(a, ref)
    assert abs(e["max_rel"] - 0.5 / 4.0) < 1e-15
    assert abs(e["rms_rel"] - 0.5 / 5.0) < 1e-15


def test_accuracy_check_flags_a_planted_error():
    wl, _ = load_golden("small_f")
    _, grid, ns, nm = bench.cpu_run(wl, 2, keep=True)
    bad = grid.copy()
    i = np.unravel_index(np.abs(bad).argmax(), bad.shape)
    bad[i] *= np.float32(1.001)
    acc = bench.accuracy_vs_fp64(wl, bad, ns, nm, 2, with_d=False)
    assert not acc["ok"]
    assert acc["grid_max_rel_err"] > bench.GRID_TOL
    acc = bench.accuracy_vs_fp64(wl, grid, ns + 1, nm, 2, with_d=False)
    assert not acc["ok"]
    # Beyond the stated tolerance against the reference's _f only.
    cpu = bench.cpu_run(wl, 2, keep=True)
    acc = bench.accuracy_vs_fp64(wl, grid, ns, nm, 2, cpu, with_d=False)
    assert acc["ok"]
    off = grid.copy()
    off[i] += np.float32(2 * acc["vs_reference_f"]["tolerance"]) * \
        np.abs(grid).max()
    acc = bench.accuracy_vs_fp64(wl, off, ns, nm, 2, cpu, with_d=False)
    assert not acc["ok"]


def test_max_rel_err():
    ref = np.array([1.0, -4.0, 2.0])
    assert bench.max_rel_err(ref, ref) == 0.0
    assert abs(bench.max_rel_err(ref + [0.0, 0.0, 0.4], ref) - 0.1) < 1e-15
    assert bench.max_rel_err(np.ones(2), np.zeros(2)) == 1.0
