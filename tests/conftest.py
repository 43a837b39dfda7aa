"""Shared test setup.

Marker ``gpu``: the test needs a CUDA GPU (GB300); run with ``-m gpu``.
Everything else runs on a CPU-only host.
"""
from __future__ import annotations

import glob
import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def pkg():
    return importlib.import_module("gpu-gridding_gb300")


@pytest.fixture(scope="session")
def synthetic():
    return importlib.import_module("gpu-gridding_gb300.synthetic")


def golden_names(prefix=""):
    return sorted(os.path.basename(p)[:-4] for p in
                  glob.glob(os.path.join(GOLDEN, f"{prefix}*.npz")))


def load_golden(name):
    """A golden case as (workload, dict of stored arrays)."""
    synthetic = importlib.import_module("gpu-gridding_gb300.synthetic")
    z = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    if "conv_func" not in z:
        return None, z
    wl = synthetic.Workload(
        name=name, num_w_planes=int(z["num_w_planes"]),
        support=z["support"].astype(np.int32),
        oversample=int(z["oversample"]),
        conv_size_half=int(z["conv_size_half"]), conv_func=z["conv_func"],
        uu=z["uu"], vv=z["vv"], ww=z["ww"], vis=z["vis"], weight=z["weight"],
        cell_size_rad=z["cell_size_rad"].item(), w_scale=z["w_scale"].item(),
        grid_size=int(z["grid_size"]))
    return wl, z


def max_rel(a, b):
    """max |a - b| / max |b| (b is the yardstick)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = np.abs(b).max()
    return float(np.abs(a - b).max() / scale) if scale > 0 else \
        float(np.abs(a - b).max())


def rms_rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.sqrt((b * b).sum())
    return float(np.sqrt(((a - b) ** 2).sum()) / den) if den > 0 else 0.0
